// kernels.cuh -- launchers shared between the translation units of libimdgpu.
#pragma once

#include "internal.cuh"

namespace imdgpu {

struct ForceTabs {
  DevTable pair, rho, embed;
  int eam;
  int nt1;       // single atom type
  int samegrid;  // pair and rho columns share begin / end / step: one index per pair
  int exact;     // IMD's unfused arithmetic (bitwise table values) instead of FMA form
  int epot;      // scatter per-atom energies (POTENG) in the force pass
};

// Device-side scalars of one system (results + control).
struct DevScalars {
  double epot;        // tot_pot_energy
  double virial;
  double ekin;        // tot_kin_energy
  double fnorm;
  double fmax2;       // max squared component
  double fatom2;      // max per-atom |F|^2
  double maxdisp2;    // max |x - x_ref|^2 since the last build
  int rebuild;        // 1: list invalid (check_nblist result)
  int pad;
};

constexpr int BS_FORCE = 128;
constexpr int BS_VEC = 256;

// forces.cu
// Adds pair + EAM2 forces of the current list into frc/rho/df (zeroed
// before), folds ghosts, and writes energy / virial into sc.  `mixed`
// selects FP32 pair arithmetic.  Returns kernel launches issued.
// ev (may be null): 4 events recorded around the density and force kernels.
int launch_forces(const SysView &v, const ForceTabs &t, DevScalars *sc, int mixed,
                  cudaStream_t st, cudaEvent_t *ev = nullptr);

// forces.cu: refresh ghost positions (send_cells(copy_cell))
void k_ghost_pos_launch(const SysView &v, int blocks, cudaStream_t st);
// mixed.cu: the FP32-force path over the full list
int launch_forces_mixed(const SysView &v, const ForceTabs &t, DevScalars *sc, float *dff,
                        cudaStream_t st, cudaEvent_t *ev);

// system.cu: message returned by imdgpu_last_error()
void set_last_error(const char *msg);

}  // namespace imdgpu
