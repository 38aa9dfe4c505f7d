// kernels.cuh -- launchers shared between the translation units of libimdgpu.
#pragma once

#include "internal.cuh"

namespace imdgpu {

struct ForceTabs {
  DevTable pair, rho, embed;
  int eam;
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

// system.cu: message returned by imdgpu_last_error()
void set_last_error(const char *msg);

}  // namespace imdgpu
