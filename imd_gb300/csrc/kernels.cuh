// kernels.cuh -- launchers shared between the translation units of libimdgpu.
#pragma once

#include <cuda_bf16.h>

#include "internal.cuh"

namespace imdgpu {

struct ForceTabs {
  DevTable pair, rho, embed;
  int eam;
  int nt1;       // single atom type
  int samegrid;  // pair and rho columns share begin / end / step: one index per pair
  int exact;     // IMD's unfused arithmetic (bitwise table values) instead of FMA form
  int epot;      // scatter per-atom energies (POTENG) in the force pass
  int bs;        // threads per block of the force pass (autotuned, multiple of 32)
  int bs_rho;    // threads per block of the density pass (autotuned)
  int det;       // FP64 passes on the full list without atomics (deterministic)
  const float4 *fused;  // mixed force pass: fused pair/density rows, or null
  unsigned fused_bytes;
  int stage_grid;       // >0: the force pass stages them in shared memory, this many blocks
  int cache;            // FP64: the density pass caches per-entry pair terms for the force pass
  int lpa;              // lanes per atom of the cached passes (1, 2, 4)
  int mixed_lpa;        // lanes per atom of the mixed density pass (1, 2, 4; one species)
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
  int badin;          // lowest atom with a non-finite uploaded value (put_state)
};

// batched CG (batch.cu): vector operation a cell asks for in the next round
enum { OP_NONE = 0, OP_MOVE = 1, OP_SETHG_MOVE = 2, OP_RESET_MOVE = 3, OP_IDLE = 4 };
// program counter of the resumable linmin / mnbrak / brent
enum {
  PC_START, PC_AFTER_RESET, PC_LINMIN, PC_LINMIN_FB, PC_MNBRAK_FC, PC_MNBRAK_WHILE,
  PC_MNBRAK_A, PC_MNBRAK_C, PC_MNBRAK_E, PC_MNBRAK_SHIFT, PC_MNBRAK_END, PC_BRENT_ITER,
  PC_BRENT_FU, PC_AFTER_LINMIN, PC_DONE
};
struct CgParams {
  double linmin_tol, linmin_dmax, linmin_dmin, cg_glimit, cg_zeps, fmax;
  int linmin_maxsteps, maxsteps, cg_fr, pad;
};
struct CgSys {
  double E, fnorm, fmax2, fatom2, gg, dgg;               // last evaluation (k_bt_reduce)
  double alpha, gamma, old_alphamin, f_max2, cg_poteng, old_cg_poteng;
  double ax, bx, cx, fa, fb, fc, u, fu, ulim;            // mnbrak
  double a, b, x, w, v, fx, fw, fv, e, d;                // brent
  int pc, op, pending, steps, nfc, status, iter, ctf;
  int nshort;                                            // line searches ended short, in a row
  int eval;  // the last force pass evaluated this cell: its sums are still to be taken
};

constexpr int BS_FORCE = 128;      // default block of the pair passes
constexpr int BS_FORCE_MAX = 128;  // largest block the autotuner may pick (the
                                   // kernels' launch bound; register use as tuned)
constexpr int BS_VEC = 256;

// forces.cu
// Adds pair + EAM2 forces of the current list into frc/rho/df (zeroed
// before), folds ghosts, and writes energy / virial into sc.  `mixed`
// selects FP32 pair arithmetic.  Returns kernel launches issued.
// ev (may be null): 4 events recorded around the density and force kernels.
int launch_forces(const SysView &v, const ForceTabs &t, DevScalars *sc, int mixed,
                  cudaStream_t st, cudaEvent_t *ev = nullptr);

// forces.cu: STRESS_TENS per-atom stress (6 per ext atom, xx yy zz yz zx xy)
// of the current list, after launch_forces; ghosts folded into owners
int launch_stress(const SysView &v, const ForceTabs &t, double *stress, cudaStream_t st);

// forces.cu: refresh ghost positions (send_cells(copy_cell))
void k_ghost_pos_launch(const SysView &v, int blocks, cudaStream_t st);
// send_forces(add_rho) and send_forces(add_forces): ghost sums into owners
int mixed_staged_grid(unsigned bytes);
void fold_rho_launch(const SysView &v, int blocks, cudaStream_t st);
void fold_force_launch(const SysView &v, int blocks, cudaStream_t st);
// mixed.cu: the FP32-force path over the full list
int launch_forces_mixed(const SysView &v, const ForceTabs &t, DevScalars *sc, cudaStream_t st,
                        cudaEvent_t *ev);

// batch.cu
void launch_batch_round_pre(const SysView &v, CgSys *cs, int nsys, const CgParams &P,
                            int *sys_done, int *sys_short, double4 *oldx, double4 *g,
                            double4 *h,
                            unsigned long long *maxd, int *ndone, DevScalars *sc,
                            double skin2, cudaStream_t st);
void launch_batch_round_post(const SysView &v, const int *aoff, CgSys *cs, int nsys,
                             const double4 *g, int cg_fr, cudaStream_t st);
// the persistent CG engine of a round (sums of the last evaluation, control,
// vector update, displacement test), in place of the pre and post kernels;
// `order`: cells largest first, `queue`: a work counter the launch zeroes
void launch_batch_engine(const SysView &v, const int *aoff, const int *order, CgSys *cs,
                         int nsys, const CgParams &P, int *sys_done, int *sys_short,
                         double4 *oldx, double4 *g, double4 *h, unsigned long long *maxd,
                         int *ndone, int *queue, DevScalars *sc, double skin2, int grid,
                         cudaStream_t st);
int batch_engine_grid();

// learn.cu
struct MlPair;
size_t ml_smem_bytes();
int ml_nparam();
void launch_ml_pairs(const SysView &v, MlPair *pairs, int cap, int *count, cudaStream_t st);
void launch_ml_forward(const MlPair *pairs, const int *np, const double *rho,
                       const __nv_bfloat16 *wb, const float *wf, float *dxp, int blocks,
                       cudaStream_t st);
void launch_ml_loss(int n, const float *dxp, const float *target, const float *wt, float *dldx,
                    double *loss, cudaStream_t st);
void launch_ml_forward_tc(const MlPair *pairs, const int *np, const double *rho,
                          const __nv_bfloat16 *wb, const float *wf, float *dxp, unsigned *status,
                          int blocks, cudaStream_t st);
void launch_ml_backward(const MlPair *pairs, const int *np, const double *rho,
                        const __nv_bfloat16 *wb, const float *wf, const float *dldx,
                        float *grad, int blocks, cudaStream_t st);
void launch_ml_adam(float *w, __nv_bfloat16 *wb, const float *grad, float *m, float *vv, int n,
                    float lr, int step, cudaStream_t st);
void launch_ml_to_bf16(const float *w, __nv_bfloat16 *wb, int n, cudaStream_t st);

// system.cu: message returned by imdgpu_last_error()
void set_last_error(const char *msg);

// output.cu: IMD's checkpoint lines formatted on the device
struct FormatScratch {
  long *len = nullptr;   // per line: length, then its offset within its block
  long *bsum = nullptr;  // per scan block: offset; [nb] the total
  int *bad = nullptr;    // lowest line that could not be formatted
  char *text = nullptr;
  int cap_lines = 0;
  long cap_bytes = 0;
};
int format_atom_lines(const SysView &v, const int *slot_of, const int *order, int n, int flags,
                      char *buf, long cap, long *len, FormatScratch &fs, cudaStream_t st);
void free_format_scratch(FormatScratch &fs);

}  // namespace imdgpu
