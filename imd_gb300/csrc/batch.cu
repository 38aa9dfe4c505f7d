// batch.cu -- batched CG relaxation of many independent periodic cells.
//
// Every cell runs IMD's own CG (src/imd_cg.c: reset_cg :30, cg_step :46,
// linmin :96, fonedim :295, cg_calcgamma :451, set_hg :501; mnbrak and
// brent from src/cg_utils.h:34-194) as a resumable state machine, one device
// thread per cell.  All cells advance in rounds; one round is
//   control (one thread per cell: consume the last energy, decide the next
//            trial alpha or the end of a line search)
//   -> vector update of every atom (move_atoms_cg, src/imd_integrate.c:2881,
//      fused with set_hg / the reset of h, g, old_x when a line search ends)
//      and the displacement test of check_nblist per cell
//   -> guarded rebuild (all cells, when any cell moved more than skin/2)
//   -> forces of all atoms of all unfinished cells (the force kernels of the
//      single-system path; pairs never cross cells)
//   -> per-cell reductions (energy, |F|^2, max |F|, g.g and F.(F-g)).
// The host replays a captured CUDA graph of rounds until every cell is done.
#include <algorithm>

#include "kernels.cuh"

namespace imdgpu {

__device__ __forceinline__ double sgn(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

// resumable linmin / mnbrak / brent of one cell
constexpr int SHORT_STEPS = 5;

// short_last: the evaluation just consumed had a pair closer than a table's
// first point (IMD's "Short distance").  Trial points of a line search may,
// and CG usually gets out again.  SHORT_STEPS line searches in a row that end
// on such a point without lowering the energy stop the cell with status 4:
// the tables clamp there, energy and forces no longer match, and IMD's CG
// stays there for good.
__device__ void cg_machine(CgSys &S, const CgParams &P, bool short_last) {
  const double CGOLD = 0.3819660, GOLD = 1.618034, TINY = 1.0e-20;
  const double fres = S.E;  // result of the pending evaluation (energy at alpha)
  for (int guard = 0; guard < 64; guard++) {
    switch (S.pc) {
      case PC_START:  // reset_cg: calc_forces at the start positions
        S.op = OP_NONE;
        S.pc = PC_AFTER_RESET;
        return;
      case PC_AFTER_RESET:  // calc_fnorm_g_h done lazily by OP_RESET_MOVE
        S.nshort = short_last ? 1 : 0;
        S.cg_poteng = fres;
        S.old_cg_poteng = fres;
        S.f_max2 = S.fmax2;
        S.pending = OP_RESET_MOVE;
        if (S.fatom2 <= P.fmax * P.fmax) {
          S.pc = PC_DONE;
          break;
        }
        S.steps = 1;
        S.pc = PC_LINMIN;
        break;
      case PC_LINMIN: {  // linmin (src/imd_cg.c:96-147)
        const double f_max = sqrt(S.f_max2);
        if (f_max > 100 * P.linmin_dmax) S.bx = P.linmin_dmax / f_max;
        else if (S.old_alphamin < P.linmin_dmin) S.bx = 0.05;
        else S.bx = 2.0 * S.old_alphamin;
        S.cx = 2.0 * S.bx;
        S.ax = 0.0;
        S.fa = S.old_cg_poteng;
        S.alpha = S.bx;
        S.op = S.pending;
        S.pending = OP_MOVE;
        S.pc = PC_LINMIN_FB;
        return;
      }
      case PC_LINMIN_FB:  // fb = fonedim(alpha_b); mnbrak start (src/cg_utils.h:119-134)
        S.fb = fres;
        if (S.fb > S.fa) {
          double t = S.ax; S.ax = S.bx; S.bx = t;
          t = S.fb; S.fb = S.fa; S.fa = t;
        }
        S.cx = S.bx + GOLD * (S.bx - S.ax);
        if ((S.bx - S.ax) <= 1e-4) S.cx = S.bx + 0.05;
        if (S.cx < 0.0) S.cx = S.bx - 1.0 / GOLD * (S.bx - S.ax);
        if (S.cx >= 1.0) S.cx = 1.0;
        S.alpha = S.cx;
        S.op = OP_MOVE;
        S.pc = PC_MNBRAK_FC;
        return;
      case PC_MNBRAK_FC:
        S.fc = fres;
        S.ctf = 1;
        S.pc = PC_MNBRAK_WHILE;
        break;
      case PC_MNBRAK_WHILE: {  // while (fb >= fc) (src/cg_utils.h:135-190)
        if (!(S.fb >= S.fc)) {
          S.pc = PC_MNBRAK_END;
          break;
        }
        const double r = (S.bx - S.ax) * (S.fb - S.fc);
        const double q = (S.bx - S.cx) * (S.fb - S.fa);
        S.u = S.bx - ((S.bx - S.cx) * q - (S.bx - S.ax) * r) /
                         (2.0 * sgn(fmax(fabs(q - r), TINY), q - r));
        S.ulim = S.bx + P.cg_glimit * (S.cx - S.bx);
        S.op = OP_MOVE;
        if ((S.bx - S.u) * (S.u - S.cx) > 0.0) {
          S.pc = PC_MNBRAK_A;
        } else if ((S.cx - S.u) * (S.u - S.ulim) > 0.0) {
          S.pc = PC_MNBRAK_C;
        } else if ((S.u - S.ulim) * (S.ulim - S.cx) >= 0.0) {
          S.u = S.ulim;
          S.pc = PC_MNBRAK_E;
        } else {
          S.u = S.cx + GOLD * (S.cx - S.bx);
          S.pc = PC_MNBRAK_E;
        }
        S.alpha = S.u;
        return;
      }
      case PC_MNBRAK_A:
        S.fu = fres;
        S.ctf++;
        if (S.fu < S.fc) {
          S.ax = S.bx;
          S.bx = S.u;
          S.fa = S.fb;
          S.fb = S.fu;
          S.pc = PC_MNBRAK_END;
          break;
        } else if (S.fu > S.fb) {
          S.cx = S.u;
          S.fc = S.fu;
          S.pc = PC_MNBRAK_END;
          break;
        }
        S.u = S.cx + GOLD * (S.cx - S.bx);
        S.alpha = S.u;
        S.op = OP_MOVE;
        S.pc = PC_MNBRAK_E;
        return;
      case PC_MNBRAK_C:
        S.fu = fres;
        S.ctf++;
        if (S.fu < S.fc) {
          S.bx = S.cx;
          S.cx = S.u;
          S.u = S.cx + GOLD * (S.cx - S.bx);
          S.fb = S.fc;
          S.fc = S.fu;
          S.alpha = S.u;
          S.op = OP_MOVE;
          S.pc = PC_MNBRAK_E;  // fu = fonedim(u); ctf++; then the shift
          return;
        }
        S.pc = PC_MNBRAK_SHIFT;
        break;
      case PC_MNBRAK_E:
        S.fu = fres;
        S.ctf++;
        S.pc = PC_MNBRAK_SHIFT;
        break;
      case PC_MNBRAK_SHIFT:
        S.ax = S.bx;
        S.bx = S.cx;
        S.cx = S.u;
        S.fa = S.fb;
        S.fb = S.fc;
        S.fc = S.fu;
        S.pc = PC_MNBRAK_WHILE;
        break;
      case PC_MNBRAK_END: {  // sort (src/imd_cg.c:155-167), brent set-up (src/cg_utils.h:34-52)
        double t;
        if (S.ax > S.bx) {
          t = S.ax; S.ax = S.bx; S.bx = t;
          t = S.fa; S.fa = S.fb; S.fb = t;
        }
        if (S.bx > S.cx) {
          t = S.bx; S.bx = S.cx; S.cx = t;
          t = S.fb; S.fb = S.fc; S.fc = t;
        }
        if (S.ax > S.bx) {
          t = S.ax; S.ax = S.bx; S.bx = t;
          t = S.fa; S.fa = S.fb; S.fb = t;
        }
        S.a = S.ax;
        S.b = S.bx;
        S.x = S.w = S.v = S.bx;
        S.fw = S.fv = S.fx = S.fb;
        S.e = 0.0;
        S.d = 0.0;
        S.iter = 1;
        S.pc = PC_BRENT_ITER;
        break;
      }
      case PC_BRENT_ITER: {  // one brent iteration up to fonedim(u) (src/cg_utils.h:53-92)
        if (S.iter > P.linmin_maxsteps) {
          S.status = 2;  // "Too many iterations in brent"
          S.pc = PC_DONE;
          break;
        }
        const double xm = 0.5 * (S.a + S.b);
        const double tol1 = P.linmin_tol * fabs(S.x) + P.cg_zeps;
        const double tol2 = 2.0 * tol1;
        if (fabs(S.x - xm) <= (tol2 - 0.5 * (S.b - S.a))) {
          S.old_alphamin = S.x;  // linmin: old_alphamin = alphamin
          S.pc = PC_AFTER_LINMIN;
          break;
        }
        if (fabs(S.e) > tol1) {
          const double r = (S.x - S.w) * (S.fx - S.fv);
          double q = (S.x - S.v) * (S.fx - S.fw);
          double p = (S.x - S.v) * q - (S.x - S.w) * r;
          q = 2.0 * (q - r);
          if (q > 0.0) p = -p;
          q = fabs(q);
          const double etemp = S.e;
          S.e = S.d;
          if (fabs(p) >= fabs(0.5 * q * etemp) || p <= q * (S.a - S.x) || p >= q * (S.b - S.x)) {
            S.e = (S.x >= xm) ? (S.a - S.x) : (S.b - S.x);
            S.d = CGOLD * S.e;
          } else {
            S.d = p / q;
            const double uu = S.x + S.d;
            if ((uu - S.a < tol2) || (S.b - uu < tol2)) S.d = sgn(tol1, xm - S.x);
          }
        } else {
          S.e = (S.x >= xm) ? (S.a - S.x) : (S.b - S.x);
          S.d = CGOLD * S.e;
        }
        S.u = (fabs(S.d) >= tol1) ? (S.x + S.d) : (S.x + sgn(tol1, S.d));
        S.alpha = S.u;
        S.op = OP_MOVE;
        S.pc = PC_BRENT_FU;
        return;
      }
      case PC_BRENT_FU:  // src/cg_utils.h:93-110
        S.fu = fres;
        if (S.fu <= S.fx) {
          if (S.u >= S.x) S.a = S.x;
          else S.b = S.x;
          S.v = S.w; S.w = S.x; S.x = S.u;
          S.fv = S.fw; S.fw = S.fx; S.fx = S.fu;
        } else {
          if (S.u < S.x) S.a = S.u;
          else S.b = S.u;
          if ((S.fu <= S.fw) || (S.w == S.x)) {
            S.v = S.w; S.fv = S.fw;
            S.w = S.u; S.fw = S.fu;
          } else if ((S.fu <= S.fv) || (S.v == S.x) || (S.v == S.w)) {
            S.v = S.u; S.fv = S.fu;
          }
        }
        S.iter++;
        S.pc = PC_BRENT_ITER;
        break;
      case PC_AFTER_LINMIN:  // cg_calcgamma + set_hg (applied with the next move)
        S.nshort = (short_last && !(fres < S.old_cg_poteng)) ? S.nshort + 1 : 0;
        if (S.nshort >= SHORT_STEPS) {
          S.status = 4;
          S.op = OP_IDLE;
          S.pc = PC_DONE;
          return;
        }
        S.gamma = S.dgg / S.gg;
        S.f_max2 = S.fmax2;
        S.pending = OP_SETHG_MOVE;
        if (S.fatom2 <= P.fmax * P.fmax || S.steps >= P.maxsteps) {
          if (S.fatom2 > P.fmax * P.fmax) S.status = 1;  // stopped by maxsteps
          S.pc = PC_DONE;
          break;
        }
        S.steps++;
        S.cg_poteng = fres;  // tot_pot_energy at the last evaluated point
        S.old_cg_poteng = fres;
        S.pc = PC_LINMIN;
        break;
      case PC_DONE:
      default:
        S.op = OP_IDLE;
        S.pc = PC_DONE;
        return;
    }
  }
  S.status = 3;  // control did not reach an evaluation: stop the cell
  S.op = OP_IDLE;
  S.pc = PC_DONE;
}

__global__ void k_bt_control(CgSys *cs, int nsys, CgParams P, int *sys_done, int *sys_short,
                             unsigned long long *maxd, int *ndone) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  CgSys S = cs[s];
  // the flag of the last evaluation; the next force pass sets it afresh
  const bool short_last = sys_short[s] != 0;
  sys_short[s] = 0;
  if (S.pc != PC_DONE) cg_machine(S, P, short_last);
  maxd[s] = 0ull;
  const int done = (S.pc == PC_DONE);
  if (done && !sys_done[s]) atomicAdd(ndone, 1);
  sys_done[s] = done;
  cs[s] = S;
}

// move_atoms_cg (x = old_x + alpha h), preceded by set_hg or the reset of
// g, h and old_x when the cell's control asks for it; then the
// check_nblist displacement of the atom, max-reduced per cell
__global__ void __launch_bounds__(BS_VEC) k_bt_vec(SysView v, const CgSys *cs, double4 *oldx,
                                                   double4 *g, double4 *h,
                                                   unsigned long long *maxd) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const int sy = v.atom_sys[i];
  const int op = cs[sy].op;
  if (op == OP_IDLE) return;
  double4 x = v.pos[i];
  if (op != OP_NONE) {
    const double alpha = cs[sy].alpha;
    double4 ox = oldx[i], hh = h[i];
    if (op == OP_RESET_MOVE || op == OP_SETHG_MOVE) {
      const double4 f = v.frc[i];
      ox = make_double4(x.x, x.y, x.z, 0.0);
      if (op == OP_RESET_MOVE) {
        hh = f;
      } else {
        const double gm = cs[sy].gamma;
        hh.x = f.x + gm * hh.x;
        hh.y = f.y + gm * hh.y;
        hh.z = f.z + gm * hh.z;
      }
      g[i] = f;
      h[i] = hh;
      oldx[i] = ox;
    }
    x.x = ox.x + alpha * hh.x;
    x.y = ox.y + alpha * hh.y;
    x.z = ox.z + alpha * hh.z;
    v.pos[i] = x;
  }
  const double4 r = v.ref[i];
  const double dx = x.x - r.x, dy = x.y - r.y, dz = x.z - r.z;
  const double d2 = dx * dx + dy * dy + dz * dz;
  atomicMax(&maxd[sy], (unsigned long long)__double_as_longlong(d2));
}

// any unfinished cell beyond skin/2 -> rebuild the list of the batch
// with per-system rebuilds (sys_rb) only the cells that moved are flagged
__global__ void k_bt_flag(const unsigned long long *maxd, const int *sys_done, int nsys,
                          double skin2, DevScalars *sc, int *sys_rb) {
  int need = 0;
  for (int s = threadIdx.x; s < nsys; s += blockDim.x)
    if (!sys_done[s] && __longlong_as_double((long long)maxd[s]) > skin2) {
      need = 1;
      if (sys_rb) sys_rb[s] = 1;
    }
  need = __syncthreads_or(need);
  if (threadIdx.x == 0 && need) {
    if (sys_rb) atomicOr(&sc->rebuild, RB_FLAGGED);
    else sc->rebuild = RB_ALL;
  }
}

// per-cell sums in a fixed order: energy (per-atom shares in frc.w),
// |F|^2, max component^2, max atom |F|^2, g.g, F.(F-g) (or F.F for
// Fletcher-Reeves); one block per cell
__global__ void __launch_bounds__(256) k_bt_reduce(SysView v, const int *aoff, CgSys *cs,
                                                   const double4 *g, int cg_fr) {
  const int s = blockIdx.x;
  if (v.sys_done[s]) return;
  double e = 0, fn = 0, fm = 0, fa = 0, gg = 0, dgg = 0;
  for (int i = aoff[s] + threadIdx.x; i < aoff[s + 1]; i += blockDim.x) {
    const double4 f = v.frc[i];
    const double4 gi = g[i];
    const double ff = f.x * f.x + f.y * f.y + f.z * f.z;
    e += f.w;
    fn += ff;
    fm = fmax(fm, fmax(fmax(f.x * f.x, f.y * f.y), f.z * f.z));
    fa = fmax(fa, ff);
    gg += gi.x * gi.x + gi.y * gi.y + gi.z * gi.z;
    dgg += cg_fr ? ff : f.x * (f.x - gi.x) + f.y * (f.y - gi.y) + f.z * (f.z - gi.z);
  }
  __shared__ double sh[6][8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  e = warp_sum(e);
  fn = warp_sum(fn);
  fm = warp_max(fm);
  fa = warp_max(fa);
  gg = warp_sum(gg);
  dgg = warp_sum(dgg);
  if (lane == 0) {
    sh[0][w] = e; sh[1][w] = fn; sh[2][w] = fm; sh[3][w] = fa; sh[4][w] = gg; sh[5][w] = dgg;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double r[6] = {0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 8; k++) {
      r[0] += sh[0][k];
      r[1] += sh[1][k];
      r[2] = fmax(r[2], sh[2][k]);
      r[3] = fmax(r[3], sh[3][k]);
      r[4] += sh[4][k];
      r[5] += sh[5][k];
    }
    CgSys &S = cs[s];
    S.E = r[0];
    S.fnorm = r[1];
    S.fmax2 = r[2];
    S.fatom2 = r[3];
    S.gg = r[4];
    S.dgg = r[5];
    S.nfc++;
  }
}

// ---------------------------------------------------------------------------
// The persistent CG engine.  One launch per round replaces the control,
// vector, flag and reduction kernels: resident blocks of BS_ENGINE threads
// take cells from a queue, largest first, and carry each cell through
//   (1) the sums of its last force evaluation (k_bt_reduce's, same order),
//   (2) its control (cg_machine, on thread 0),
//   (3) the move / set_hg / reset of its atoms (k_bt_vec's),
//   (4) its largest displacement since the list build, and the batch's
//       rebuild flag when it passes skin/2 (k_bt_flag's test).
// A cell's atoms are read once for (1) and once for (3) by the same block, so
// the forces, g and h of (1) are still in L1/L2 for (3).  The force passes
// stay separate kernels: they need every cell's list and run at their own
// tuned shapes.
constexpr int BS_ENGINE = 256;  // k_bt_reduce's block: the same summation order

__global__ void __launch_bounds__(BS_ENGINE) k_bt_engine(
    SysView v, const int *aoff, const int *order, CgSys *cs, int nsys, CgParams P,
    int *sys_done, int *sys_short, double4 *oldx, double4 *g, double4 *h,
    unsigned long long *maxd, int *ndone, int *queue, DevScalars *sc, double skin2) {
  __shared__ double sh[6][BS_ENGINE / 32];
  __shared__ CgSys S;
  __shared__ int cell, active;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) {
      const int c = atomicAdd(queue, 1);
      cell = c < nsys ? order[c] : -1;
      active = cell >= 0 && !sys_done[cell];
      if (active) S = cs[cell];
    }
    __syncthreads();
    const int s = cell;
    if (s < 0) break;
    if (active) {
      const int a0 = aoff[s], a1 = aoff[s + 1];
      if (S.eval) {  // (1) k_bt_reduce's sums of the last evaluation
        double e = 0, fn = 0, fm = 0, fa = 0, gg = 0, dgg = 0;
        for (int i = a0 + threadIdx.x; i < a1; i += BS_ENGINE) {
          const double4 f = v.frc[i];
          const double4 gi = g[i];
          const double ff = f.x * f.x + f.y * f.y + f.z * f.z;
          e += f.w;
          fn += ff;
          fm = fmax(fm, fmax(fmax(f.x * f.x, f.y * f.y), f.z * f.z));
          fa = fmax(fa, ff);
          gg += gi.x * gi.x + gi.y * gi.y + gi.z * gi.z;
          dgg += P.cg_fr ? ff : f.x * (f.x - gi.x) + f.y * (f.y - gi.y) + f.z * (f.z - gi.z);
        }
        e = warp_sum(e);
        fn = warp_sum(fn);
        fm = warp_max(fm);
        fa = warp_max(fa);
        gg = warp_sum(gg);
        dgg = warp_sum(dgg);
        if (lane == 0) {
          sh[0][w] = e; sh[1][w] = fn; sh[2][w] = fm; sh[3][w] = fa; sh[4][w] = gg; sh[5][w] = dgg;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          double r[6] = {0, 0, 0, 0, 0, 0};
          for (int k = 0; k < BS_ENGINE / 32; k++) {
            r[0] += sh[0][k];
            r[1] += sh[1][k];
            r[2] = fmax(r[2], sh[2][k]);
            r[3] = fmax(r[3], sh[3][k]);
            r[4] += sh[4][k];
            r[5] += sh[5][k];
          }
          S.E = r[0];
          S.fnorm = r[1];
          S.fmax2 = r[2];
          S.fatom2 = r[3];
          S.gg = r[4];
          S.dgg = r[5];
          S.nfc++;
        }
      }
      if (threadIdx.x == 0) {  // (2) k_bt_control's step
        const bool short_last = sys_short[s] != 0;
        sys_short[s] = 0;
        if (S.pc != PC_DONE) cg_machine(S, P, short_last);
        const int done = (S.pc == PC_DONE);
        if (done) {
          atomicAdd(ndone, 1);
          sys_done[s] = 1;
        }
        S.eval = !done;  // the coming force pass evaluates every unfinished cell
        cs[s] = S;
      }
      __syncthreads();
      // (3) k_bt_vec's update and (4) the displacement of every atom
      const int op = S.op;
      double dmax = 0.0;
      if (op != OP_IDLE) {
        const double alpha = S.alpha, gm = S.gamma;
        for (int i = a0 + threadIdx.x; i < a1; i += BS_ENGINE) {
          double4 x = v.pos[i];
          if (op != OP_NONE) {
            double4 ox = oldx[i], hh = h[i];
            if (op == OP_RESET_MOVE || op == OP_SETHG_MOVE) {
              const double4 f = v.frc[i];
              ox = make_double4(x.x, x.y, x.z, 0.0);
              if (op == OP_RESET_MOVE) {
                hh = f;
              } else {
                hh.x = f.x + gm * hh.x;
                hh.y = f.y + gm * hh.y;
                hh.z = f.z + gm * hh.z;
              }
              g[i] = f;
              h[i] = hh;
              oldx[i] = ox;
            }
            x.x = ox.x + alpha * hh.x;
            x.y = ox.y + alpha * hh.y;
            x.z = ox.z + alpha * hh.z;
            v.pos[i] = x;
          }
          const double4 r = v.ref[i];
          const double dx = x.x - r.x, dy = x.y - r.y, dz = x.z - r.z;
          dmax = fmax(dmax, dx * dx + dy * dy + dz * dz);
        }
      }
      dmax = warp_max(dmax);
      if (lane == 0) sh[0][w] = dmax;
      __syncthreads();
      if (threadIdx.x == 0) {
        double d = 0.0;
        for (int k = 0; k < BS_ENGINE / 32; k++) d = fmax(d, sh[0][k]);
        maxd[s] = (unsigned long long)__double_as_longlong(d);
        if (!sys_done[s] && d > skin2) {
          if (v.sys_rb) {
            v.sys_rb[s] = 1;
            atomicOr(&sc->rebuild, RB_FLAGGED);
          } else {
            atomicExch(&sc->rebuild, RB_ALL);
          }
        }
      }
    }
    __syncthreads();  // cell, active and S are rewritten for the next cell
  }
}

static inline int nblk(long n, int bs) { return (int)((n + bs - 1) / bs); }

int batch_engine_grid() {
  int d = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, d);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_bt_engine, BS_ENGINE, 0) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return nsm * std::max(1, per_sm);
}

void launch_batch_engine(const SysView &v, const int *aoff, const int *order, CgSys *cs,
                         int nsys, const CgParams &P, int *sys_done, int *sys_short,
                         double4 *oldx, double4 *g, double4 *h, unsigned long long *maxd,
                         int *ndone, int *queue, DevScalars *sc, double skin2, int grid,
                         cudaStream_t st) {
  cudaMemsetAsync(queue, 0, sizeof(int), st);
  k_bt_engine<<<std::max(1, std::min(grid, nsys)), BS_ENGINE, 0, st>>>(
      v, aoff, order, cs, nsys, P, sys_done, sys_short, oldx, g, h, maxd, ndone, queue, sc,
      skin2);
}

void launch_batch_round_pre(const SysView &v, CgSys *cs, int nsys, const CgParams &P,
                            int *sys_done, int *sys_short, double4 *oldx, double4 *g,
                            double4 *h, unsigned long long *maxd, int *ndone, DevScalars *sc,
                            double skin2, cudaStream_t st) {
  k_bt_control<<<nblk(nsys, 128), 128, 0, st>>>(cs, nsys, P, sys_done, sys_short, maxd, ndone);
  k_bt_vec<<<nblk(v.n, BS_VEC), BS_VEC, 0, st>>>(v, cs, oldx, g, h, maxd);
  k_bt_flag<<<1, 1024, 0, st>>>(maxd, sys_done, nsys, skin2, sc, v.sys_rb);
}

void launch_batch_round_post(const SysView &v, const int *aoff, CgSys *cs, int nsys,
                             const double4 *g, int cg_fr, cudaStream_t st) {
  k_bt_reduce<<<nsys, 256, 0, st>>>(v, aoff, cs, g, cg_fr);
}

}  // namespace imdgpu
