// forces.cu -- pair and EAM2 force kernels of libimdgpu (sm_103a).
//
// FP64 path: the half neighbour list of make_nblist (IMD pair orientation,
// src/imd_forces_nbl.c:136-273), one thread per real atom, partner updates
// by FP64 atomics, exact (unfused) r^2 and table-index arithmetic so every
// pair sees the same table row as the reference.  Two passes as
// calc_forces (src/imd_forces_nbl.c:423-1323): density (rho), embedding
// F(rho) per atom, then a fused pass that adds the pair force (loop 1's
// PAIR branch) and the EAM force (loop 2) of each pair with one set of
// atomics.
#include <algorithm>

#include "kernels.cuh"

namespace imdgpu {

// ---------------------------------------------------------------------------
// ghosts: send_cells(copy_cell) (src/imd_comm_force_3d.c:247-358).  A ghost
// copies its owner through the z, y, x copies in that order, so its position
// is ((x + s_z box_z) + s_y box_y) + s_x box_x component-wise.
// ---------------------------------------------------------------------------
__global__ void k_ghost_pos(SysView v) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
  {
    const int o = v.gowner[g];
    if (o < 0) continue;  // an unused slot of a system's ghost range
    if (!in_bounds(v, o, v.n, CK_OWNER)) continue;
    v.pos[v.n + g] = ghost_image(v, v.pos[o], v.gcode[g], sys_of(v, o));
  }
}

// ---------------------------------------------------------------------------
// density pass: loop 1 EAM branch (src/imd_forces_nbl.c:586-611, :907-918)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(BS_FORCE_MAX) k_density64(SysView v, DevTable rho) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const double4 pi = v.pos[i];
  const int it = (int)pi.w, nt = v.ntypes;
  const int nn = v.nnb[i];
  unsigned shortf = 0;
  double eam_r = 0.0;
  const uint32_t *nb = v.nbr + i;
  for (int k = 0; k < nn; k++) {
    const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const double4 pj = ldg4(&v.pos[j]);
    const double dx = dsub(pj.x, pi.x), dy = dsub(pj.y, pi.y), dz = dsub(pj.z, pi.z);
    const double r2 = r2_exact(dx, dy, dz);
    const int jt = (int)pj.w;
    const int col = it * nt + jt;
    double rho_h = 0.0;
    if (r2 < rho.end[col]) {
      rho_h = val_func2(rho, col, r2, shortf);
      eam_r += rho_h;
    }
    if (it == jt) {
      if (r2 < rho.end[col]) atomicAdd(&v.rho[j], rho_h);
    } else {
      const int col2 = jt * nt + it;
      if (r2 < rho.end[col2]) atomicAdd(&v.rho[j], val_func2(rho, col2, r2, shortf));
    }
  }
  atomicAdd(&v.rho[i], eam_r);
  if (shortf) flag_short(v, i);
}

// send_forces(add_rho) (src/imd_forces_nbl.c:1076): ghosts into owners
__global__ void k_fold_rho(SysView v) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    // an unused slot of a system's ghost range is normally zero, but the
    // lists of a system that overflowed its range reach into the next
    // range's unused slots until the overflow is replayed: skip them
    const int o = v.gowner[g];
    const double r = v.rho[v.n + g];
    if (r != 0.0 && o >= 0 && in_bounds(v, o, v.n, CK_OWNER)) atomicAdd(&v.rho[o], r);
  }
}

// embedding energy (src/imd_forces_nbl.c:1079-1112): F(rho), EAM_DF = 2F'
__global__ void __launch_bounds__(BS_VEC) k_embed(SysView v, DevTable emb, double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e[1] = {0.0};
  if (i < v.n) {
    const int t = (int)v.pos[i].w;
    unsigned dummy = 0;
    double pot, grad;
    pair_int2(emb, t, v.rho[i], pot, grad, dummy);
    v.df[i] = grad;
    atomicAdd(&v.frc[i].w, pot);
    e[0] = pot;
  }
  block_sum_store<1, BS_VEC>(e, partial);
}

// send_cells(copy_dF) (src/imd_forces_nbl.c:1115)
__global__ void k_ghost_df(SysView v) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int o = v.gowner[g];
    if (o >= 0 && in_bounds(v, o, v.n, CK_OWNER)) v.df[v.n + g] = v.df[o];
  }
}

// ---------------------------------------------------------------------------
// force pass: loop 1 PAIR branch (src/imd_forces_nbl.c:490-584) fused with
// loop 2 (:1117-1323).  Energy: each pair's pot goes to the total once and
// half to each partner's per-atom energy (POTENG).  Virial as in the
// reference: -r^2 grad for the pair part, -d.F for the EAM part.
// ---------------------------------------------------------------------------
template <bool EAM>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_force64(SysView v, DevTable pair, DevTable rho,
                                                      double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};  // energy, virial
  if (i < v.n) {
    const double4 pi = v.pos[i];
    const int it = (int)pi.w, nt = v.ntypes;
    const int nn = v.nnb[i];
    const double dfi = EAM ? v.df[i] : 0.0;
    unsigned shortf = 0;
    double ffx = 0.0, ffy = 0.0, ffz = 0.0, ee = 0.0;
    const uint32_t *nb = v.nbr + i;
    for (int k = 0; k < nn; k++) {
      const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
      if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
      const double4 pj = ldg4(&v.pos[j]);
      const double dx = dsub(pj.x, pi.x), dy = dsub(pj.y, pi.y), dz = dsub(pj.z, pi.z);
      const double r2 = r2_exact(dx, dy, dz);
      const int jt = (int)pj.w;
      const int col = it * nt + jt;
      double grad = 0.0, ehalf = 0.0;
      bool have = false;
      if (r2 <= pair.end[col]) {
        double pot, gp;
        pair_int2(pair, col, r2, pot, gp, shortf);
        acc[0] += pot;
        acc[1] -= r2 * gp;
        ehalf = 0.5 * pot;
        ee += ehalf;
        grad = gp;
        have = true;
      }
      if (EAM) {
        const int col1 = jt * nt + it, col2 = col;
        if ((r2 < rho.end[col1]) || (r2 < rho.end[col2])) {
          const double ris = deriv_func2(rho, col1, r2, shortf);
          const double rjs = (col1 == col2) ? ris : deriv_func2(rho, col2, r2, shortf);
          const double dfj = __ldg(&v.df[j]);
          const double ge = 0.5 * (dfi * rjs + dfj * ris);
          acc[1] -= r2 * ge;
          grad += ge;
          have = true;
        }
      }
      if (have) {
        const double fx = dx * grad, fy = dy * grad, fz = dz * grad;
        double *fj = &v.frc[j].x;
        atomicAdd(fj + 0, -fx);
        atomicAdd(fj + 1, -fy);
        atomicAdd(fj + 2, -fz);
        if (ehalf != 0.0) atomicAdd(fj + 3, ehalf);
        ffx += fx;
        ffy += fy;
        ffz += fz;
      }
    }
    double *fi = &v.frc[i].x;
    atomicAdd(fi + 0, ffx);
    atomicAdd(fi + 1, ffy);
    atomicAdd(fi + 2, ffz);
    atomicAdd(fi + 3, ee);
    if (shortf) flag_short(v, i);
  }
  block_sum_store_dyn<2, BS_FORCE_MAX>(acc, partial);
}

// send_forces(add_forces) (src/imd_forces_nbl.c:1997)
__global__ void k_fold_force(SysView v) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const double4 f = v.frc[v.n + g];
    const int own = v.gowner[g];  // -1: an unused slot (see k_fold_rho)
    if (own >= 0 && (f.x != 0.0 || f.y != 0.0 || f.z != 0.0 || f.w != 0.0) &&
        in_bounds(v, own, v.n, CK_OWNER)) {
      double *o = &v.frc[own].x;
      atomicAdd(o + 0, f.x);
      atomicAdd(o + 1, f.y);
      atomicAdd(o + 2, f.z);
      atomicAdd(o + 3, f.w);
    }
  }
}

// energy / virial: fixed-order sum of block partials (the MPI_Allreduce of
// 8 scalars, src/imd_forces_nbl.c:1975-1994, on one device)
__global__ void k_finalize_forces(const double *pe, int ne, const double *pf, int nf,
                                  DevScalars *sc) {
  double v[2] = {0.0, 0.0};
  for (int b = threadIdx.x; b < ne; b += FIN_BS) v[0] += pe[b];
  for (int b = threadIdx.x; b < nf; b += FIN_BS) {
    v[0] += pf[2 * b];
    v[1] += pf[2 * b + 1];
  }
  fin_block<2, 0u>(v);
  if (threadIdx.x == 0) {
    sc->epot = v[0];
    sc->virial = v[1];
  }
}

// ---------------------------------------------------------------------------
// fast FP64 kernels: coefficient-form tables with FMA, integer-domain cutoff
// tests, one table index per pair when pair and rho share their grid, single
// type specialisation, per-atom energy scatter only when requested.  Same
// pairs and formulas as above; only rounding differs (~1e-16 relative).
// ---------------------------------------------------------------------------
template <bool NT1, bool CUB>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_density_fast(SysView v, DevTable rho) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || atom_idle(v, i)) return;
  const double4 pi = v.pos[i];
  const int it = NT1 ? 0 : (int)pi.w, nt = v.ntypes;
  const int nn = v.nnb[i];
  bool shortf = false;
  double eam_r = 0.0;
  const uint32_t *__restrict__ nb = v.nbr + i;
#pragma unroll 2
  for (int k = 0; k < nn; k++) {
    const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const double4 pj = ldg4(&v.pos[j]);
    const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
    const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
    const int jt = NT1 ? 0 : (int)pj.w;
    const int col = NT1 ? 0 : it * nt + jt;
    double rho_h = 0.0;
    if (lt_pos(r2, rho.end[col])) {
      double chi;
      const int kk = tab_index_fast(rho, col, r2, chi);
      rho_h = poly_v<CUB>(cv_load(rho, col, kk), chi);
      eam_r += rho_h;
      shortf |= lt_pos(r2, rho.begin[col]);
    }
    if (NT1 || it == jt) {
      if (lt_pos(r2, rho.end[col])) atomicAdd(&v.rho[j], rho_h);
    } else {
      const int col2 = jt * nt + it;
      if (lt_pos(r2, rho.end[col2])) {
        double chi;
        const int kk = tab_index_fast(rho, col2, r2, chi);
        atomicAdd(&v.rho[j], poly_v<CUB>(cv_load(rho, col2, kk), chi));
        shortf |= lt_pos(r2, rho.begin[col2]);
      }
    }
  }
  atomicAdd(&v.rho[i], eam_r);
  if (shortf) flag_short(v, i);
}

template <bool NT1, bool EAM, bool EPOT, bool SAMEGRID, bool CUB>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_force_fast(SysView v, DevTable pair, DevTable rho,
                                                         double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};  // energy, virial
  if (i < v.n && !atom_idle(v, i)) {
    const double4 pi = v.pos[i];
    const int it = NT1 ? 0 : (int)pi.w, nt = v.ntypes;
    const int nn = v.nnb[i];
    const double dfi = EAM ? v.df[i] : 0.0;
    bool shortf = false;
    // ng* = minus the gradient: the partner's force d * ng is used as is
    double fnx = 0.0, fny = 0.0, fnz = 0.0, ee = 0.0, esum = 0.0, vir = 0.0;
    const uint32_t *__restrict__ nb = v.nbr + i;
#pragma unroll 2
    for (int k = 0; k < nn; k++) {
      const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
      if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
      const double4 pj = ldg4(&v.pos[j]);
      const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
      const int jt = NT1 ? 0 : (int)pj.w;
      const int col = NT1 ? 0 : it * nt + jt;
      double ngrad = 0.0, ehalf = 0.0;
      bool have = false;
      int kk = 0;
      double chi = 0.0;
      if (le_pos(r2, pair.end[col])) {
        kk = tab_index_fast(pair, col, r2, chi);
        const double pot = poly_v<CUB>(cv_load(pair, col, kk), chi);
        ngrad = poly_g<CUB>(cgn_load(pair, col, kk), chi);
        esum += pot;
        if (EPOT) {
          ehalf = 0.5 * pot;
          ee += ehalf;
        }
        shortf |= lt_pos(r2, pair.begin[col]);
        have = true;
      }
      if (EAM) {
        const int col1 = NT1 ? 0 : jt * nt + it, col2 = col;
        if (lt_pos(r2, rho.end[col1]) || lt_pos(r2, rho.end[col2])) {
          double chi1 = chi;
          int k1 = kk;
          if (!(SAMEGRID && have)) k1 = tab_index_fast(rho, col1, r2, chi1);
          // rho.cgn holds -rho'/2
          const double nris = poly_g<CUB>(cgn_load(rho, col1, k1), chi1);
          const double dfj = __ldg(&v.df[j]);
          if (NT1 || col1 == col2) {
            ngrad = fma(nris, dfi + dfj, ngrad);
          } else {
            double chi2 = chi;
            int k2 = kk;
            if (!(SAMEGRID && have)) k2 = tab_index_fast(rho, col2, r2, chi2);
            const double nrjs = poly_g<CUB>(cgn_load(rho, col2, k2), chi2);
            ngrad = fma(dfi, nrjs, fma(dfj, nris, ngrad));
          }
          have = true;
        }
      }
      if (have) {
        const double fx = dx * ngrad, fy = dy * ngrad, fz = dz * ngrad;
        double *fj = &v.frc[j].x;
        atomicAdd(fj + 0, fx);
        atomicAdd(fj + 1, fy);
        atomicAdd(fj + 2, fz);
        if (EPOT) atomicAdd(fj + 3, ehalf);
        fnx += fx;
        fny += fy;
        fnz += fz;
        vir = fma(r2, ngrad, vir);
      }
    }
    double *fi = &v.frc[i].x;
    atomicAdd(fi + 0, -fnx);
    atomicAdd(fi + 1, -fny);
    atomicAdd(fi + 2, -fnz);
    if (EPOT) atomicAdd(fi + 3, ee);
    // energy share of the atom: its own half-list pairs (deterministic order)
    if (!EPOT && v.eshare) atomicAdd(fi + 3, esum);
    acc[0] = esum;
    acc[1] = vir;
    if (shortf) flag_short(v, i);
  }
  block_sum_store_dyn<2, BS_FORCE_MAX>(acc, partial);
}

// ---------------------------------------------------------------------------
// Pair cache (imdgpu_set_pair_cache): one species, EAM2, pair and density
// tables on one grid.  The density pass computes r^2 and the table index of
// every half-list pair anyway; it also evaluates the pair's table terms the
// force pass needs and stores them per list entry, column-major like the
// list (entry k of atom i at k * ncap + i): r^2, the pair term of -grad
// (phi' from cgn), -rho'/2 and phi, or r^2 = -1 beyond both cutoffs.  The
// force pass streams them and gathers only the partner's position and F'.
// Both passes are bound by the FP64 pipe with DRAM nearly idle, so 32 bytes
// written and read per entry buy back the r^2, index and table arithmetic
// of the second pass.  Formulas and order are k_density_fast's and
// k_force_fast's, so every pair term is the same bits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void st_stream(double4 *p, const double4 c) {
  double2 *q = reinterpret_cast<double2 *>(p);
  __stcs(q, make_double2(c.x, c.y));
  __stcs(q + 1, make_double2(c.z, c.w));
}
__device__ __forceinline__ double4 ld_stream(const double4 *p) {
  const double2 *q = reinterpret_cast<const double2 *>(p);
  const double2 a = __ldcs(q), b = __ldcs(q + 1);
  return make_double4(a.x, a.y, b.x, b.y);
}

// LPA lanes serve one atom (the autotuner's tile dimension: 1, 2 or 4):
// lane q takes the entries q, q + LPA, ... of the atom's list and the lanes'
// sums meet in a shuffle tree of the lane group.  More lanes per atom give
// more warps when few atoms are active (the end of a batched relaxation).
template <int LPA>
__device__ __forceinline__ unsigned lane_group_mask() {
  if (LPA == 1) return 1u << (threadIdx.x & 31);
  const unsigned g = (1u << LPA) - 1u;
  return g << ((threadIdx.x & 31) & ~(LPA - 1));
}
template <int LPA>
__device__ __forceinline__ double group_sum(double x, unsigned mask) {
#pragma unroll
  for (int o = 1; o < LPA; o <<= 1) x += __shfl_xor_sync(mask, x, o);
  return x;
}

template <bool CUB, int LPA>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_density_cache(SysView v, DevTable pair,
                                                            DevTable rho) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gid / LPA), q = (int)(gid % LPA);
  if (i >= v.n || atom_idle(v, i)) return;  // the whole lane group alike
  const unsigned mask = lane_group_mask<LPA>();
  const double4 pi = v.pos[i];
  const int nn = v.nnb[i];
  bool shortf = false;
  double eam_r = 0.0;
  const uint32_t *__restrict__ nb = v.nbr + i;
  double4 *__restrict__ pc = v.pcache + i;
#pragma unroll 2
  for (int k = q; k < nn; k += LPA) {
    const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const double4 pj = ldg4(&v.pos[j]);
    const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
    const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
    double4 c = make_double4(-1.0, 0.0, 0.0, 0.0);
    const bool inp = le_pos(r2, pair.end[0]), inr = lt_pos(r2, rho.end[0]);
    if (inp || inr) {
      double chi;
      const int kk = tab_index_fast(pair, 0, r2, chi);  // rho's index too: one grid
      c.x = r2;
      if (inp) {
        c.w = poly_v<CUB>(cv_load(pair, 0, kk), chi);
        c.y = poly_g<CUB>(cgn_load(pair, 0, kk), chi);
      }
      if (inr) {
        const double rho_h = poly_v<CUB>(cv_load(rho, 0, kk), chi);
        eam_r += rho_h;
        atomicAdd(&v.rho[j], rho_h);
        c.z = poly_g<CUB>(cgn_load(rho, 0, kk), chi);  // rho.cgn holds -rho'/2
      }
      shortf |= lt_pos(r2, pair.begin[0]);
    }
    st_stream(pc + (size_t)k * v.ncap, c);
  }
  eam_r = group_sum<LPA>(eam_r, mask);
  if (q == 0) atomicAdd(&v.rho[i], eam_r);
  if (shortf) flag_short(v, i);
}

template <bool EPOT, int LPA>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_force_cache(SysView v, double *partial) {
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gid / LPA), q = (int)(gid % LPA);
  double acc[2] = {0.0, 0.0};  // energy, virial
  if (i < v.n && !atom_idle(v, i)) {  // the whole lane group alike
    const unsigned mask = lane_group_mask<LPA>();
    const double4 pi = v.pos[i];
    const int nn = v.nnb[i];
    const double dfi = v.df[i];
    double fnx = 0.0, fny = 0.0, fnz = 0.0, ee = 0.0, esum = 0.0, vir = 0.0;
    const uint32_t *__restrict__ nb = v.nbr + i;
    const double4 *__restrict__ pc = v.pcache + i;
#pragma unroll 2
    for (int k = q; k < nn; k += LPA) {
      const double4 c = ld_stream(pc + (size_t)k * v.ncap);
      if (c.x < 0.0) continue;  // beyond both cutoffs
      const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
      if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
      const double4 pj = ldg4(&v.pos[j]);
      const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const double dfj = __ldg(&v.df[j]);
      // c.z = 0 outside rho's cutoff and c.y = 0 outside phi's: the fma
      // then returns the other term exactly, as the two branches would
      const double ngrad = fma(c.z, dfi + dfj, c.y);
      esum += c.w;
      const double fx = dx * ngrad, fy = dy * ngrad, fz = dz * ngrad;
      double *fj = &v.frc[j].x;
      atomicAdd(fj + 0, fx);
      atomicAdd(fj + 1, fy);
      atomicAdd(fj + 2, fz);
      if (EPOT) {
        const double ehalf = 0.5 * c.w;
        ee += ehalf;
        atomicAdd(fj + 3, ehalf);
      }
      fnx += fx;
      fny += fy;
      fnz += fz;
      vir = fma(c.x, ngrad, vir);
    }
    fnx = group_sum<LPA>(fnx, mask);
    fny = group_sum<LPA>(fny, mask);
    fnz = group_sum<LPA>(fnz, mask);
    esum = group_sum<LPA>(esum, mask);
    vir = group_sum<LPA>(vir, mask);
    if (EPOT) ee = group_sum<LPA>(ee, mask);
    if (q == 0) {
      double *fi = &v.frc[i].x;
      atomicAdd(fi + 0, -fnx);
      atomicAdd(fi + 1, -fny);
      atomicAdd(fi + 2, -fnz);
      if (EPOT) atomicAdd(fi + 3, ee);
      if (!EPOT && v.eshare) atomicAdd(fi + 3, esum);
      acc[0] = esum;
      acc[1] = vir;
    }
  }
  block_sum_store_dyn<2, BS_FORCE_MAX>(acc, partial);
}

template <int LPA>
static void launch_cache_passes(const ForceTabs &t, const SysView &v, int which, double *pf,
                                cudaStream_t st) {
  const long threads = (long)v.n * LPA;
  if (which == 0) {
    const int nb = (int)((threads + t.bs_rho - 1) / t.bs_rho);
    if (t.rho.mode == TAB_QUADRATIC)
      k_density_cache<false, LPA><<<nb, t.bs_rho, 0, st>>>(v, t.pair, t.rho);
    else
      k_density_cache<true, LPA><<<nb, t.bs_rho, 0, st>>>(v, t.pair, t.rho);
  } else {
    const int nb = (int)((threads + t.bs - 1) / t.bs);
    if (t.epot) k_force_cache<true, LPA><<<nb, t.bs, 0, st>>>(v, pf);
    else k_force_cache<false, LPA><<<nb, t.bs, 0, st>>>(v, pf);
  }
}
// which: 0 the density pass, 1 the force pass
static void launch_cache(const ForceTabs &t, const SysView &v, int which, double *pf,
                         cudaStream_t st) {
  if (t.lpa == 4) launch_cache_passes<4>(t, v, which, pf, st);
  else if (t.lpa == 2) launch_cache_passes<2>(t, v, which, pf, st);
  else launch_cache_passes<1>(t, v, which, pf, st);
}

// ---------------------------------------------------------------------------
// Deterministic FP64 passes (imdgpu_set_deterministic).  The half-list
// kernels above add the reaction on the second atom of a pair with FP64
// atomics, so the order of the per-atom sums, and their last bits, change
// from run to run.  These kernels use the full list instead (every pair in
// both directions, as the mixed path does): each atom owns its sums.  A quad
// of four consecutive lanes serves one atom: lane q takes the entries
// q, q + 4, q + 8, ... of the atom's list in order, and the four partial
// sums of rho, of the force, the energy and the virial are combined by a
// fixed shuffle tree, (l0 + l1) + (l2 + l3).  Same pairs, tables and
// formulas as k_density_fast / k_force_fast; twice the pair arithmetic.
// ---------------------------------------------------------------------------
constexpr int DET_Q = 4;  // lanes per atom

__device__ __forceinline__ double quad_sum(double x) {
  x += __shfl_xor_sync(0xffffffffu, x, 1);
  return x + __shfl_xor_sync(0xffffffffu, x, 2);
}

// rho_i = sum_j rho_{it,jt}(r_ij) over the full list (loop 1's eam_r,
// src/imd_forces_nbl.c:586-611, for the atom that receives)
template <bool NT1, bool CUB>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_density_det(SysView v, DevTable rho) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gid / DET_Q, q = gid % DET_Q;
  const bool live = i < v.n && !atom_idle(v, i);
  double r = 0.0;
  bool shortf = false;
  if (live) {
    const double4 pi = v.pos[i];
    const int it = NT1 ? 0 : (int)pi.w, nt = v.ntypes;
    const int nn = v.nnb[i];
    const uint32_t *__restrict__ nb = v.nbr + i;
    for (int k = q; k < nn; k += DET_Q) {
      const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
      if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
      const double4 pj = ldg4(&v.pos[j]);
      const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
      const int col = NT1 ? 0 : it * nt + (int)pj.w;
      if (lt_pos(r2, rho.end[col])) {
        double chi;
        const int kk = tab_index_fast(rho, col, r2, chi);
        r += poly_v<CUB>(cv_load(rho, col, kk), chi);
        shortf |= lt_pos(r2, rho.begin[col]);
      }
    }
  }
  r = quad_sum(r);
  if (live && q == 0) v.rho[i] = r;
  if (live && shortf) flag_short(v, i);
}

template <bool NT1, bool EAM, bool SAMEGRID, bool CUB>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_force_det(SysView v, DevTable pair, DevTable rho,
                                                        double *partial) {
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = gid / DET_Q, q = gid % DET_Q;
  const bool live = i < v.n && !atom_idle(v, i);
  // f* = sum of d * (minus the gradient); the atom's force is -f
  double fx = 0.0, fy = 0.0, fz = 0.0, ee = 0.0, vir = 0.0;
  bool shortf = false;
  if (live) {
    const double4 pi = v.pos[i];
    const int it = NT1 ? 0 : (int)pi.w, nt = v.ntypes;
    const int nn = v.nnb[i];
    const double dfi = EAM ? v.df[i] : 0.0;
    const uint32_t *__restrict__ nb = v.nbr + i;
    for (int k = q; k < nn; k += DET_Q) {
      const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
      if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
      const double4 pj = ldg4(&v.pos[j]);
      const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
      const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
      const int jt = NT1 ? 0 : (int)pj.w;
      const int col = NT1 ? 0 : it * nt + jt;
      double ngrad = 0.0;
      bool have = false;
      int kk = 0;
      double chi = 0.0;
      if (le_pos(r2, pair.end[col])) {
        kk = tab_index_fast(pair, col, r2, chi);
        ee = fma(0.5, poly_v<CUB>(cv_load(pair, col, kk), chi), ee);
        ngrad = poly_g<CUB>(cgn_load(pair, col, kk), chi);
        shortf |= lt_pos(r2, pair.begin[col]);
        have = true;
      }
      if (EAM) {
        const int col1 = NT1 ? 0 : jt * nt + it, col2 = col;
        if (lt_pos(r2, rho.end[col1]) || lt_pos(r2, rho.end[col2])) {
          double chi1 = chi;
          int k1 = kk;
          if (!(SAMEGRID && have)) k1 = tab_index_fast(rho, col1, r2, chi1);
          const double nris = poly_g<CUB>(cgn_load(rho, col1, k1), chi1);
          const double dfj = __ldg(&v.df[j]);
          if (NT1 || col1 == col2) {
            ngrad = fma(nris, dfi + dfj, ngrad);
          } else {
            double chi2 = chi;
            int k2 = kk;
            if (!(SAMEGRID && have)) k2 = tab_index_fast(rho, col2, r2, chi2);
            const double nrjs = poly_g<CUB>(cgn_load(rho, col2, k2), chi2);
            ngrad = fma(dfi, nrjs, fma(dfj, nris, ngrad));
          }
          have = true;
        }
      }
      if (have) {
        fx = fma(dx, ngrad, fx);
        fy = fma(dy, ngrad, fy);
        fz = fma(dz, ngrad, fz);
        vir = fma(r2, ngrad, vir);
      }
    }
  }
  fx = quad_sum(fx);
  fy = quad_sum(fy);
  fz = quad_sum(fz);
  ee = quad_sum(ee);
  vir = quad_sum(vir);
  double acc[2] = {0.0, 0.0};  // energy, virial (each pair counted from both atoms)
  if (live && q == 0) {
    double4 f = v.frc[i];  // .w holds the embedding energy
    f.x = -fx;
    f.y = -fy;
    f.z = -fz;
    f.w += ee;
    v.frc[i] = f;
    acc[0] = ee;
    acc[1] = 0.5 * vir;
  }
  if (live && shortf) flag_short(v, i);
  block_sum_store_dyn<2, BS_FORCE_MAX>(acc, partial);
}

// embedding with the coefficient-form table
__global__ void __launch_bounds__(BS_VEC) k_embed_fast(SysView v, DevTable emb, double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e[1] = {0.0};
  if (i < v.n && !atom_idle(v, i)) {
    const int t = (int)v.pos[i].w;
    double chi;
    const int k = tab_index_fast(emb, t, v.rho[i], chi);
    const double pot = poly_v<true>(cv_load(emb, t, k), chi);
    v.df[i] = poly_g<true>(cg_load(emb, t, k), chi);
    atomicAdd(&v.frc[i].w, pot);
    e[0] = pot;
  }
  block_sum_store<1, BS_VEC>(e, partial);
}

// ---------------------------------------------------------------------------
// STRESS_TENS (src/imd_forces_nbl.c:558-580, :1284-1318): for every pair the
// pair + EAM force f = d grad is halved ("avoid double counting of the
// virial") and -d_a f_b is added to both atoms; components xx yy zz yz zx xy
// (sym_tensor).  A pass of its own after the force passes (it reads 2F' of
// every atom), run on the steps that want pressure (IMD's do_press_calc), so
// the force pass of the other steps stays as it is.  Ghost sums fold into
// their owners afterwards (send_forces(add_forces), src/imd_comm_force_3d.c:916).
// ---------------------------------------------------------------------------
template <bool NT1, bool EAM, bool SAMEGRID, bool CUB>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_stress_fast(SysView v, DevTable pair,
                                                          DevTable rho, double *stress) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n || atom_idle(v, i)) return;
  const double4 pi = v.pos[i];
  const int it = NT1 ? 0 : (int)pi.w, nt = v.ntypes;
  const int nn = v.nnb[i];
  const double dfi = EAM ? v.df[i] : 0.0;
  double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  const uint32_t *__restrict__ nb = v.nbr + i;
  for (int k = 0; k < nn; k++) {
    const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const double4 pj = ldg4(&v.pos[j]);
    const double dx = pj.x - pi.x, dy = pj.y - pi.y, dz = pj.z - pi.z;
    const double r2 = fma(dx, dx, fma(dy, dy, dz * dz));
    const int jt = NT1 ? 0 : (int)pj.w;
    const int col = NT1 ? 0 : it * nt + jt;
    double ngrad = 0.0;  // minus grad of the pair: the force on j is d * ngrad
    bool have = false;
    int kk = 0;
    double chi = 0.0;
    if (le_pos(r2, pair.end[col])) {
      kk = tab_index_fast(pair, col, r2, chi);
      ngrad = poly_g<CUB>(cgn_load(pair, col, kk), chi);
      have = true;
    }
    if (EAM) {
      const int col1 = NT1 ? 0 : jt * nt + it, col2 = col;
      if (lt_pos(r2, rho.end[col1]) || lt_pos(r2, rho.end[col2])) {
        double chi1 = chi;
        int k1 = kk;
        if (!(SAMEGRID && have)) k1 = tab_index_fast(rho, col1, r2, chi1);
        const double nris = poly_g<CUB>(cgn_load(rho, col1, k1), chi1);
        const double dfj = __ldg(&v.df[j]);
        if (NT1 || col1 == col2) {
          ngrad = fma(nris, dfi + dfj, ngrad);
        } else {
          double chi2 = chi;
          int k2 = kk;
          if (!(SAMEGRID && have)) k2 = tab_index_fast(rho, col2, r2, chi2);
          const double nrjs = poly_g<CUB>(cgn_load(rho, col2, k2), chi2);
          ngrad = fma(dfi, nrjs, fma(dfj, nris, ngrad));
        }
        have = true;
      }
    }
    if (have) {
      // -d_a (f_b / 2) with f = -d * ngrad on i
      const double h = 0.5 * ngrad;
      const double hx = dx * h, hy = dy * h, hz = dz * h;
      const double c[6] = {dx * hx, dy * hy, dz * hz, dy * hz, dz * hx, dx * hy};
      double *sj = stress + 6 * (size_t)j;
#pragma unroll
      for (int q = 0; q < 6; q++) {
        acc[q] += c[q];
        atomicAdd(sj + q, c[q]);
      }
    }
  }
  double *si = stress + 6 * (size_t)i;
#pragma unroll
  for (int q = 0; q < 6; q++) atomicAdd(si + q, acc[q]);
}

__global__ void k_fold_stress(SysView v, double *stress) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int o = v.gowner[g];
    if (o < 0) continue;  // an unused slot of a system's ghost range
    if (!in_bounds(v, o, v.n, CK_OWNER)) continue;
    const double *sg = stress + 6 * (size_t)(v.n + g);
    double *so = stress + 6 * (size_t)o;
#pragma unroll
    for (int q = 0; q < 6; q++)
      if (sg[q] != 0.0) atomicAdd(so + q, sg[q]);
  }
}

template <bool NT1, bool EAM>
static void launch_stress2(const ForceTabs &t, const SysView &v, double *stress, cudaStream_t st) {
  const int nb = (v.n + t.bs - 1) / t.bs;
  const bool cub = (t.pair.mode != TAB_QUADRATIC);
  if (t.samegrid) {
    if (cub) k_stress_fast<NT1, EAM, true, true><<<nb, t.bs, 0, st>>>(v, t.pair, t.rho, stress);
    else k_stress_fast<NT1, EAM, true, false><<<nb, t.bs, 0, st>>>(v, t.pair, t.rho, stress);
  } else {
    if (cub) k_stress_fast<NT1, EAM, false, true><<<nb, t.bs, 0, st>>>(v, t.pair, t.rho, stress);
    else k_stress_fast<NT1, EAM, false, false><<<nb, t.bs, 0, st>>>(v, t.pair, t.rho, stress);
  }
}

int launch_stress(const SysView &v, const ForceTabs &t, double *stress, cudaStream_t st) {
  const size_t ext = (size_t)v.ncap + v.gcap;
  cudaMemsetAsync(stress, 0, 6 * ext * sizeof(double), st);
  if (t.eam) {
    if (t.nt1) launch_stress2<true, true>(t, v, stress, st);
    else launch_stress2<false, true>(t, v, stress, st);
  } else {
    if (t.nt1) launch_stress2<true, false>(t, v, stress, st);
    else launch_stress2<false, false>(t, v, stress, st);
  }
  const int gblocks = std::max(1, (int)((v.gcap + BS_VEC - 1) / BS_VEC));
  k_fold_stress<<<gblocks, BS_VEC, 0, st>>>(v, stress);
  return 2;
}

template <bool NT1, bool EAM, bool EPOT>
static void launch_force_fast(int samegrid, int nbf, cudaStream_t st, const SysView &v,
                              const ForceTabs &t, double *pf) {
  const bool cub = (t.pair.mode != TAB_QUADRATIC);
  if (samegrid) {
    if (cub) k_force_fast<NT1, EAM, EPOT, true, true><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    else k_force_fast<NT1, EAM, EPOT, true, false><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
  } else {
    if (cub) k_force_fast<NT1, EAM, EPOT, false, true><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    else k_force_fast<NT1, EAM, EPOT, false, false><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
  }
}

template <bool EAM, bool EPOT>
static void launch_force_fast2(const ForceTabs &t, int nbf, cudaStream_t st, const SysView &v,
                               double *pf) {
  if (t.nt1)
    launch_force_fast<true, EAM, EPOT>(t.samegrid, nbf, st, v, t, pf);
  else
    launch_force_fast<false, EAM, EPOT>(t.samegrid, nbf, st, v, t, pf);
}

static void launch_force_any(const ForceTabs &t, int nbf, cudaStream_t st, const SysView &v,
                             double *pf) {
  if (t.exact && t.pair.mode == TAB_QUADRATIC) {
    if (t.eam) k_force64<true><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    else k_force64<false><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    return;
  }
  if (t.eam) {
    if (t.epot) launch_force_fast2<true, true>(t, nbf, st, v, pf);
    else launch_force_fast2<true, false>(t, nbf, st, v, pf);
  } else {
    if (t.epot) launch_force_fast2<false, true>(t, nbf, st, v, pf);
    else launch_force_fast2<false, false>(t, nbf, st, v, pf);
  }
}

static inline int nblk(long n, int bs) { return (int)((n + bs - 1) / bs); }

void k_ghost_pos_launch(const SysView &v, int blocks, cudaStream_t st) {
  k_ghost_pos<<<blocks, BS_VEC, 0, st>>>(v);
}
void fold_rho_launch(const SysView &v, int blocks, cudaStream_t st) {
  k_fold_rho<<<blocks, BS_VEC, 0, st>>>(v);
}
void fold_force_launch(const SysView &v, int blocks, cudaStream_t st) {
  k_fold_force<<<blocks, BS_VEC, 0, st>>>(v);
}

template <bool NT1, bool EAM>
static void launch_force_det(const ForceTabs &t, int nq, cudaStream_t st, const SysView &v,
                             double *pf) {
  const bool cub = (t.pair.mode != TAB_QUADRATIC);
  if (t.samegrid) {
    if (cub) k_force_det<NT1, EAM, true, true><<<nq, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    else k_force_det<NT1, EAM, true, false><<<nq, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
  } else {
    if (cub) k_force_det<NT1, EAM, false, true><<<nq, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
    else k_force_det<NT1, EAM, false, false><<<nq, t.bs, 0, st>>>(v, t.pair, t.rho, pf);
  }
}

// the deterministic FP64 sequence: ghosts, density (quads, full list),
// embedding, 2F' to the ghosts, force (quads, full list), totals; no
// atomics on per-atom sums and no ghost folds
static int launch_forces_det(const SysView &v, const ForceTabs &t, DevScalars *sc,
                             cudaStream_t st, cudaEvent_t *ev) {
  const int gblocks = nblk(v.gcap, BS_VEC) > 0 ? nblk(v.gcap, BS_VEC) : 1;
  const size_t ext = (size_t)v.ncap + v.gcap;
  cudaMemsetAsync(v.frc, 0, ext * sizeof(double4), st);
  k_ghost_pos<<<gblocks, BS_VEC, 0, st>>>(v);
  const long lanes = (long)v.n * DET_Q;
  const int nq = nblk(lanes, t.bs), nqr = nblk(lanes, t.bs_rho), nbe = nblk(v.n, BS_VEC);
  double *pe = v.partial, *pf = v.partial + nbe;
  if (t.eam) {
    if (ev) cudaEventRecord(ev[0], st);
    const bool cubr = (t.rho.mode != TAB_QUADRATIC);
    if (t.nt1 && !cubr) k_density_det<true, false><<<nqr, t.bs_rho, 0, st>>>(v, t.rho);
    else if (t.nt1) k_density_det<true, true><<<nqr, t.bs_rho, 0, st>>>(v, t.rho);
    else if (!cubr) k_density_det<false, false><<<nqr, t.bs_rho, 0, st>>>(v, t.rho);
    else k_density_det<false, true><<<nqr, t.bs_rho, 0, st>>>(v, t.rho);
    if (ev) cudaEventRecord(ev[1], st);
    k_embed_fast<<<nbe, BS_VEC, 0, st>>>(v, t.embed, pe);
    k_ghost_df<<<gblocks, BS_VEC, 0, st>>>(v);
    if (ev) cudaEventRecord(ev[2], st);
    if (t.nt1) launch_force_det<true, true>(t, nq, st, v, pf);
    else launch_force_det<false, true>(t, nq, st, v, pf);
    if (ev) cudaEventRecord(ev[3], st);
  } else {
    if (ev) {
      cudaEventRecord(ev[0], st);
      cudaEventRecord(ev[1], st);
      cudaEventRecord(ev[2], st);
    }
    if (t.nt1) launch_force_det<true, false>(t, nq, st, v, pf);
    else launch_force_det<false, false>(t, nq, st, v, pf);
    if (ev) cudaEventRecord(ev[3], st);
  }
  k_finalize_forces<<<1, FIN_BS, 0, st>>>(pe, t.eam ? nbe : 0, pf, nq, sc);
  return t.eam ? 7 : 4;
}

int launch_forces(const SysView &v, const ForceTabs &t, DevScalars *sc, int mixed,
                  cudaStream_t st, cudaEvent_t *ev) {
  if (mixed) return launch_forces_mixed(v, t, sc, st, ev);
  if (t.det) return launch_forces_det(v, t, sc, st, ev);
  int launches = 0;
  const int gblocks = nblk(v.gcap, BS_VEC) > 0 ? nblk(v.gcap, BS_VEC) : 1;
  const size_t ext = (size_t)v.ncap + v.gcap;
  cudaMemsetAsync(v.frc, 0, ext * sizeof(double4), st);
  k_ghost_pos<<<gblocks, BS_VEC, 0, st>>>(v);
  launches++;
  const int lpa = t.cache ? t.lpa : 1;
  const int nbf = nblk((long)v.n * lpa, t.bs), nbe = nblk(v.n, BS_VEC), nbr = nblk(v.n, t.bs_rho);
  double *pe = v.partial, *pf = v.partial + nbe;
  if (t.eam) {
    cudaMemsetAsync(v.rho, 0, ext * sizeof(double), st);
    if (ev) cudaEventRecord(ev[0], st);
    const bool quad = (t.rho.mode == TAB_QUADRATIC);
    if (t.cache) launch_cache(t, v, 0, nullptr, st);
    else if (t.exact && quad) k_density64<<<nbr, t.bs_rho, 0, st>>>(v, t.rho);
    else if (t.nt1 && quad) k_density_fast<true, false><<<nbr, t.bs_rho, 0, st>>>(v, t.rho);
    else if (t.nt1) k_density_fast<true, true><<<nbr, t.bs_rho, 0, st>>>(v, t.rho);
    else if (quad) k_density_fast<false, false><<<nbr, t.bs_rho, 0, st>>>(v, t.rho);
    else k_density_fast<false, true><<<nbr, t.bs_rho, 0, st>>>(v, t.rho);
    if (ev) cudaEventRecord(ev[1], st);
    k_fold_rho<<<gblocks, BS_VEC, 0, st>>>(v);
    if (t.exact && t.embed.mode == TAB_QUADRATIC) k_embed<<<nbe, BS_VEC, 0, st>>>(v, t.embed, pe);
    else k_embed_fast<<<nbe, BS_VEC, 0, st>>>(v, t.embed, pe);
    k_ghost_df<<<gblocks, BS_VEC, 0, st>>>(v);
    if (ev) cudaEventRecord(ev[2], st);
    if (t.cache) launch_cache(t, v, 1, pf, st);
    else launch_force_any(t, nbf, st, v, pf);
    if (ev) cudaEventRecord(ev[3], st);
    launches += 5;
  } else {
    if (ev) {
      cudaEventRecord(ev[0], st);
      cudaEventRecord(ev[1], st);
      cudaEventRecord(ev[2], st);
    }
    launch_force_any(t, nbf, st, v, pf);
    if (ev) cudaEventRecord(ev[3], st);
    launches += 1;
  }
  k_fold_force<<<gblocks, BS_VEC, 0, st>>>(v);
  k_finalize_forces<<<1, FIN_BS, 0, st>>>(pe, t.eam ? nbe : 0, pf, nbf, sc);
  launches += 2;
  return launches;
}

}  // namespace imdgpu
