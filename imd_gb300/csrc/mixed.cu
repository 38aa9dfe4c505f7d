// mixed.cu -- FP32-force / FP64-accumulate path (IMDGPU_MIXED).
//
// Same physics as forces.cu (calc_forces PAIR + EAM2, src/imd_forces_nbl.c:
// 423-1323) with the pair and EAM arithmetic in FP32:
//   * positions stay FP64; every step each real and ghost atom is split into
//     an FP32 high part and an FP32 residual (x = hi + lo to ~1e-14), so
//     d = (hi_j - hi_i) + (lo_j - lo_i) is accurate to the last FP32 bit of d
//     itself: the coordinates an FP32 pair sees are relative to the atom,
//     never absolute box coordinates;
//   * the list is the split list of k_rb_build_half: in every row the
//     balanced half list (IMD's pair set, every pair once) comes first and
//     the partners the other atom keeps follow from the back of the row, so
//     one list serves as a half list and as a full list;
//   * the density pass walks the half list: each pair's FP32 arithmetic and
//     partner gather happen once, the partner's rho goes in with an FP64
//     atomic and ghost rho folds into its owner;
//   * the force pass walks the full row: each atom owns its sums, with no
//     atomics and no ghost fold;
//   * per-atom sums of rho, force, energy and virial are kept as error-free
//     (TwoSum) pairs of FP32 values and converted to FP64 once per atom; the
//     block and device reductions are FP64;
//   * the embedding function and the integrator stay FP64.
#include <algorithm>

#include "kernels.cuh"

namespace imdgpu {

// error-free accumulation: s + c carries the exact running sum to ~2^-48
struct Acc {
  float s, c;
  __device__ __forceinline__ Acc() : s(0.f), c(0.f) {}
  __device__ __forceinline__ void add(float x) {
    const float t = s + x;
    const float z = t - s;
    c += (s - (t - z)) + (x - z);
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__global__ void k_split(SysView v, SplitPos *sp) {
  const int ne = v.n + v.counters[0];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x)
    sp[e] = split_pos(v.pos[e]);
}

__device__ __forceinline__ int tab_index_f(const DevTable &t, int col, float r2, float &chi) {
  float r2a = fmaf(fminf(r2, t.fend[col]), t.finv[col], -t.fbegin[col] * t.finv[col]);
  r2a = fmaxf(r2a, 0.0f);
  int k = __float2int_rz(r2a);
  if (t.mode == TAB_FOURPOINT) k = max(k, 1);
  chi = r2a - (float)k;
  return k;
}
__device__ __forceinline__ float polyf_v(const DevTable &t, int col, int k, float chi) {
  const float4 c = __ldg(&t.cvf[row_of(t, col, k)]);
  return fmaf(chi, fmaf(chi, fmaf(chi, c.w, c.z), c.y), c.x);
}
__device__ __forceinline__ float polyf_g(const DevTable &t, int col, int k, float chi) {
  const float4 g = __ldg(&t.cgf[row_of(t, col, k)]);
  return fmaf(chi, fmaf(chi, g.z, g.y), g.x);
}

// loop 1's EAM branch over the half list (src/imd_forces_nbl.c:586-611):
// rho_{it,jt}(r) to atom i, rho_{jt,it}(r) to atom j
template <bool NT1, int LPA>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_density_mixed(SysView v, DevTable rho,
                                                            const SplitPos *sp) {
  // LPA lanes per atom (the autotuner's tile): lane q takes the entries
  // q, q + LPA, ... and the lanes' FP64 sums meet in a shuffle tree
  const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(gid / LPA), q = (int)(gid % LPA);
  if (i >= v.n || atom_idle(v, i)) return;  // the whole lane group alike
  const SplitPos a = sp[i];
  const int it = NT1 ? 0 : __float_as_int(a.hi.w), nt = v.ntypes;
  const int nn = v.nnb[i];
  Acc r;
  bool shortf = false;
  const uint32_t *__restrict__ nb = v.nbr + i;
#pragma unroll 4
  for (int k = q; k < nn; k += LPA) {
    const int j = (int)(__ldg(nb + (size_t)k * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const SplitPos b = ldsp(&sp[j]);
    const float dx = (b.hi.x - a.hi.x) + (b.lo.x - a.lo.x);
    const float dy = (b.hi.y - a.hi.y) + (b.lo.y - a.lo.y);
    const float dz = (b.hi.z - a.hi.z) + (b.lo.z - a.lo.z);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const int jt = NT1 ? 0 : __float_as_int(b.hi.w);
    const int col = NT1 ? 0 : it * nt + jt;
    float rho_h = 0.f;
    if (r2 < rho.fend[col]) {
      float chi;
      const int kk = tab_index_f(rho, col, r2, chi);
      rho_h = polyf_v(rho, col, kk, chi);
      r.add(rho_h);
      shortf |= r2 < rho.fbegin[col];
    }
    if (NT1 || it == jt) {
      if (r2 < rho.fend[col]) atomicAdd(&v.rho[j], (double)rho_h);
    } else {
      const int col2 = jt * nt + it;
      if (r2 < rho.fend[col2]) {
        float chi;
        const int kk = tab_index_f(rho, col2, r2, chi);
        atomicAdd(&v.rho[j], (double)polyf_v(rho, col2, kk, chi));
        shortf |= r2 < rho.fbegin[col2];
      }
    }
  }
  double ri = r.value();
  if (LPA > 1) {
    const unsigned g = ((1u << LPA) - 1u) << ((threadIdx.x & 31) & ~(LPA - 1));
#pragma unroll
    for (int o = 1; o < LPA; o <<= 1) ri += __shfl_xor_sync(g, ri, o);
  }
  if (q == 0) atomicAdd(&v.rho[i], ri);
  if (shortf) flag_short(v, i);
}

// embedding in FP64 (per atom), F' also as FP32 for the pair kernel
__global__ void __launch_bounds__(BS_VEC) k_embed_mixed(SysView v, DevTable emb, SplitPos *sp,
                                                        double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double e[1] = {0.0};
  if (i < v.n && !atom_idle(v, i)) {
    const int t = (int)v.pos[i].w;
    double chi;
    const int k = tab_index_fast(emb, t, v.rho[i], chi);
    const double pot = poly_v<true>(cv_load(emb, t, k), chi);
    const double df = poly_g<true>(cg_load(emb, t, k), chi);
    v.df[i] = df;
    sp[i].lo.w = (float)df;  // F' in FP32 travels with the position split
    v.frc[i].w = pot;
    e[0] = pot;
  }
  block_sum_store<1, BS_VEC>(e, partial);
}

__global__ void k_ghost_dff(SysView v, SplitPos *sp) {
  const int ng = v.counters[0];
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x) {
    const int o = v.gowner[g];
    if (o >= 0 && in_bounds(v, o, v.n, CK_OWNER)) sp[v.n + g].lo.w = sp[o].lo.w;
  }
}

// where the fused rows are read from
enum RowSrc { ROWS_NONE = 0, ROWS_GLOBAL = 1, ROWS_SHARED = 2 };

// forces over the full row of atom i (the half list at the front, the other
// partners at the back): each directed pair adds d*grad to atom i and half
// of the pair energy and virial
template <bool NT1, bool EAM, int SRC>
__device__ __forceinline__ void force_row_mixed(const SysView &v, const DevTable &pair,
                                                const DevTable &rho, const float4 *rows,
                                                const SplitPos *__restrict__ sp, int i,
                                                double (&acc)[2]) {
  const SplitPos a = sp[i];
  const int it = NT1 ? 0 : __float_as_int(a.hi.w), nt = v.ntypes;
  const int n1 = v.nnb[i], n2 = v.nnb2[i];
  const float dfi = EAM ? a.lo.w : 0.f;
  Acc fx, fy, fz, ee, vir;
  bool shortf = false;
  const uint32_t *__restrict__ nb = v.nbr + i;
  const int nn = n1 + n2, back = v.nbcap - n1 - n2;  // row k >= n1 lives at k + back
#pragma unroll 4
  for (int k = 0; k < nn; k++) {
    const int row = k < n1 ? k : k + back;
    const int j = (int)(__ldg(nb + (size_t)row * v.ncap) & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const SplitPos b = ldsp(&sp[j]);
    const float dx = (b.hi.x - a.hi.x) + (b.lo.x - a.lo.x);
    const float dy = (b.hi.y - a.hi.y) + (b.lo.y - a.lo.y);
    const float dz = (b.hi.z - a.hi.z) + (b.lo.z - a.lo.z);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const int jt = NT1 ? 0 : __float_as_int(b.hi.w);
    const int col = NT1 ? 0 : it * nt + jt;
    float grad = 0.f;
    bool have = false;
    if (SRC != ROWS_NONE) {
      // one species, quadratic pair and density tables on one grid: one
      // index and one 32-byte row serve the three lookups below (the
      // cubic coefficients of a quadratic table are zero and left out)
      const bool inp = r2 <= pair.fend[0], inr = r2 < rho.fend[0];
      if (inp || inr) {
        float chi;
        const int kk = (int)row_of(pair, 0, tab_index_f(pair, 0, r2, chi));
        float4 f0, f1;
        if (SRC == ROWS_SHARED) {
          f0 = rows[2 * kk];
          f1 = rows[2 * kk + 1];
        } else {
          f0 = __ldg(&rows[2 * kk]);
          f1 = __ldg(&rows[2 * kk + 1]);
        }
        if (inp) {
          ee.add(0.5f * fmaf(chi, fmaf(chi, f0.z, f0.y), f0.x));
          grad = fmaf(chi, f1.x, f0.w);
          shortf |= r2 < pair.fbegin[0];
        }
        if (inr) {
          const float ris = fmaf(chi, f1.z, f1.y);
          grad += 0.5f * (dfi * ris + b.lo.w * ris);
        }
        have = true;
      }
    } else if (r2 <= pair.fend[col]) {
      float chi;
      const int kk = tab_index_f(pair, col, r2, chi);
      ee.add(0.5f * polyf_v(pair, col, kk, chi));
      grad = polyf_g(pair, col, kk, chi);
      shortf |= r2 < pair.fbegin[col];
      have = true;
    }
    if (EAM && SRC == ROWS_NONE) {
      const int col1 = NT1 ? 0 : jt * nt + it, col2 = col;
      if (r2 < rho.fend[col1] || r2 < rho.fend[col2]) {
        float chi;
        const int kk = tab_index_f(rho, col1, r2, chi);
        const float ris = polyf_g(rho, col1, kk, chi);
        float rjs = ris;
        if (!NT1 && col1 != col2) {
          const int k2 = tab_index_f(rho, col2, r2, chi);
          rjs = polyf_g(rho, col2, k2, chi);
        }
        const float dfj = b.lo.w;
        grad += 0.5f * (dfi * rjs + dfj * ris);
        have = true;
      }
    }
    if (have) {
      fx.add(dx * grad);
      fy.add(dy * grad);
      fz.add(dz * grad);
      vir.add(-0.5f * r2 * grad);
    }
  }
  const double e = ee.value();
  double4 f = v.frc[i];  // .w holds the embedding energy
  f.x = fx.value();
  f.y = fy.value();
  f.z = fz.value();
  f.w += e;
  v.frc[i] = f;
  acc[0] += e;
  acc[1] += vir.value();
  if (shortf) flag_short(v, i);
}

template <bool NT1, bool EAM, bool FUSED>
__global__ void __launch_bounds__(BS_FORCE_MAX) k_force_mixed(SysView v, DevTable pair,
                                                          DevTable rho, const float4 *fused,
                                                          const SplitPos *sp,
                                                          double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double acc[2] = {0.0, 0.0};
  if (i < v.n && !atom_idle(v, i))
    force_row_mixed<NT1, EAM, FUSED ? ROWS_GLOBAL : ROWS_NONE>(v, pair, rho, fused, sp, i, acc);
  block_sum_store_dyn<2, BS_FORCE_MAX>(acc, partial);
}

// ---------------------------------------------------------------------------
// fused rows staged in shared memory
//
// One thread of each block issues bulk asynchronous copies (cp.async.bulk,
// the TMA's untiled form) of the fused rows into dynamic shared memory; they
// complete on an mbarrier that every thread waits on.  The blocks are
// resident for the whole pass (STAGE_BLOCKS per SM) and take atoms
// blockIdx.x * STAGE_BS + t, then every gridDim.x * STAGE_BS further, so the
// rows are copied once per block rather than once per 128 atoms.
constexpr int STAGE_BS = 384;
constexpr unsigned STAGE_CHUNK = 16384;     // bytes per bulk copy
constexpr int STAGE_WAIT_LIMIT = 1 << 20;   // try_wait rounds before giving up

__device__ __forceinline__ bool mbar_try_wait(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (int it = 0; it < STAGE_WAIT_LIMIT; it++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// copies `bytes` (a multiple of 16; src 16-byte aligned) into dst; false in
// every thread if the copy did not complete (ST_WAIT is then set)
__device__ bool stage_rows(float4 *dst, const float4 *src, unsigned bytes,
                           unsigned long long *bar, unsigned *status) {
  const unsigned b = (unsigned)__cvta_generic_to_shared(bar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes)
                 : "memory");
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    unsigned long long g;
    asm("cvta.to.global.u64 %0, %1;" : "=l"(g) : "l"(src));
    for (unsigned o = 0; o < bytes; o += STAGE_CHUNK) {
      const unsigned sz = min(STAGE_CHUNK, bytes - o);
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
          "[%3];" ::"r"(d + o),
          "l"(g + o), "r"(sz), "r"(b)
          : "memory");
    }
  }
  bool ok = mbar_wait(b, 0);
  if (!ok) {
    atomicOr(status, ST_WAIT);
    mbar_wait(b, 0);  // the copies may still land: give them a second bound
  }
  return __syncthreads_and(ok) != 0;
}

__global__ void __launch_bounds__(STAGE_BS) k_force_mixed_staged(SysView v, DevTable pair,
                                                                DevTable rho,
                                                                const float4 *fused,
                                                                unsigned fused_bytes,
                                                                const SplitPos *sp,
                                                                double *partial) {
  extern __shared__ __align__(16) float4 srows[];
  __shared__ __align__(8) unsigned long long bar;
  double acc[2] = {0.0, 0.0};
  if (stage_rows(srows, fused, fused_bytes, &bar, v.status))
    for (int i = blockIdx.x * STAGE_BS + threadIdx.x; i < v.n; i += gridDim.x * STAGE_BS)
      if (!atom_idle(v, i))
        force_row_mixed<true, true, ROWS_SHARED>(v, pair, rho, srows, sp, i, acc);
  block_sum_store_dyn<2, STAGE_BS>(acc, partial);
}

__global__ void k_finalize_mixed(const double *pe, int ne, const double *pf, int nf,
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

static inline int nblk(long n, int bs) { return (int)((n + bs - 1) / bs); }

// resident blocks of the staged force pass for `bytes` of fused rows on the
// current device; 0 where fewer than two blocks fit on an SM
int mixed_staged_grid(unsigned bytes) {
  int d = 0, nsm = 0, optin = 0, per_sm = 0;
  if (cudaGetDevice(&d) != cudaSuccess) return 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, d);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, d);
  if (bytes == 0 || bytes % 16 || (long)bytes + 64 > optin) return 0;
  // the attribute only grows, so the rows of every live system still fit
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, k_force_mixed_staged) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  if (cudaFuncSetAttribute(k_force_mixed_staged, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           std::max((int)bytes, fa.maxDynamicSharedSizeBytes)) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_force_mixed_staged, STAGE_BS,
                                                    bytes) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm >= 2 ? nsm * per_sm : 0;
}

int mixed_force_blocks(const ForceTabs &t, int n) {
  if (t.fused && t.stage_grid > 0 && t.nt1 && t.eam)
    return std::min(t.stage_grid, std::max(1, nblk(n, STAGE_BS)));
  return nblk(n, t.bs);
}

template <bool NT1, bool EAM>
static void launch_force_mixed2(const ForceTabs &t, int nbf, cudaStream_t st, const SysView &v,
                                const SplitPos *sp, double *pf) {
  if constexpr (NT1 && EAM) {
    if (t.fused) {
      if (t.stage_grid > 0)
        k_force_mixed_staged<<<nbf, STAGE_BS, t.fused_bytes, st>>>(
            v, t.pair, t.rho, t.fused, t.fused_bytes, sp, pf);
      else
        k_force_mixed<true, true, true><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, t.fused, sp, pf);
      return;
    }
  }
  k_force_mixed<NT1, EAM, false><<<nbf, t.bs, 0, st>>>(v, t.pair, t.rho, nullptr, sp, pf);
}

int launch_forces_mixed(const SysView &v, const ForceTabs &t, DevScalars *sc, cudaStream_t st,
                        cudaEvent_t *ev) {
  const int gblocks = std::max(1, nblk(v.gcap, BS_VEC));
  const size_t ext = (size_t)v.ncap + v.gcap;
  SplitPos *sp = reinterpret_cast<SplitPos *>(v.xl);
  cudaMemsetAsync(v.frc, 0, ext * sizeof(double4), st);
  k_ghost_pos_launch(v, gblocks, st);
  k_split<<<nblk(ext, BS_VEC), BS_VEC, 0, st>>>(v, sp);
  const int nbf = mixed_force_blocks(t, v.n), nbe = nblk(v.n, BS_VEC), nbr = nblk(v.n, t.bs_rho);
  double *pe = v.partial, *pf = v.partial + nbe;
  int launches = 4;
  if (t.eam) {
    cudaMemsetAsync(v.rho, 0, ext * sizeof(double), st);
    if (ev) cudaEventRecord(ev[0], st);
    const int lpa = t.mixed_lpa;
    const int nbl = nblk((long)v.n * lpa, t.bs_rho);
    if (t.nt1 && lpa == 4) k_density_mixed<true, 4><<<nbl, t.bs_rho, 0, st>>>(v, t.rho, sp);
    else if (t.nt1 && lpa == 2) k_density_mixed<true, 2><<<nbl, t.bs_rho, 0, st>>>(v, t.rho, sp);
    else if (t.nt1) k_density_mixed<true, 1><<<nbr, t.bs_rho, 0, st>>>(v, t.rho, sp);
    else k_density_mixed<false, 1><<<nbr, t.bs_rho, 0, st>>>(v, t.rho, sp);
    if (ev) cudaEventRecord(ev[1], st);
    fold_rho_launch(v, gblocks, st);
    k_embed_mixed<<<nbe, BS_VEC, 0, st>>>(v, t.embed, sp, pe);
    k_ghost_dff<<<gblocks, BS_VEC, 0, st>>>(v, sp);
    if (ev) cudaEventRecord(ev[2], st);
    if (t.nt1) launch_force_mixed2<true, true>(t, nbf, st, v, sp, pf);
    else launch_force_mixed2<false, true>(t, nbf, st, v, sp, pf);
    if (ev) cudaEventRecord(ev[3], st);
    launches += 5;
  } else {
    if (ev) {
      cudaEventRecord(ev[0], st);
      cudaEventRecord(ev[1], st);
      cudaEventRecord(ev[2], st);
    }
    if (t.nt1) launch_force_mixed2<true, false>(t, nbf, st, v, sp, pf);
    else launch_force_mixed2<false, false>(t, nbf, st, v, sp, pf);
    if (ev) cudaEventRecord(ev[3], st);
    launches += 1;
  }
  k_finalize_mixed<<<1, FIN_BS, 0, st>>>(pe, t.eam ? nbe : 0, pf, nbf, sc);
  return launches + 1;
}

}  // namespace imdgpu
