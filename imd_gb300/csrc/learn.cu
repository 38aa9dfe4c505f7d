// learn.cu -- learned starting guess for CG: an equivariant per-pair MLP.
//
// For every directed neighbour pair (i, j) with r_ij < 5.5 A the network
// maps x_ij = [16 Gaussian radial basis functions of r_ij (centres 2.0-5.5 A,
// width 0.25 A), rho_i / 100] through 17 -> 64 -> 64 -> 1 with SiLU to a
// scalar w_ij; the predicted displacement of atom i is
//   dx_i = sum_j w_ij (r_j - r_i) / r_ij,
// which rotates with the crystal (equivariant).  Weights are BF16, products
// accumulate in FP32 on the tensor cores (mma.sync m16n8k16, one 16-pair
// slab per warp, 64 pairs per block); SiLU, the radial basis and the output
// layer are FP32.  The backward kernel recomputes the forward pass of its
// tile and accumulates weight gradients per block in FP32 before one atomic
// add per weight; Adam updates FP32 master weights and refreshes the BF16
// copies.  k_ml_forward_tc is the forward pass on tcgen05 with tensor-memory
// accumulators, opt-in per system.
#include <cuda_bf16.h>

#include "kernels.cuh"

namespace imdgpu {

constexpr int ML_IN = 17;
constexpr int ML_K1 = 32;   // padded input width
constexpr int ML_H = 64;
constexpr int ML_TILE = 64;  // pairs per block
constexpr float ML_RC = 5.5f;

// parameters in one FP32 array: W1[64][32] (inputs >= 17 stay 0), b1[64],
// W2[64][64], b2[64], W3[64], b3
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + ML_H * ML_K1;
constexpr int OFF_W2 = OFF_B1 + ML_H;
constexpr int OFF_B2 = OFF_W2 + ML_H * ML_H;
constexpr int OFF_W3 = OFF_B2 + ML_H;
constexpr int OFF_B3 = OFF_W3 + ML_H;
constexpr int ML_NPARAM = OFF_B3 + 1;

struct MlPair {
  int i;       // atom receiving the displacement
  float dx, dy, dz;  // r_j - r_i
};

// ---------------------------------------------------------------------------
// pair extraction from the half list: both directions of every entry within
// 5.5 A (ghost partners map to their owning atom)
// ---------------------------------------------------------------------------
__global__ void k_ml_pairs(SysView v, MlPair *pairs, int cap, int *count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= v.n) return;
  const double4 pi = v.pos[i];
  const int nn = v.nnb[i];
  for (int k = 0; k < nn; k++) {
    const int j = (int)(v.nbr[(size_t)k * v.ncap + i] & NB_MASK);
    if (!in_bounds(v, j, (long)v.n + v.gcap, CK_PARTNER)) continue;
    const double4 pj = v.pos[j];
    const float dx = (float)(pj.x - pi.x), dy = (float)(pj.y - pi.y), dz = (float)(pj.z - pi.z);
    const float r2 = dx * dx + dy * dy + dz * dz;
    if (r2 >= ML_RC * ML_RC) continue;
    const int jo = (j >= v.n) ? v.gowner[j - v.n] : j;
    if (jo < 0) continue;  // an unused ghost slot (only after a range overflow)
    if (!in_bounds(v, jo, v.n, CK_OWNER)) continue;
    const int at = atomicAdd(count, 2);
    if (at + 1 < cap) {
      pairs[at] = MlPair{i, dx, dy, dz};
      pairs[at + 1] = MlPair{jo, -dx, -dy, -dz};
    }
  }
}

// ---------------------------------------------------------------------------
// tensor-core helpers (BF16 in, FP32 accumulate)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ uint32_t pack2b(__nv_bfloat16 lo, __nv_bfloat16 hi) {
  __nv_bfloat162 v;
  v.x = lo;
  v.y = hi;
  return *reinterpret_cast<const uint32_t *>(&v);
}
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment of rows r0..r0+15, columns k0..k0+15 of a row-major bf16
// matrix with leading dimension ld (transposed read when T)
template <bool T>
__device__ __forceinline__ void load_a(uint32_t (&a)[4], const __nv_bfloat16 *M, int ld, int r0,
                                       int k0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  auto at = [&](int r, int c) { return T ? M[c * ld + r] : M[r * ld + c]; };
  a[0] = pack2b(at(r0 + g, k0 + 2 * t), at(r0 + g, k0 + 2 * t + 1));
  a[1] = pack2b(at(r0 + g + 8, k0 + 2 * t), at(r0 + g + 8, k0 + 2 * t + 1));
  a[2] = pack2b(at(r0 + g, k0 + 2 * t + 8), at(r0 + g, k0 + 2 * t + 9));
  a[3] = pack2b(at(r0 + g + 8, k0 + 2 * t + 8), at(r0 + g + 8, k0 + 2 * t + 9));
}
// B fragment B(k, n), k = k0..k0+15, n = n0..n0+7, element B(k,n) = M[n*ld + k]
// (NT: "weights[out][in]" layout) or M[k*ld + n] (T)
template <bool T>
__device__ __forceinline__ void load_b(uint32_t (&b)[2], const __nv_bfloat16 *M, int ld, int k0,
                                       int n0) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  auto at = [&](int k, int n) { return T ? M[k * ld + n] : M[n * ld + k]; };
  b[0] = pack2b(at(k0 + 2 * t, n0 + g), at(k0 + 2 * t + 1, n0 + g));
  b[1] = pack2b(at(k0 + 2 * t + 8, n0 + g), at(k0 + 2 * t + 9, n0 + g));
}

__device__ __forceinline__ float silu(float z) { return z / (1.0f + __expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.0f / (1.0f + __expf(-z));
  return s * (1.0f + z * (1.0f - s));
}

struct MlSmem {
  __nv_bfloat16 W1[ML_H * ML_K1];   // [out][in]
  __nv_bfloat16 W2[ML_H * ML_H];    // [out][in]
  float b1[ML_H], b2[ML_H], W3[ML_H];
  float b3;
  __nv_bfloat16 X[ML_TILE * ML_K1];  // [pair][in]
  __nv_bfloat16 H1[ML_TILE * ML_H];  // [pair][hidden]
  __nv_bfloat16 D2[ML_TILE * ML_H];  // backward: dz2 [pair][hidden]
  __nv_bfloat16 D1[ML_TILE * ML_H];  // backward: dz1 [pair][hidden]
  float gsc[ML_TILE];                // backward: dL/dw per pair
  float ux[ML_TILE], uy[ML_TILE], uz[ML_TILE];
  int ip[ML_TILE];
};

__device__ void ml_load_weights(MlSmem &S, const __nv_bfloat16 *wb, const float *wf) {
  for (int k = threadIdx.x; k < ML_H * ML_K1; k += blockDim.x) S.W1[k] = wb[OFF_W1 + k];
  for (int k = threadIdx.x; k < ML_H * ML_H; k += blockDim.x) S.W2[k] = wb[OFF_W2 + k];
  for (int k = threadIdx.x; k < ML_H; k += blockDim.x) {
    S.b1[k] = wf[OFF_B1 + k];
    S.b2[k] = wf[OFF_B2 + k];
    S.W3[k] = __bfloat162float(wb[OFF_W3 + k]);
  }
  if (threadIdx.x == 0) S.b3 = wf[OFF_B3];
}

// features of the tile's pairs -> S.X, unit vectors, receiving atoms
__device__ void ml_features(MlSmem &S, const MlPair *pairs, int p0, int np, const double *rho) {
  for (int q = threadIdx.x; q < ML_TILE; q += blockDim.x) {
    const int p = p0 + q;
    float f[ML_K1];
#pragma unroll
    for (int k = 0; k < ML_K1; k++) f[k] = 0.f;
    float ux = 0.f, uy = 0.f, uz = 0.f;
    int i = -1;
    if (p < np) {
      const MlPair P = pairs[p];
      const float r = sqrtf(P.dx * P.dx + P.dy * P.dy + P.dz * P.dz);
      const float ir = 1.0f / r;
      ux = P.dx * ir;
      uy = P.dy * ir;
      uz = P.dz * ir;
      i = P.i;
#pragma unroll
      for (int k = 0; k < 16; k++) {
        const float c = 2.0f + k * (3.5f / 15.0f);
        const float t = (r - c) * (1.0f / 0.25f);
        f[k] = __expf(-0.5f * t * t);
      }
      f[16] = (float)rho[i] * 0.01f;
    }
#pragma unroll
    for (int k = 0; k < ML_K1; k++) S.X[q * ML_K1 + k] = __float2bfloat16(f[k]);
    S.ux[q] = ux;
    S.uy[q] = uy;
    S.uz[q] = uz;
    S.ip[q] = i;
  }
}

// forward of one tile: z1, z2 fragments of this warp's 16 pairs; H1 to smem;
// returns w of the two rows this thread owns (g, g+8) after the quad sum
__device__ void ml_forward_tile(MlSmem &S, float (&z1)[8][4], float (&z2)[8][4], float &w_lo,
                                float &w_hi) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int r0 = warp * 16;
#pragma unroll
  for (int n = 0; n < 8; n++) z1[n][0] = z1[n][1] = z1[n][2] = z1[n][3] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < ML_K1; k0 += 16) {
    uint32_t a[4];
    load_a<false>(a, S.X, ML_K1, r0, k0);
#pragma unroll
    for (int n = 0; n < 8; n++) {
      uint32_t b[2];
      load_b<false>(b, S.W1, ML_K1, k0, n * 8);
      mma16816(z1[n], a, b);
    }
  }
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int c = n * 8 + 2 * t;
    z1[n][0] += S.b1[c];
    z1[n][1] += S.b1[c + 1];
    z1[n][2] += S.b1[c];
    z1[n][3] += S.b1[c + 1];
    S.H1[(r0 + g) * ML_H + c] = __float2bfloat16(silu(z1[n][0]));
    S.H1[(r0 + g) * ML_H + c + 1] = __float2bfloat16(silu(z1[n][1]));
    S.H1[(r0 + g + 8) * ML_H + c] = __float2bfloat16(silu(z1[n][2]));
    S.H1[(r0 + g + 8) * ML_H + c + 1] = __float2bfloat16(silu(z1[n][3]));
  }
  __syncwarp();
#pragma unroll
  for (int n = 0; n < 8; n++) z2[n][0] = z2[n][1] = z2[n][2] = z2[n][3] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < ML_H; k0 += 16) {
    uint32_t a[4];
    load_a<false>(a, S.H1, ML_H, r0, k0);
#pragma unroll
    for (int n = 0; n < 8; n++) {
      uint32_t b[2];
      load_b<false>(b, S.W2, ML_H, k0, n * 8);
      mma16816(z2[n], a, b);
    }
  }
  float lo = 0.f, hi = 0.f;
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int c = n * 8 + 2 * t;
    z2[n][0] += S.b2[c];
    z2[n][1] += S.b2[c + 1];
    z2[n][2] += S.b2[c];
    z2[n][3] += S.b2[c + 1];
    lo += silu(z2[n][0]) * S.W3[c] + silu(z2[n][1]) * S.W3[c + 1];
    hi += silu(z2[n][2]) * S.W3[c] + silu(z2[n][3]) * S.W3[c + 1];
  }
  lo += __shfl_xor_sync(0xffffffffu, lo, 1);
  lo += __shfl_xor_sync(0xffffffffu, lo, 2);
  hi += __shfl_xor_sync(0xffffffffu, hi, 1);
  hi += __shfl_xor_sync(0xffffffffu, hi, 2);
  w_lo = lo + S.b3;
  w_hi = hi + S.b3;
}

// inference / training forward: dx_i += w_ij * unit(r_ij)
__global__ void __launch_bounds__(128) k_ml_forward(const MlPair *pairs, const int *npairs,
                                                    const double *rho, const __nv_bfloat16 *wb,
                                                    const float *wf, float *dxp) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MlSmem &S = *reinterpret_cast<MlSmem *>(smraw);
  ml_load_weights(S, wb, wf);
  const int np = *npairs;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  for (int p0 = blockIdx.x * ML_TILE; p0 < np; p0 += gridDim.x * ML_TILE) {
    __syncthreads();
    ml_features(S, pairs, p0, np, rho);
    __syncthreads();
    float z1[8][4], z2[8][4], wlo, whi;
    ml_forward_tile(S, z1, z2, wlo, whi);
    if (t == 0) {
      const int ra = warp * 16 + g, rb = ra + 8;
      const int ia = S.ip[ra], ib = S.ip[rb];
      if (ia >= 0) {
        atomicAdd(&dxp[3 * ia], wlo * S.ux[ra]);
        atomicAdd(&dxp[3 * ia + 1], wlo * S.uy[ra]);
        atomicAdd(&dxp[3 * ia + 2], wlo * S.uz[ra]);
      }
      if (ib >= 0) {
        atomicAdd(&dxp[3 * ib], whi * S.ux[rb]);
        atomicAdd(&dxp[3 * ib + 1], whi * S.uy[rb]);
        atomicAdd(&dxp[3 * ib + 2], whi * S.uz[rb]);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// The forward pass on the fifth-generation tensor cores (tcgen05); opt-in
// per system (imdgpu_ml_set_tensor_cores), the mma.sync kernel above is the
// default.  One CTA of 128 threads takes 128 pairs per tile:
// - the tile's features (A: 128 x 32) and the weights (B: W1 64 x 32 and
//   W2 64 x 64, [out][in]) sit in shared memory as 8-row x 16-byte core
//   matrices, K-major, without swizzle;
// - one thread issues tcgen05.mma (M 128, N 64, K 16; BF16 in, FP32
//   accumulate) into tensor memory: 128 lanes (one pair each) x 128
//   columns, layer 1 in columns 0-63 and layer 2 in 64-127, and commits to
//   an mbarrier that the CTA waits on (bounded);
// - each warp reads its 32 lanes with tcgen05.ld, one pair per thread;
//   layer 1's epilogue (bias, SiLU, BF16) writes the A operand of layer 2;
// - layer 3 (64 -> 1) and the scatter of w_ij * unit(r_ij) stay on the CUDA
//   cores, one pair per thread, with no shuffles.
// A wait that runs out sets ST_WAIT in the status word; the CTA then stops,
// waits once more (bounded) for its products and frees its tensor memory.
// ---------------------------------------------------------------------------
constexpr int TC_M = 128;                  // pairs per tile = TMEM lanes
constexpr uint32_t TC_COLS = 128;          // TMEM columns of a CTA
constexpr uint32_t TC_WAIT_LIMIT = 1u << 22;
constexpr int TC_SMEM = 56 * 1024;         // at most 4 CTAs (512 TMEM columns) per SM

// byte offset of element (r, k) of an R x K BF16 operand stored as 8 x 8
// core matrices (8 rows of 16 bytes): the K / 8 core matrices of an 8-row
// group side by side (leading byte offset 128 along K), the groups one
// after another (stride byte offset K / 8 * 128)
__device__ __forceinline__ int core_off(int r, int k, int K) {
  return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

struct TcSmem {
  alignas(1024) __nv_bfloat16 X[TC_M * ML_K1];
  alignas(1024) __nv_bfloat16 H1[TC_M * ML_H];
  alignas(1024) __nv_bfloat16 W1[ML_H * ML_K1];
  alignas(1024) __nv_bfloat16 W2[ML_H * ML_H];
  float b1[ML_H], b2[ML_H], W3[ML_H];
  float b3;
  float ux[TC_M], uy[TC_M], uz[TC_M];
  int ip[TC_M];
  alignas(8) unsigned long long mbar;
  uint32_t tmem;
};
static_assert(sizeof(TcSmem) + 1024 <= TC_SMEM, "tcgen05 MLP shared memory");

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units, 14 bits each), descriptor version 1 (bits 46-47),
// base offset 0, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// kind::f16 instruction descriptor: D FP32 (bits 4-5 = 1), A and B BF16
// (bits 7-9 and 10-12 = 1), both K-major (bits 15, 16 = 0), N / 8 from bit
// 17, M / 16 from bit 24
__host__ __device__ constexpr uint32_t tc_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
         ((uint32_t)(M >> 4) << 24);
}
static_assert(tc_idesc(128, 64) == 0x08100490u, "instruction descriptor");

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy writes to shared memory made visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
      : "memory");
}
// 16 consecutive FP32 columns of this thread's lane; the load and its wait
// in one statement, so no use of the registers comes before the wait
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n\ttcgen05.wait::ld.sync.aligned;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr)
      : "memory");
#pragma unroll
  for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}
__device__ __forceinline__ bool tc_mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(mbar), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ bool tc_mbar_wait(uint32_t mbar, uint32_t parity) {
  for (uint32_t it = 0; it < TC_WAIT_LIMIT; it++)
    if (tc_mbar_try(mbar, parity)) return true;
  return false;
}

__global__ void __launch_bounds__(128) k_ml_forward_tc(const MlPair *pairs, const int *npairs,
                                                       const double *rho,
                                                       const __nv_bfloat16 *wb, const float *wf,
                                                       float *dxp, unsigned *status) {
  extern __shared__ __align__(16) unsigned char smraw[];
  TcSmem &S = *reinterpret_cast<TcSmem *>(smraw + ((1024u - (smem_u32(smraw) & 1023u)) & 1023u));
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int e = tid; e < ML_H * ML_K1; e += blockDim.x)
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(S.W1) +
                                       core_off(e / ML_K1, e % ML_K1, ML_K1)) = wb[OFF_W1 + e];
  for (int e = tid; e < ML_H * ML_H; e += blockDim.x)
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(S.W2) +
                                       core_off(e / ML_H, e % ML_H, ML_H)) = wb[OFF_W2 + e];
  for (int k = tid; k < ML_H; k += blockDim.x) {
    S.b1[k] = wf[OFF_B1 + k];
    S.b2[k] = wf[OFF_B2 + k];
    S.W3[k] = __bfloat162float(wb[OFF_W3 + k]);
  }
  const uint32_t mbar = smem_u32(&S.mbar);
  if (tid == 0) {
    S.b3 = wf[OFF_B3];
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(&S.tmem)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.tmem;
  const uint32_t lane_base = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's 32 lanes
  const uint32_t idesc = tc_idesc(TC_M, ML_H);
  const uint32_t xa = smem_u32(S.X), ha = smem_u32(S.H1);
  const uint32_t w1a = smem_u32(S.W1), w2a = smem_u32(S.W2);
  const int np = *npairs;
  uint32_t parity = 0;
  bool failed = false;
  for (int p0 = blockIdx.x * TC_M; p0 < np; p0 += gridDim.x * TC_M) {
    {  // features of pair p0 + tid (row tid of A), as ml_features
      const int p = p0 + tid;
      float f[ML_K1];
#pragma unroll
      for (int k = 0; k < ML_K1; k++) f[k] = 0.f;
      float ux = 0.f, uy = 0.f, uz = 0.f;
      int i = -1;
      if (p < np) {
        const MlPair P = pairs[p];
        const float r = sqrtf(P.dx * P.dx + P.dy * P.dy + P.dz * P.dz);
        const float ir = 1.0f / r;
        ux = P.dx * ir;
        uy = P.dy * ir;
        uz = P.dz * ir;
        i = P.i;
#pragma unroll
        for (int k = 0; k < 16; k++) {
          const float c = 2.0f + k * (3.5f / 15.0f);
          const float t = (r - c) * (1.0f / 0.25f);
          f[k] = __expf(-0.5f * t * t);
        }
        f[16] = (float)rho[i] * 0.01f;
      }
#pragma unroll
      for (int k8 = 0; k8 < ML_K1; k8 += 8) {
        const uint4 q = make_uint4(pack2(f[k8], f[k8 + 1]), pack2(f[k8 + 2], f[k8 + 3]),
                                   pack2(f[k8 + 4], f[k8 + 5]), pack2(f[k8 + 6], f[k8 + 7]));
        *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.X) + core_off(tid, k8, ML_K1)) = q;
      }
      S.ux[tid] = ux;
      S.uy[tid] = uy;
      S.uz[tid] = uz;
      S.ip[tid] = i;
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {  // layer 1: D[0, 64) = X W1^T over K = 32
#pragma unroll
      for (int k = 0; k < ML_K1 / 16; k++)
        tc_mma(tmem, tc_sdesc(xa + 256 * k, 128, ML_K1 / 8 * 128),
               tc_sdesc(w1a + 256 * k, 128, ML_K1 / 8 * 128), idesc, k > 0);
      tc_commit(mbar);
    }
    failed = !tc_mbar_wait(mbar, parity);
    parity ^= 1u;
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    tc_fence_after();
#pragma unroll
    for (int c0 = 0; c0 < ML_H; c0 += 16) {  // bias, SiLU, BF16 -> row tid of H1
      float d[16];
      tc_ld16(lane_base + c0, d);
#pragma unroll
      for (int h = 0; h < 16; h += 8) {
        float a[8];
#pragma unroll
        for (int q = 0; q < 8; q++) a[q] = silu(d[h + q] + S.b1[c0 + h + q]);
        const uint4 q = make_uint4(pack2(a[0], a[1]), pack2(a[2], a[3]), pack2(a[4], a[5]),
                                   pack2(a[6], a[7]));
        *reinterpret_cast<uint4 *>(reinterpret_cast<char *>(S.H1) + core_off(tid, c0 + h, ML_H)) =
            q;
      }
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (tid == 0) {  // layer 2: D[64, 128) = H1 W2^T over K = 64
#pragma unroll
      for (int k = 0; k < ML_H / 16; k++)
        tc_mma(tmem + ML_H, tc_sdesc(ha + 256 * k, 128, ML_H / 8 * 128),
               tc_sdesc(w2a + 256 * k, 128, ML_H / 8 * 128), idesc, k > 0);
      tc_commit(mbar);
    }
    failed = !tc_mbar_wait(mbar, parity);
    parity ^= 1u;
    if (__syncthreads_or(failed)) {
      failed = true;
      break;
    }
    tc_fence_after();
    float w = S.b3;  // layer 3 on this thread's pair
#pragma unroll
    for (int c0 = 0; c0 < ML_H; c0 += 16) {
      float d[16];
      tc_ld16(lane_base + ML_H + c0, d);
#pragma unroll
      for (int q = 0; q < 16; q++) w += silu(d[q] + S.b2[c0 + q]) * S.W3[c0 + q];
    }
    const int i = S.ip[tid];
    if (i >= 0) {
      atomicAdd(&dxp[3 * i], w * S.ux[tid]);
      atomicAdd(&dxp[3 * i + 1], w * S.uy[tid]);
      atomicAdd(&dxp[3 * i + 2], w * S.uz[tid]);
    }
  }
  if (failed) {  // the products of the last commit, once more before the memory goes
    if (tid == 0) atomicOr(status, ST_WAIT);
    tc_mbar_wait(mbar, parity ^ 1u);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TC_COLS)
                 : "memory");
  }
}

// loss = sum_i |dx_i - t_i|^2 / N; writes dL/d(dx_i) and the block sums of
// the loss
__global__ void k_ml_loss(int n, const float *dxp, const float *target, const float *wt,
                          float inv_n, float *dldx, double *loss) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double l = 0.0;
  if (i < n) {
    const float w = wt ? wt[i] : 1.0f;   // per-atom loss weight (1: the plain mean)
#pragma unroll
    for (int c = 0; c < 3; c++) {
      const float e = dxp[3 * i + c] - target[3 * i + c];
      dldx[3 * i + c] = 2.0f * e * inv_n * w;
      l += (double)e * e * inv_n * w;
    }
  }
  l = warp_sum(l);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
}

// backward: gradients of the loss with respect to all parameters
__global__ void __launch_bounds__(128) k_ml_backward(const MlPair *pairs, const int *npairs,
                                                     const double *rho, const __nv_bfloat16 *wb,
                                                     const float *wf, const float *dldx,
                                                     float *grad) {
  extern __shared__ __align__(16) unsigned char smraw[];
  MlSmem &S = *reinterpret_cast<MlSmem *>(smraw);
  __shared__ float gW3[ML_H], gb2[ML_H], gb1[ML_H];
  __shared__ float gb3;
  ml_load_weights(S, wb, wf);
  for (int k = threadIdx.x; k < ML_H; k += blockDim.x) gW3[k] = gb2[k] = gb1[k] = 0.f;
  if (threadIdx.x == 0) gb3 = 0.f;
  const int np = *npairs;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int r0 = warp * 16;
  // per-warp slices of the weight-gradient GEMMs, accumulated over tiles:
  // dW2 rows (outputs) r0..r0+15 x 64 inputs, dW1 rows r0..r0+15 x 32 inputs
  float gW2[8][4], gW1[4][4];
#pragma unroll
  for (int n = 0; n < 8; n++) gW2[n][0] = gW2[n][1] = gW2[n][2] = gW2[n][3] = 0.f;
#pragma unroll
  for (int n = 0; n < 4; n++) gW1[n][0] = gW1[n][1] = gW1[n][2] = gW1[n][3] = 0.f;
  for (int p0 = blockIdx.x * ML_TILE; p0 < np; p0 += gridDim.x * ML_TILE) {
    __syncthreads();
    ml_features(S, pairs, p0, np, rho);
    __syncthreads();
    float z1[8][4], z2[8][4], wlo, whi;
    ml_forward_tile(S, z1, z2, wlo, whi);
    (void)wlo;
    (void)whi;
    // dL/dw per pair (this warp's rows)
    if (t == 0) {
      for (int h = 0; h < 2; h++) {
        const int r = r0 + g + 8 * h;
        const int i = S.ip[r];
        S.gsc[r] = (i >= 0) ? dldx[3 * i] * S.ux[r] + dldx[3 * i + 1] * S.uy[r] +
                                  dldx[3 * i + 2] * S.uz[r]
                            : 0.f;
      }
    }
    __syncwarp();
    const float ga = S.gsc[r0 + g], gbv = S.gsc[r0 + g + 8];
    // output layer and dz2 = g * W3 * silu'(z2)
    float p3[8][2];
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int c = n * 8 + 2 * t;
      const float h0 = silu(z2[n][0]), h1v = silu(z2[n][1]), h2v = silu(z2[n][2]),
                  h3 = silu(z2[n][3]);
      p3[n][0] = ga * h0 + gbv * h2v;  // dW3[c]
      p3[n][1] = ga * h1v + gbv * h3;  // dW3[c+1]
      const float d0 = ga * S.W3[c] * dsilu(z2[n][0]);
      const float d1 = ga * S.W3[c + 1] * dsilu(z2[n][1]);
      const float d2 = gbv * S.W3[c] * dsilu(z2[n][2]);
      const float d3 = gbv * S.W3[c + 1] * dsilu(z2[n][3]);
      S.D2[(r0 + g) * ML_H + c] = __float2bfloat16(d0);
      S.D2[(r0 + g) * ML_H + c + 1] = __float2bfloat16(d1);
      S.D2[(r0 + g + 8) * ML_H + c] = __float2bfloat16(d2);
      S.D2[(r0 + g + 8) * ML_H + c + 1] = __float2bfloat16(d3);
      z2[n][0] = d0;
      z2[n][1] = d1;
      z2[n][2] = d2;
      z2[n][3] = d3;
    }
    // column sums over the warp's 16 rows: reduce over g (lane bits 2..4)
#pragma unroll
    for (int n = 0; n < 8; n++) {
      float s0 = p3[n][0], s1 = p3[n][1];
      float q0 = z2[n][0] + z2[n][2], q1 = z2[n][1] + z2[n][3];
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
      }
      if (g == 0) {
        const int c = n * 8 + 2 * t;
        atomicAdd(&gW3[c], s0);
        atomicAdd(&gW3[c + 1], s1);
        atomicAdd(&gb2[c], q0);
        atomicAdd(&gb2[c + 1], q1);
      }
    }
    if (lane == 0) {
      float s = 0.f;
      for (int r = 0; r < 16; r++) s += S.gsc[r0 + r];
      atomicAdd(&gb3, s);
    }
    __syncthreads();  // D2 complete for all rows
    // dh1 = dz2 . W2  (rows = this warp's pairs, K = 64 outputs, N = 64 inputs)
    float dh[8][4];
#pragma unroll
    for (int n = 0; n < 8; n++) dh[n][0] = dh[n][1] = dh[n][2] = dh[n][3] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < ML_H; k0 += 16) {
      uint32_t a[4];
      load_a<false>(a, S.D2, ML_H, r0, k0);
#pragma unroll
      for (int n = 0; n < 8; n++) {
        uint32_t b[2];
        load_b<true>(b, S.W2, ML_H, k0, n * 8);  // B(k=out, n=in) = W2[out][in]
        mma16816(dh[n], a, b);
      }
    }
    // dz1 = dh1 * silu'(z1)
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const int c = n * 8 + 2 * t;
      const float d0 = dh[n][0] * dsilu(z1[n][0]), d1 = dh[n][1] * dsilu(z1[n][1]);
      const float d2 = dh[n][2] * dsilu(z1[n][2]), d3 = dh[n][3] * dsilu(z1[n][3]);
      S.D1[(r0 + g) * ML_H + c] = __float2bfloat16(d0);
      S.D1[(r0 + g) * ML_H + c + 1] = __float2bfloat16(d1);
      S.D1[(r0 + g + 8) * ML_H + c] = __float2bfloat16(d2);
      S.D1[(r0 + g + 8) * ML_H + c + 1] = __float2bfloat16(d3);
      float q0 = d0 + d2, q1 = d1 + d3;
#pragma unroll
      for (int o = 4; o < 32; o <<= 1) {
        q0 += __shfl_xor_sync(0xffffffffu, q0, o);
        q1 += __shfl_xor_sync(0xffffffffu, q1, o);
      }
      if (g == 0) {
        atomicAdd(&gb1[c], q0);
        atomicAdd(&gb1[c + 1], q1);
      }
    }
    __syncthreads();  // D1, H1 complete
    // dW2[out][in] += sum_p D2[p][out] H1[p][in]: this warp owns outputs r0..r0+15
#pragma unroll
    for (int k0 = 0; k0 < ML_TILE; k0 += 16) {
      uint32_t a[4];
      load_a<true>(a, S.D2, ML_H, r0, k0);  // A(out, p) = D2[p][out]
#pragma unroll
      for (int n = 0; n < 8; n++) {
        uint32_t b[2];
        load_b<true>(b, S.H1, ML_H, k0, n * 8);  // B(p, in) = H1[p][in]
        mma16816(gW2[n], a, b);
      }
    }
    // dW1[out][k] += sum_p D1[p][out] X[p][k]
#pragma unroll
    for (int k0 = 0; k0 < ML_TILE; k0 += 16) {
      uint32_t a[4];
      load_a<true>(a, S.D1, ML_H, r0, k0);
#pragma unroll
      for (int n = 0; n < 4; n++) {
        uint32_t b[2];
        load_b<true>(b, S.X, ML_K1, k0, n * 8);
        mma16816(gW1[n], a, b);
      }
    }
  }
  __syncthreads();
  // flush: one atomic per parameter and block
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const int c = n * 8 + 2 * t;
    atomicAdd(&grad[OFF_W2 + (r0 + g) * ML_H + c], gW2[n][0]);
    atomicAdd(&grad[OFF_W2 + (r0 + g) * ML_H + c + 1], gW2[n][1]);
    atomicAdd(&grad[OFF_W2 + (r0 + g + 8) * ML_H + c], gW2[n][2]);
    atomicAdd(&grad[OFF_W2 + (r0 + g + 8) * ML_H + c + 1], gW2[n][3]);
  }
#pragma unroll
  for (int n = 0; n < 4; n++) {
    const int c = n * 8 + 2 * t;
    if (c < ML_IN) {
      atomicAdd(&grad[OFF_W1 + (r0 + g) * ML_K1 + c], gW1[n][0]);
      atomicAdd(&grad[OFF_W1 + (r0 + g + 8) * ML_K1 + c], gW1[n][2]);
    }
    if (c + 1 < ML_IN) {
      atomicAdd(&grad[OFF_W1 + (r0 + g) * ML_K1 + c + 1], gW1[n][1]);
      atomicAdd(&grad[OFF_W1 + (r0 + g + 8) * ML_K1 + c + 1], gW1[n][3]);
    }
  }
  for (int k = threadIdx.x; k < ML_H; k += blockDim.x) {
    atomicAdd(&grad[OFF_W3 + k], gW3[k]);
    atomicAdd(&grad[OFF_B2 + k], gb2[k]);
    atomicAdd(&grad[OFF_B1 + k], gb1[k]);
  }
  if (threadIdx.x == 0) atomicAdd(&grad[OFF_B3], gb3);
}

// Adam on the FP32 master weights; refresh the BF16 copies
__global__ void k_ml_adam(float *w, __nv_bfloat16 *wb, const float *grad, float *m, float *vv,
                          int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = grad[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * vv[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  vv[k] = vk;
  float wk = w[k] - lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  // the padded inputs of W1 stay exactly zero
  if (k < OFF_B1 && (k % ML_K1) >= ML_IN) wk = 0.f;
  w[k] = wk;
  wb[k] = __float2bfloat16(wk);
}

__global__ void k_ml_to_bf16(const float *w, __nv_bfloat16 *wb, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) wb[k] = __float2bfloat16(w[k]);
}

size_t ml_smem_bytes() { return sizeof(MlSmem); }
int ml_nparam() { return ML_NPARAM; }

void launch_ml_pairs(const SysView &v, MlPair *pairs, int cap, int *count, cudaStream_t st) {
  k_ml_pairs<<<(v.n + 127) / 128, 128, 0, st>>>(v, pairs, cap, count);
}
void launch_ml_forward(const MlPair *pairs, const int *np, const double *rho,
                       const __nv_bfloat16 *wb, const float *wf, float *dxp, int blocks,
                       cudaStream_t st) {
  k_ml_forward<<<blocks, 128, sizeof(MlSmem), st>>>(pairs, np, rho, wb, wf, dxp);
}
void launch_ml_forward_tc(const MlPair *pairs, const int *np, const double *rho,
                          const __nv_bfloat16 *wb, const float *wf, float *dxp, unsigned *status,
                          int blocks, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_ml_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM);
    attr = true;
  }
  k_ml_forward_tc<<<blocks, 128, TC_SMEM, st>>>(pairs, np, rho, wb, wf, dxp, status);
}
void launch_ml_loss(int n, const float *dxp, const float *target, const float *wt, float *dldx,
                    double *loss, cudaStream_t st) {
  k_ml_loss<<<(n + 255) / 256, 256, 0, st>>>(n, dxp, target, wt, 1.0f / n, dldx, loss);
}
void launch_ml_backward(const MlPair *pairs, const int *np, const double *rho,
                        const __nv_bfloat16 *wb, const float *wf, const float *dldx,
                        float *grad, int blocks, cudaStream_t st) {
  k_ml_backward<<<blocks, 128, sizeof(MlSmem), st>>>(pairs, np, rho, wb, wf, dldx, grad);
}
void launch_ml_adam(float *w, __nv_bfloat16 *wb, const float *grad, float *m, float *vv, int n,
                    float lr, int step, cudaStream_t st) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_ml_adam<<<(n + 255) / 256, 256, 0, st>>>(w, wb, grad, m, vv, n, lr, b1, b2, 1e-8f, c1, c2);
}
void launch_ml_to_bf16(const float *w, __nv_bfloat16 *wb, int n, cudaStream_t st) {
  k_ml_to_bf16<<<(n + 255) / 256, 256, 0, st>>>(w, wb, n);
}

}  // namespace imdgpu
