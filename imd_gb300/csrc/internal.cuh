// internal.cuh -- device data layout and helpers shared by the kernels of
// libimdgpu (sm_103a).
//
// Layout in HBM (one system, N atoms, G ghost atoms):
//   * atoms are sorted by cell at every list build; cells are visited in
//     Morton order, atoms inside a cell by their number (NUMMER), so the
//     layout is a pure function of the positions;
//   * "ext" arrays hold the N real atoms followed by the G buffer-cell
//     copies (ghosts) of IMD's serial build (src/imd_comm_force_3d.c:247);
//   * pos  double4 (x, y, z, type)    -- gathered per pair: one 32 B sector
//     mom  double4 (px, py, pz, mass)
//     frc  double4 (fx, fy, fz, epot) -- scattered by atomics per pair
//   * the half neighbour list is column-major ELL: entry k of atom i at
//     nbr[k * ncap_atoms + i], so consecutive threads read consecutive words.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace imdgpu {

constexpr int MAXT = 4;              // atom types
constexpr int MAXCOL = MAXT * MAXT;  // columns of pair / rho tables
constexpr int CELLCAP = 256;         // atoms per cell supported by the builder
constexpr int NB_SHIFT = 27;         // list entry: ext index (27 bits) | half-shell slot << 27
constexpr uint32_t NB_MASK = (1u << NB_SHIFT) - 1u;

// status bits (device status word)
constexpr unsigned ST_SHORT = 1u;      // r^2 below a table begin
constexpr unsigned ST_NBOVER = 2u;     // list entries beyond capacity
constexpr unsigned ST_GHOSTOVER = 4u;  // ghost atoms beyond capacity
constexpr unsigned ST_CELLOVER = 8u;   // atoms per cell beyond CELLCAP
constexpr unsigned ST_WAIT = 16u;      // a bounded wait on an asynchronous copy ran out
constexpr unsigned ST_BOUNDS = 32u;    // bounds-checked build: an index failed its check

// ---------------------------------------------------------------------------
// Bounds-checked build (-DIMDGPU_CHECK, not the default).  The indices the
// kernels take from device data (list partners, ghost owners, table rows,
// cell bins, permutation slots) are checked before use.  A failed check sets
// ST_BOUNDS in the status word and the site's bit in counters[CK_SITES],
// which nothing clears while the system lives (imdgpu_check_sites reads it),
// and the access is skipped, or the index clamped where the kernel needs
// one.  Without the macro every check is the constant true and compiles away.
// ---------------------------------------------------------------------------
constexpr int CK_PARTNER = 1;  // a list partner outside the real and ghost slots
constexpr int CK_OWNER = 2;    // a ghost's owner outside the real atoms
constexpr int CK_ROW = 4;      // a table row or column outside the table
constexpr int CK_BIN = 8;      // an atom's bin outside the cell grid
constexpr int CK_SLOT = 16;    // a permutation slot or caller index outside the atoms
constexpr int CK_SITES = 4;    // the counters slot of the failed sites

#ifdef IMDGPU_CHECK
static __device__ __noinline__ void check_failed(unsigned *status, int *counters, int site) {
  atomicOr(status, ST_BOUNDS);
  atomicOr(&counters[CK_SITES], site);
}
#endif

// One pot_table_t on the device.  `tri` holds, per column and row k, the
// three table values the quadratic interpolation reads (rows k, k+1, k+2):
// one aligned 32 B record per lookup instead of three strided loads.
//
// The fast kernels read the same quadratic in coefficient form: with
// dv = p1 - p0 and d2v = p2 - 2 p1 + p0 of row k,
//   value(chi) = A + chi (B + chi C),   A = p0, B = dv - d2v/2, C = d2v/2
//   2 dV/dr2   = G0 + chi G1,           G0 = 2 istep B, G1 = 4 istep C
// (algebraically IMD's p0 + chi dv + chi (chi-1) d2v / 2 and
// 2 istep (dv + (chi - 1/2) d2v)), three FMAs instead of ~15 operations.
// The 4-point and spline modes of IMD (src/potaccess.h:365-457) are cubic in
// chi on each row: value = A + chi (B + chi (C + chi D)), 2 dV/dr2 =
// G0 + chi (G1 + chi G2).  Quadratic rows have D = G2 = 0.
constexpr int TAB_QUADRATIC = 0, TAB_FOURPOINT = 1, TAB_SPLINE = 2;

struct DevTable {
  int ncols;
  int rows;                 // maxsteps + 2
  int mode;                 // TAB_*
  const double4 *tri;       // tri[col * rows + k] = (t[k], t[k+1], t[k+2], 0)
  const float4 *trif;       // same in FP32 (mixed precision)
  const double4 *cv;        // (A, B, C, D) per column and row
  const double4 *cg;        // (G0, G1, G2, 0)
  const double4 *cgn;       // -s (G0, G1, G2): negated gradient for the force pass
                            // (s = 1 for pair tables, 1/2 for rho: the EAM
                            // force term 0.5 (F'_i + F'_j) rho' needs rho'/2)
  const float4 *cvf;        // FP32 copies for the mixed path
  const float4 *cgf;
  double begin[MAXCOL];
  double end[MAXCOL];
  double invstep[MAXCOL];
  double boff[MAXCOL];      // -begin * invstep
  float fbegin[MAXCOL];
  float fend[MAXCOL];
  float finv[MAXCOL];
#ifdef IMDGPU_CHECK
  unsigned *chk_status;     // the system's status word and counters
  int *chk_counters;
#endif
};

// element of column col, row k of a table array; a checked build confirms
// both and reads row 0 of column 0 in place of a bad one
__device__ __forceinline__ size_t row_of(const DevTable &t, int col, int k) {
#ifdef IMDGPU_CHECK
  if (col < 0 || col >= t.ncols || k < 0 || k >= t.rows) {
    check_failed(t.chk_status, t.chk_counters, CK_ROW);
    return 0;
  }
#endif
  return (size_t)col * t.rows + k;
}

// Everything a kernel of one system needs, passed by value.
struct SysView {
  int n;                    // real atoms
  int ncap;                 // capacity of real-atom arrays (list stride)
  int gcap;                 // ghost capacity
  int ntypes;
  int nbcap;                // list entries per atom
  int nreal_cells;
  int nall_cells;
  int cdim[3], gdim[3];
  double box[3][3];
  double tbox[3][3];
  double cellvec[3][3];     // box rows / gdim
  int pbc[3];
  double cellsz;            // list radius^2
  double skin2;             // (nbl_margin/2)^2
  double restr[MAXT * 3];

  double4 *pos, *mom, *frc, *ref;
  double *rho, *df;
  float4 *xl;               // mixed: per atom FP32 (hi, lo) split of the position
  int *number, *orig;
  int *ecell;               // buffered cell id of every ext atom
  int *gowner;              // ghost -> owning real slot
  int *gcode;               // ghost -> packed image shift (sx+1) + 3(sy+1) + 9(sz+1)
  uint32_t *nbr;            // ELL list
  double4 *pcache;          // per list entry (same layout): r^2, -grad of phi, -rho'/2, phi
  int *nnb;                 // entries per atom
  int *cstart, *ccount;     // per buffered cell: first ext index, atoms
  const int *cell_rank;     // buffered lin -> Morton rank of real cell (-1 for buffer)
  const int *rank_lin;      // rank -> buffered lin
  const int *hshell;        // nshell buffered lin per real rank (-1 none): half or full shell
  int nshell;               // 14 (half list, IMD's AR order) or 27 (full or balanced list)
  int balanced;             // balanced half list: 27 cells, IMD's 14 first (see k_rb_build_half)
  int split;                // mixed: balanced half list at the front of each row (nnb), the
                            // other partners at its back (nnb2 of them, from nbcap - 1 down)
  int *nnb2;
  const int *bsrc;          // per buffer cell (enumerated): source real lin
  const int *blin;          // per buffer cell: its lin
  const int *bcode;         // per buffer cell: packed image shift
  int nbuf;                 // number of buffer cells used
  unsigned *status;
  int *counters;            // [0] ghosts, [1] max entries per atom, [2] max cell atoms
  double *partial;          // per-block partial sums

  // batch of independent systems (null for a single system): system of each
  // real atom, per-system box rows, reciprocal rows, cell grid, buffered
  // grid and first global cell index, and a per-system "finished" flag
  const int *atom_sys;
  const double *sbox, *stbox;  // 9 per system
  const int *sgdim, *scdim;    // 3 per system
  const int *scoff;            // 1 per system
  const int *sys_done;
  double4 *wrap_oldx;          // batch CG: old_x moved with the wrap of x
  int *sys_short;              // batch: per-system flag, a pair below a table begin
  int eshare;                  // force pass adds each atom's own pair energies to frc.w
  // per-system rebuilds (batch, imdgpu_batch_set_partial_rebuild): the flag
  // of each system that moved past skin/2, each system's fixed ghost range
  // [goff[q], goff[q + 1]) (unused slots have gowner -1), the system of each
  // real bin, of each buffer cell, and each system's first buffered cell
  int *sys_rb;
  const int *goff, *rank_sys, *buf_sys, *coff;
};

// idx within [0, lim): always true without -DIMDGPU_CHECK; a checked build
// records a failure (see CK_PARTNER ...)
__device__ __forceinline__ bool in_bounds(const SysView &v, long idx, long lim, int site) {
#ifdef IMDGPU_CHECK
  if (idx >= 0 && idx < lim) return true;
  check_failed(v.status, v.counters, site);
  return false;
#else
  (void)v, (void)idx, (void)lim, (void)site;
  return true;
#endif
}

// sc->rebuild: bit 0 rebuild everything, bit 1 rebuild the systems whose
// sys_rb flag is set
constexpr int RB_ALL = 1, RB_FLAGGED = 2;

// atoms of finished cells of a batch are skipped by the force passes
__device__ __forceinline__ bool atom_idle(const SysView &v, int i) {
  return v.sys_done && v.sys_done[v.atom_sys[i]];
}

// a rebuild in progress covers system q (flag: the value of sc->rebuild)
__device__ __forceinline__ bool rb_covers(const SysView &v, int flag, int q) {
  return (flag & RB_ALL) || !v.sys_rb || v.sys_rb[q];
}

// a pair of atom i closer than a table's first point (IMD's "Short
// distance"): the status word, and in a batch the flag of i's system
__device__ __forceinline__ void flag_short(const SysView &v, int i) {
  atomicOr(v.status, ST_SHORT);
  if (v.sys_short) atomicOr(&v.sys_short[v.atom_sys[i]], 1);
}

// system of real atom i (0 for a single system)
__device__ __forceinline__ int sys_of(const SysView &v, int i) {
  return v.atom_sys ? v.atom_sys[i] : 0;
}
// box row a, component c of the system
__device__ __forceinline__ double box_of(const SysView &v, int sys, int a, int c) {
  return v.sbox ? v.sbox[9 * sys + 3 * a + c] : v.box[a][c];
}
__device__ __forceinline__ double tbox_of(const SysView &v, int sys, int a, int c) {
  return v.stbox ? v.stbox[9 * sys + 3 * a + c] : v.tbox[a][c];
}

// ---------------------------------------------------------------------------
// exact FP64 helpers: no contraction into FMA, so bits match the C oracle and
// the reference built without fused multiply-add
// ---------------------------------------------------------------------------
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// r^2 = dx*dx + dy*dy + dz*dz, left to right (SPROD, src/makros.h:409)
__device__ __forceinline__ double r2_exact(double dx, double dy, double dz) {
  return dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
}

// Table index of PAIR_INT2 / VAL_FUNC2 / DERIV_FUNC2 (src/potaccess.h:323-345)
__device__ __forceinline__ int tab_index(double r2, double begin, double end,
                                         double invstep, double &chi, unsigned &shortf) {
  double r2a = r2 < end ? r2 : end;
  r2a = dsub(r2a, begin);
  if (r2a < 0) {
    r2a = 0;
    shortf = 1;
  }
  r2a = dmul(r2a, invstep);
  int k = __double2int_rz(r2a);
  chi = dsub(r2a, (double)k);
  return k;
}

// PAIR_INT2 (src/potaccess.h:323-354): value and twice the derivative
__device__ __forceinline__ void quad_vg(const double4 p, double chi, double istep,
                                        double &pot, double &grad) {
  double dv = dsub(p.y, p.x);
  double d2v = dadd(dsub(p.z, dmul(2.0, p.y)), p.x);
  pot = dadd(dadd(p.x, dmul(chi, dv)), dmul(dmul(dmul(0.5, chi), dsub(chi, 1.0)), d2v));
  grad = dmul(dmul(2.0, istep), dadd(dv, dmul(dsub(chi, 0.5), d2v)));
}
// VAL_FUNC2 (:465-495)
__device__ __forceinline__ double quad_v(const double4 p, double chi) {
  double dv = dsub(p.y, p.x);
  double d2v = dadd(dsub(p.z, dmul(2.0, p.y)), p.x);
  return dadd(dadd(p.x, dmul(chi, dv)), dmul(dmul(dmul(0.5, chi), dsub(chi, 1.0)), d2v));
}
// DERIV_FUNC2 (:591-621)
__device__ __forceinline__ double quad_g(const double4 p, double chi, double istep) {
  double dv = dsub(p.y, p.x);
  double d2v = dadd(dsub(p.z, dmul(2.0, p.y)), p.x);
  return dmul(dmul(2.0, istep), dadd(dv, dmul(dsub(chi, 0.5), d2v)));
}

// read-only 32 B load (two 16 B non-coherent loads)
__device__ __forceinline__ double4 ldg4(const double4 *p) {
  const double2 a = __ldg(reinterpret_cast<const double2 *>(p));
  const double2 b = __ldg(reinterpret_cast<const double2 *>(p) + 1);
  return make_double4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ double4 tab_load(const DevTable &t, int col, int k) {
  return ldg4(&t.tri[row_of(t, col, k)]);
}

__device__ __forceinline__ void pair_int2(const DevTable &t, int col, double r2, double &pot,
                                          double &grad, unsigned &shortf) {
  double chi;
  int k = tab_index(r2, t.begin[col], t.end[col], t.invstep[col], chi, shortf);
  quad_vg(tab_load(t, col, k), chi, t.invstep[col], pot, grad);
}
__device__ __forceinline__ double val_func2(const DevTable &t, int col, double r2,
                                            unsigned &shortf) {
  double chi;
  int k = tab_index(r2, t.begin[col], t.end[col], t.invstep[col], chi, shortf);
  return quad_v(tab_load(t, col, k), chi);
}
__device__ __forceinline__ double deriv_func2(const DevTable &t, int col, double r2,
                                              unsigned &shortf) {
  double chi;
  int k = tab_index(r2, t.begin[col], t.end[col], t.invstep[col], chi, shortf);
  return quad_g(tab_load(t, col, k), chi, t.invstep[col]);
}

// ---------------------------------------------------------------------------
// fast FP64 table access (FMA, coefficient form)
// ---------------------------------------------------------------------------
// r2 <= end / r2 < end for non-negative doubles, compared as integers so the
// test does not occupy the FP64 pipe
__device__ __forceinline__ bool le_pos(double a, double b) {
  return __double_as_longlong(a) <= __double_as_longlong(b);
}
__device__ __forceinline__ bool lt_pos(double a, double b) {
  return __double_as_longlong(a) < __double_as_longlong(b);
}

// floor(x) for 0 <= x < 2^21 from the bits of x (integer pipe only)
__device__ __forceinline__ int ifloor_pos(double x) {
  const int hi = __double2hiint(x);
  const int e = (hi >> 20) - 1023;                 // unbiased exponent, < 0 for x < 1
  const int m = (hi & 0xFFFFF) | 0x100000;         // top 21 bits of the significand
  return m >> min(20 - e, 31);
}
// (double)k for 0 <= k < 2^21, assembled from bits (exact)
__device__ __forceinline__ double small_int_to_double(int k) {
  const int p = 31 - __clz(k | 1);
  const int hi = ((1023 + p) << 20) | ((k << (20 - p)) & 0xFFFFF);
  return k ? __hiloint2double(hi, 0) : 0.0;
}

// Table index of the fast path: r2a = (min(r2, end) - begin) * invstep as one
// FMA; clamps, floor and int->double on the integer pipe, so only the FMA
// and the final subtraction use the (slow) FP64 pipe.  chi = r2a - k is
// exact.  Tables have fewer than 2^20 rows (checked at upload).
__device__ __forceinline__ int tab_index_fast(const DevTable &t, int col, double r2, double &chi) {
  const double rm = lt_pos(r2, t.end[col]) ? r2 : t.end[col];
  double r2a = fma(rm, t.invstep[col], t.boff[col]);
  if (__double2hiint(r2a) < 0) r2a = 0.0;          // below begin (short distance)
  int k = ifloor_pos(r2a);
  if (t.mode == TAB_FOURPOINT) k = max(k, 1);  // PAIR_INT3: rows k-1..k+2, k >= 1
  chi = r2a - small_int_to_double(k);
  return k;
}
__device__ __forceinline__ double4 cv_load(const DevTable &t, int col, int k) {
  return ldg4(&t.cv[row_of(t, col, k)]);
}
__device__ __forceinline__ double4 cg_load(const DevTable &t, int col, int k) {
  return ldg4(&t.cg[row_of(t, col, k)]);
}
__device__ __forceinline__ double4 cgn_load(const DevTable &t, int col, int k) {
  return ldg4(&t.cgn[row_of(t, col, k)]);
}
// CUB: cubic rows (4-point / spline); quadratic rows skip the zero terms
template <bool CUB = false>
__device__ __forceinline__ double poly_v(const double4 c, double chi) {
  return CUB ? fma(chi, fma(chi, fma(chi, c.w, c.z), c.y), c.x)
             : fma(chi, fma(chi, c.z, c.y), c.x);
}
template <bool CUB = false>
__device__ __forceinline__ double poly_g(const double4 g, double chi) {
  return CUB ? fma(chi, fma(chi, g.z, g.y), g.x) : fma(chi, g.y, g.x);
}

// Per-atom FP32 split of an FP64 position: x = hi + lo to ~2^-48 relative.
// The difference of two atoms, (hi_j - hi_i) + (lo_j - lo_i), is accurate to
// the last FP32 bit of the difference itself.
struct __align__(16) SplitPos {
  float4 hi;  // x, y, z, type (int bits)
  float4 lo;  // residuals
};
__device__ __forceinline__ SplitPos split_pos(const double4 p) {
  SplitPos o;
  o.hi.x = (float)p.x;
  o.hi.y = (float)p.y;
  o.hi.z = (float)p.z;
  o.hi.w = __int_as_float((int)p.w);
  o.lo.x = (float)(p.x - (double)o.hi.x);
  o.lo.y = (float)(p.y - (double)o.hi.y);
  o.lo.z = (float)(p.z - (double)o.hi.z);
  o.lo.w = 0.f;
  return o;
}
__device__ __forceinline__ SplitPos ldsp(const SplitPos *p) {
  SplitPos o;
  o.hi = __ldg(&p->hi);
  o.lo = __ldg(&p->lo);
  return o;
}

// A ghost copies its owner through the z, y, x buffer copies of send_cells
// (src/imd_comm_force_3d.c:247-358) in that order, so its position is
// ((x + s_z box_z) + s_y box_y) + s_x box_x component-wise.
__device__ __forceinline__ double4 ghost_image(const SysView &v, double4 p, int code, int sys) {
  const int sx = code % 3 - 1, sy = (code / 3) % 3 - 1, sz = code / 9 - 1;
  double c[3] = {p.x, p.y, p.z};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    double t = c[a];
    if (sz) t = dadd(t, sz > 0 ? box_of(v, sys, 2, a) : -box_of(v, sys, 2, a));
    if (sy) t = dadd(t, sy > 0 ? box_of(v, sys, 1, a) : -box_of(v, sys, 1, a));
    if (sx) t = dadd(t, sx > 0 ? box_of(v, sys, 0, a) : -box_of(v, sys, 0, a));
    c[a] = t;
  }
  return make_double4(c[0], c[1], c[2], p.w);
}

// ---------------------------------------------------------------------------
// FP32 variants (mixed precision): same index rule on r^2 computed in FP32
// ---------------------------------------------------------------------------
struct TabF {
  float begin, end, invstep;
};

__device__ __forceinline__ int tab_index_f(float r2, float begin, float end, float invstep,
                                           float &chi) {
  float r2a = fminf(r2, end) - begin;
  r2a = fmaxf(r2a, 0.0f) * invstep;
  int k = __float2int_rz(r2a);
  chi = r2a - (float)k;
  return k;
}
__device__ __forceinline__ void quadf_vg(const float4 p, float chi, float istep, float &pot,
                                         float &grad) {
  float dv = p.y - p.x;
  float d2v = p.z - 2.0f * p.y + p.x;
  pot = p.x + chi * dv + 0.5f * chi * (chi - 1.0f) * d2v;
  grad = 2.0f * istep * (dv + (chi - 0.5f) * d2v);
}
__device__ __forceinline__ float quadf_v(const float4 p, float chi) {
  float dv = p.y - p.x;
  float d2v = p.z - 2.0f * p.y + p.x;
  return p.x + chi * dv + 0.5f * chi * (chi - 1.0f) * d2v;
}
__device__ __forceinline__ float quadf_g(const float4 p, float chi, float istep) {
  float dv = p.y - p.x;
  float d2v = p.z - 2.0f * p.y + p.x;
  return 2.0f * istep * (dv + (chi - 0.5f) * d2v);
}

// ---------------------------------------------------------------------------
// reductions
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide sum of K values per thread into out[blockIdx.x * K + k]
// (deterministic: fixed shuffle tree, fixed warp order).
template <int K, int BS>
__device__ __forceinline__ void block_sum_store(double (&v)[K], double *out) {
  __shared__ double sh[K][BS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < BS / 32; i++) s += sh[threadIdx.x][i];
    out[(size_t)blockIdx.x * K + threadIdx.x] = s;
  }
}

// The same for any block of at most MAXBS threads, a multiple of 32 (the
// block shape the autotuner picked); deterministic for a given shape.
template <int K, int MAXBS>
__device__ __forceinline__ void block_sum_store_dyn(double (&v)[K], double *out) {
  __shared__ double sh[K][MAXBS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double s = warp_sum(v[k]);
    if (lane == 0) sh[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < K) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < MAXBS / 32; i++)
      if (i < nw) s += sh[threadIdx.x][i];
    out[(size_t)blockIdx.x * K + threadIdx.x] = s;
  }
}

// The per-block partials of a pass reduced by one block of FIN_BS threads:
// each thread folds a strided share, then warps and the block combine in a
// fixed order (sums, or maxima where bit k of MAXMASK is set); thread 0
// holds the totals.  Many independent loads in flight instead of one warp
// walking every partial.
constexpr int FIN_BS = 1024;
template <int K, unsigned MAXMASK>
__device__ __forceinline__ void fin_block(double (&v)[K]) {
  __shared__ double sh[K][FIN_BS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    v[k] = ((MAXMASK >> k) & 1u) ? warp_max(v[k]) : warp_sum(v[k]);
    if (lane == 0) sh[k][w] = v[k];
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; k++)
      v[k] = ((MAXMASK >> k) & 1u) ? warp_max(sh[k][lane]) : warp_sum(sh[k][lane]);
  }
}

}  // namespace imdgpu
