// output.cu -- IMD's checkpoint text formatted on the device.
//
// write_atoms_config (src/imd_io_3d.c:696-948, the text branch) prints one
// line per atom with sprintf: "%d %d" NUMMER and type, then RESOL1 mass,
// RESOL3 position, RESOL3 velocity (momentum / mass; not in CG runs),
// RESOL1 POTENG and, in EAM2 builds, RESOL1 EAM_RHO, and "\n"; RESOL1 is
// " %12.16f" with the hpo option and " %f" without (:704-711).  For N atoms
// that is 10-11 N printf conversions on one host core, after a copy of the
// whole state to the host.  Here every line is formatted by one device
// thread (fmtfixed.cuh, byte for byte glibc's output): a first pass measures
// each line, an exclusive scan places them, a second pass writes them, and
// only the finished text crosses to the host.
#include <algorithm>
#include <cstdio>

#include "../../include/imdgpu.h"
#include "fmtfixed.cuh"
#include "kernels.cuh"

namespace imdgpu {

constexpr int FMT_LINE_MAX = 448;   // one atom line: 2 ints + 9 numbers + padding
constexpr int SCAN_BS = 1024;

struct LineSrc {
  // atoms: slot of line a = slot_of[order ? order[a] : a]
  const double4 *pos, *mom, *frc;
  const double *rho;
  const int *number, *slot_of, *order;
  // plain numbers (imdgpu_format_fixed)
  const double *x;
  int prec, width;
  int flags;
};

// the text of line a into out; its length, or -1 when a value is outside
// what fmt_fixed handles (|v| >= 2^63)
__device__ int make_line(const LineSrc &L, int a, char *out) {
  using namespace imdfmt;
  if (L.x) {
    int n = fmt_fixed(L.x[a], L.prec, L.width, out);
    if (n < 0) return -1;
    out[n++] = '\n';
    return n;
  }
  const int caller = L.order ? L.order[a] : a;
  const int s = L.slot_of[caller];
  const double4 p = L.pos[s], m = L.mom[s];
  const bool hpo = (L.flags & IMDGPU_FMT_HPO) != 0;
  const int prec = hpo ? 16 : 6, width = hpo ? 12 : 0;
  int n = fmt_int(L.number[s], out);
  out[n++] = ' ';
  n += fmt_int((int)p.w, out + n);
  double vals[9];
  int nv = 0;
  vals[nv++] = m.w;
  vals[nv++] = p.x;
  vals[nv++] = p.y;
  vals[nv++] = p.z;
  if (L.flags & IMDGPU_FMT_VELOCITY) {
    vals[nv++] = __ddiv_rn(m.x, m.w);
    vals[nv++] = __ddiv_rn(m.y, m.w);
    vals[nv++] = __ddiv_rn(m.z, m.w);
  }
  vals[nv++] = L.frc[s].w;
  if (L.flags & IMDGPU_FMT_EAM_RHO) vals[nv++] = L.rho[s];
  for (int k = 0; k < nv; k++) {
    out[n++] = ' ';
    const int w = fmt_fixed(vals[k], prec, width, out + n);
    if (w < 0) return -1;
    n += w;
  }
  out[n++] = '\n';
  return n;
}

// pass 1: lengths; the lowest line that cannot be formatted goes to *bad
__global__ void k_line_len(LineSrc L, int n, long *len, int *bad) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  char buf[FMT_LINE_MAX];
  const int l = make_line(L, a, buf);
  if (l < 0) {
    atomicMin(bad, a);
    len[a] = 0;
  } else {
    len[a] = l;
  }
}

// exclusive scan of len in blocks of SCAN_BS, block totals to bsum
__global__ void __launch_bounds__(SCAN_BS) k_scan_block(long *len, int n, long *bsum) {
  __shared__ long sh[SCAN_BS];
  const int a = blockIdx.x * SCAN_BS + threadIdx.x;
  const long v = a < n ? len[a] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < SCAN_BS; o <<= 1) {
    const long t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (a < n) len[a] = sh[threadIdx.x] - v;
  if (threadIdx.x == SCAN_BS - 1) bsum[blockIdx.x] = sh[threadIdx.x];
}

// exclusive scan of the block totals (one thread walks them; a few
// thousand blocks at most), the grand total into bsum[nb]
__global__ void k_scan_totals(long *bsum, int nb) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  long run = 0;
  for (int b = 0; b < nb; b++) {
    const long t = bsum[b];
    bsum[b] = run;
    run += t;
  }
  bsum[nb] = run;
}

// pass 2: every line at its offset
__global__ void k_line_write(LineSrc L, int n, const long *off, const long *bsum, char *out) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a >= n) return;
  char buf[FMT_LINE_MAX];
  const int l = make_line(L, a, buf);
  if (l <= 0) return;
  char *dst = out + off[a] + bsum[a / SCAN_BS];
  for (int k = 0; k < l; k++) dst[k] = buf[k];
}

static int fmt_fail(int code, const char *msg) {
  set_last_error(msg);
  return code;
}

#define FCK(x)                                                                  \
  do {                                                                          \
    cudaError_t e_ = (x);                                                       \
    if (e_ != cudaSuccess) return fmt_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e_)); \
  } while (0)

// Formats the n lines of L: sizes them, and when cap >= the total writes
// the text to buf (host).  Scratch from the caller's FormatScratch.
static int format_lines(const LineSrc &L, int n, char *buf, long cap, long *len,
                        FormatScratch &fs, cudaStream_t st) {
  if (n < 0 || !len) return fmt_fail(IMDGPU_ERR_ARG, "format: bad arguments");
  if (n == 0) {
    *len = 0;
    return IMDGPU_OK;
  }
  const int nb = (n + SCAN_BS - 1) / SCAN_BS;
  if (fs.cap_lines < n) {
    cudaFree(fs.len);
    cudaFree(fs.bsum);
    fs.len = nullptr;
    fs.bsum = nullptr;
    FCK(cudaMalloc(&fs.len, sizeof(long) * (size_t)n));
    FCK(cudaMalloc(&fs.bsum, sizeof(long) * ((size_t)nb + 1)));
    fs.cap_lines = n;
  }
  if (!fs.bad) FCK(cudaMalloc(&fs.bad, sizeof(int)));
  FCK(cudaMemcpyAsync(fs.bad, &n, sizeof(int), cudaMemcpyHostToDevice, st));
  const int bs = 128, grid = (n + bs - 1) / bs;
  k_line_len<<<grid, bs, 0, st>>>(L, n, fs.len, fs.bad);
  k_scan_block<<<nb, SCAN_BS, 0, st>>>(fs.len, n, fs.bsum);
  k_scan_totals<<<1, 32, 0, st>>>(fs.bsum, nb);
  FCK(cudaGetLastError());
  long total = 0;
  int bad = n;
  FCK(cudaMemcpyAsync(&total, fs.bsum + nb, sizeof(long), cudaMemcpyDeviceToHost, st));
  FCK(cudaMemcpyAsync(&bad, fs.bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  FCK(cudaStreamSynchronize(st));
  if (bad < n) {
    char msg[128];
    snprintf(msg, sizeof msg, "format: a value of line %d is 2^63 or more in magnitude", bad);
    return fmt_fail(IMDGPU_ERR_ARG, msg);
  }
  *len = total;
  if (!buf || cap < total) return IMDGPU_OK;
  if (fs.cap_bytes < total) {
    cudaFree(fs.text);
    fs.text = nullptr;
    FCK(cudaMalloc(&fs.text, (size_t)total));
    fs.cap_bytes = total;
  }
  k_line_write<<<grid, bs, 0, st>>>(L, n, fs.len, fs.bsum, fs.text);
  FCK(cudaGetLastError());
  FCK(cudaMemcpyAsync(buf, fs.text, (size_t)total, cudaMemcpyDeviceToHost, st));
  FCK(cudaStreamSynchronize(st));
  return IMDGPU_OK;
}

void free_format_scratch(FormatScratch &fs) {
  cudaFree(fs.len);
  cudaFree(fs.bsum);
  cudaFree(fs.bad);
  cudaFree(fs.text);
  fs = FormatScratch{};
}

// the atom lines of write_atoms_config for a system: order (device, caller
// indices) or caller order when null
int format_atom_lines(const SysView &v, const int *slot_of, const int *order, int n, int flags,
                      char *buf, long cap, long *len, FormatScratch &fs, cudaStream_t st) {
  LineSrc L{};
  L.pos = v.pos;
  L.mom = v.mom;
  L.frc = v.frc;
  L.rho = v.rho;
  L.number = v.number;
  L.slot_of = slot_of;
  L.order = order;
  L.flags = flags;
  return format_lines(L, n, buf, cap, len, fs, st);
}

}  // namespace imdgpu

using namespace imdgpu;

extern "C" int imdgpu_format_fixed(const double *x, int n, int prec, int width, char *buf,
                                   long cap, long *len) {
  if (!x || n < 0 || prec < 0 || prec > 17 || width < 0 || width > 64 || !len)
    return fmt_fail(IMDGPU_ERR_ARG, "imdgpu_format_fixed: bad arguments");
  double *dx = nullptr;
  FCK(cudaMalloc(&dx, sizeof(double) * (size_t)(n > 0 ? n : 1)));
  FCK(cudaMemcpy(dx, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice));
  LineSrc L{};
  L.x = dx;
  L.prec = prec;
  L.width = width;
  FormatScratch fs{};
  int rc = format_lines(L, n, buf, cap, len, fs, 0);
  free_format_scratch(fs);
  cudaFree(dx);
  return rc;
}
