// noalloc.cu -- move_atoms_nve for callers that cannot allocate device memory.
//
// The NVE integrator of system.cu reduces kinetic energy, |F|^2, the largest
// force component and the largest displacement since the last list build
// through per-block partial sums: scratch memory beyond its inputs and
// outputs.  imdgpu_create() and friends obtain that scratch with cudaMalloc.
// Some callers cannot do that: a host program whose device memory is owned by
// its own pool or arena (every byte on the device handed out and accounted for
// by it), or one that must never hit the implicit device synchronisation that
// cudaMalloc / cudaFree can cause in the middle of its time step.  For them
// this file provides one entry point that allocates nothing: the caller passes
// its own device arrays, and the partial sums live in a file-scope
// __device__ array of fixed size, present on every device that loads the
// library until the process exits.
#include <cstdio>
#include <mutex>

#include "../../include/imdgpu.h"
#include "kernels.cuh"

namespace {

constexpr int NA_BS = 256;                        // threads per block
constexpr int NA_MAX_ATOMS = 1 << 24;             // 16,777,216 atoms per call
constexpr int NA_MAX_BLOCKS = NA_MAX_ATOMS / NA_BS;
constexpr int NA_MAX_DEVICES = 64;
constexpr int NA_SLOTS = 5;                       // partial results per block
// 5 partials per block + 5 final values: 2.5 MiB + 40 B per device
constexpr size_t NA_SCRATCH_DOUBLES = NA_SLOTS * (size_t)NA_MAX_BLOCKS + NA_SLOTS;

__device__ __align__(256) double g_nve_scratch[NA_SCRATCH_DOUBLES];

// In host code g_nve_scratch names a host-side stand-in, not device memory:
// kernels receive the device address obtained below, once per device.
double *g_scratch_dev[NA_MAX_DEVICES] = {nullptr};
std::mutex g_scratch_mu;

struct Restr {
  double r[imdgpu::MAXT * 3];
};

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }

// Same arithmetic as k_nve (src/imd_integrate.c:32-497), on atom-major
// caller arrays x[3i+c], p[3i+c], f[3i+c]; the masked force is written back
// as the reference does with KRAFT.  The types come straight from the
// caller's device memory: an atom whose type is outside 0..ntypes-1 is left
// as it is (its restriction row does not exist) and the lowest such atom
// index goes to the fifth partial, so that the call can refuse the input.
__global__ void __launch_bounds__(NA_BS) k_nve_noalloc(int n, int ntypes, double *x, double *p,
                                                       double *f, const double *mass,
                                                       const int *type, Restr rs, double dt,
                                                       const double *xref, double *partial) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double ek = 0.0, fn = 0.0, fm = 0.0, dm = 0.0;
  double bad = (double)n;  // lowest atom with a bad type; n = none
  if (i < n && (type[i] < 0 || type[i] >= ntypes)) bad = (double)i;
  else if (i < n) {
    const int t = type[i];
    double px = p[3 * i], py = p[3 * i + 1], pz = p[3 * i + 2];
    double fx = f[3 * i], fy = f[3 * i + 1], fz = f[3 * i + 2];
    const double m = mass[i];
    const double kin1 = dadd(dadd(dmul(px, px), dmul(py, py)), dmul(pz, pz));
    fx = dmul(fx, rs.r[3 * t]);
    fy = dmul(fy, rs.r[3 * t + 1]);
    fz = dmul(fz, rs.r[3 * t + 2]);
    f[3 * i] = fx;
    f[3 * i + 1] = fy;
    f[3 * i + 2] = fz;
    fn = dadd(dadd(dmul(fx, fx), dmul(fy, fy)), dmul(fz, fz));
    fm = fmax(fmax(fx * fx, fy * fy), fz * fz);
    px = dadd(px, dmul(dt, fx));
    py = dadd(py, dmul(dt, fy));
    pz = dadd(pz, dmul(dt, fz));
    const double kin2 = dadd(dadd(dmul(px, px), dmul(py, py)), dmul(pz, pz));
    ek = dadd(kin1, kin2) / (4.0 * m);
    const double tmp = dt / m;
    const double nx = dadd(x[3 * i], dmul(tmp, px));
    const double ny = dadd(x[3 * i + 1], dmul(tmp, py));
    const double nz = dadd(x[3 * i + 2], dmul(tmp, pz));
    p[3 * i] = px;
    p[3 * i + 1] = py;
    p[3 * i + 2] = pz;
    x[3 * i] = nx;
    x[3 * i + 1] = ny;
    x[3 * i + 2] = nz;
    if (xref) {
      const double ddx = dsub(nx, xref[3 * i]), ddy = dsub(ny, xref[3 * i + 1]),
                   ddz = dsub(nz, xref[3 * i + 2]);
      dm = dadd(dadd(dmul(ddx, ddx), dmul(ddy, ddy)), dmul(ddz, ddz));
    }
  }
  // every block overwrites its own NA_SLOTS slots: nothing carries over
  // from an earlier call
  __shared__ double sh[NA_SLOTS][NA_BS / 32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  ek = imdgpu::warp_sum(ek);
  fn = imdgpu::warp_sum(fn);
  fm = imdgpu::warp_max(fm);
  dm = imdgpu::warp_max(dm);
  bad = -imdgpu::warp_max(-bad);
  if (lane == 0) {
    sh[0][w] = ek;
    sh[1][w] = fn;
    sh[2][w] = fm;
    sh[3][w] = dm;
    sh[4][w] = bad;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0, b = 0, c = 0, d = 0, e = (double)n;
    for (int k = 0; k < NA_BS / 32; k++) {
      a += sh[0][k];
      b += sh[1][k];
      c = fmax(c, sh[2][k]);
      d = fmax(d, sh[3][k]);
      e = fmin(e, sh[4][k]);
    }
    double *o = partial + NA_SLOTS * (size_t)blockIdx.x;
    o[0] = a;
    o[1] = b;
    o[2] = c;
    o[3] = d;
    o[4] = e;
  }
}

// fixed-order reduction of the nb block partials into out (NA_SLOTS values)
__global__ void k_nve_noalloc_final(const double *partial, int nb, int n, double *out) {
  const int lane = threadIdx.x;
  double a = 0, b = 0, c = 0, d = 0, e = (double)n;
  for (int k = lane; k < nb; k += 32) {
    const double *q = partial + NA_SLOTS * (size_t)k;
    a += q[0];
    b += q[1];
    c = fmax(c, q[2]);
    d = fmax(d, q[3]);
    e = fmin(e, q[4]);
  }
  a = imdgpu::warp_sum(a);
  b = imdgpu::warp_sum(b);
  c = imdgpu::warp_max(c);
  d = imdgpu::warp_max(d);
  e = -imdgpu::warp_max(-e);
  if (lane == 0) {
    out[0] = a;
    out[1] = b;
    out[2] = c;
    out[3] = d;
    out[4] = e;
  }
}

int na_fail(int code, const char *msg) {
  imdgpu::set_last_error(msg);  // reported by imdgpu_last_error()
  return code;
}

// Device address of g_nve_scratch on the current device, looked up the first
// time this device is used (with it current) and cached.
int scratch_for_current_device(double **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(IMDGPU_ERR_ARG, "device index out of range");
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (!g_scratch_dev[dev]) {
    void *ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_nve_scratch);
    if (e != cudaSuccess) return na_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e));
    g_scratch_dev[dev] = static_cast<double *>(ptr);
  }
  *out = g_scratch_dev[dev];
  return IMDGPU_OK;
}

}  // namespace

extern "C" {

int imdgpu_move_atoms_nve_noalloc(int n, int ntypes, double *x, double *p, double *f,
                                  const double *mass, const int *type, const double *restr,
                                  double timestep, const double *x_ref, double *out,
                                  void *stream) {
  if (n <= 0 || !x || !p || !f || !mass || !type || !out)
    return na_fail(IMDGPU_ERR_ARG, "imdgpu_move_atoms_nve_noalloc: bad arguments");
  if (n > NA_MAX_ATOMS)
    return na_fail(IMDGPU_ERR_ARG,
                   "imdgpu_move_atoms_nve_noalloc: more than 16777216 atoms (the size of its "
                   "fixed scratch); use imdgpu_move_atoms_nve");
  if (ntypes < 1 || ntypes > imdgpu::MAXT)
    return na_fail(IMDGPU_ERR_ARG, "imdgpu_move_atoms_nve_noalloc: ntypes must be 1..4");
  double *scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  Restr rs;
  for (int k = 0; k < imdgpu::MAXT * 3; k++) rs.r[k] = 1.0;
  if (restr)
    for (int k = 0; k < 3 * ntypes; k++) rs.r[k] = restr[k];
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int nb = (n + NA_BS - 1) / NA_BS;
  double *fin = scratch + NA_SLOTS * (size_t)NA_MAX_BLOCKS;
  k_nve_noalloc<<<nb, NA_BS, 0, st>>>(n, ntypes, x, p, f, mass, type, rs, timestep, x_ref,
                                      scratch);
  k_nve_noalloc_final<<<1, 32, 0, st>>>(scratch, nb, n, fin);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e));
  double res[NA_SLOTS];
  e = cudaMemcpyAsync(res, fin, sizeof(res), cudaMemcpyDeviceToHost, st);
  if (e != cudaSuccess) return na_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e));
  e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return na_fail(IMDGPU_ERR_CUDA, cudaGetErrorString(e));
  for (int k = 0; k < 4; k++) out[k] = res[k];
  if (res[4] < (double)n) {
    char msg[160];
    snprintf(msg, sizeof msg,
             "imdgpu_move_atoms_nve_noalloc: atom %ld has a type outside 0..%d; atoms with "
             "such types were not moved",
             (long)res[4], ntypes - 1);
    return na_fail(IMDGPU_ERR_ARG, msg);
  }
  return IMDGPU_OK;
}

}  // extern "C"
