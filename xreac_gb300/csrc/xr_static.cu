// Allocation-free neighbour counting: xr_count_neighbors_static (include/xreac_gb300.h).
//
// The count pass of the neighbour search (k_prep + k_neighbors<false>, the kernels xr_eval runs)
// with every piece of device scratch carved out of one statically sized array in this library,
// so the call performs no cudaMalloc, cudaFree or other allocating runtime or library call.
//
// Who needs it: callers that cannot allocate device memory at the point where they need the
// count. A host process whose device memory is owned by a framework's pool allocator (a caching
// allocator, or a runtime that reserves most of the free memory up front) can see a library's own
// cudaMalloc fail or fragment the pool; an MD or serving loop cannot afford the implicit device-wide
// synchronisation of cudaFree (and, on some drivers, of cudaMalloc) between steps; and a caller
// that sizes its own neighbour buffers must learn the row lengths before it allocates anything.
// xr_eval's context grows its buffers on demand and so serves none of them.
//
// Limits: at most XR_STATIC_MAX_ATOMS atoms per call (about 2 MiB of device scratch, resident
// from the moment the library's device code is loaded). The scratch is shared by every call in
// the process on that device, so calls that overlap in time (two host threads, or two streams
// without ordering between them) race on it. The first call on a device does the set-up
// (cudaGetSymbolAddress with that device current, which also loads this module's device code);
// make that first call before any stream capture begins.
#include <cmath>
#include <cstring>
#include <mutex>

#include "xr_common.cuh"
#include "xreac_gb300.h"

namespace {

constexpr int kMax = XR_STATIC_MAX_ATOMS;
constexpr int kMaxDevices = 64;
static_assert(kMax == 16384, "the size-limit message below quotes the limit");

constexpr size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

// Scratch layout (byte offsets), each region 256-byte aligned.
constexpr size_t kOffX = 0;                                                      // double4_32a[kMax]
constexpr size_t kOffXyz = kOffX + align256(sizeof(double4_32a) * kMax);         // double[3 kMax]
constexpr size_t kOffSysOf = kOffXyz + align256(sizeof(double) * 3 * kMax);      // int[kMax]
constexpr size_t kOffWrap = kOffSysOf + align256(sizeof(int) * kMax);            // int4[kMax]
constexpr size_t kOffXw = kOffWrap + align256(sizeof(int4) * kMax);              // float4[kMax]
constexpr size_t kOffFw = kOffXw + align256(sizeof(float4) * kMax);              // float4[kMax]
constexpr size_t kOffCnt = kOffFw + align256(sizeof(float4) * kMax);             // int[4 (kMax + 1)]
constexpr size_t kOffStatus = kOffCnt + align256(sizeof(int) * 4 * (kMax + 1));  // int
constexpr size_t kOffSys = kOffStatus + 256;                                     // XrSystem
constexpr size_t kScratchBytes = kOffSys + align256(sizeof(XrSystem));

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kMaxDevices] = {};
thread_local const char* g_err = "";

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}

// Device address of the scratch array on the current device, looked up once per device.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(XR_ECUDA, "no usable current CUDA device");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) return fail(XR_ECUDA, "cudaGetSymbolAddress of the static scratch failed");
    g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[dev];
  return XR_OK;
}

void inverse3(const double m[9], double inv[9], double* det_out) {
  const double a = m[0], b = m[1], c = m[2], d = m[3], e = m[4], f = m[5], g = m[6], h = m[7], i = m[8];
  const double A = e * i - f * h, B = -(d * i - f * g), C = d * h - e * g;
  const double det = a * A + b * B + c * C;
  *det_out = det;
  inv[0] = A / det;
  inv[3] = B / det;
  inv[6] = C / det;
  inv[1] = -(b * i - c * h) / det;
  inv[4] = (a * i - c * g) / det;
  inv[7] = -(a * h - b * g) / det;
  inv[2] = (b * f - c * e) / det;
  inv[5] = -(a * f - c * d) / det;
  inv[8] = (a * e - b * d) / det;
}

// System descriptor with the same fields, image reach and FP32 error band as xr_eval's.
int describe(const xr_system& in, double rc, XrSystem& S) {
  std::memset(&S, 0, sizeof(S));
  S.natoms = in.natoms;
  bool any = false;
  for (int k = 0; k < 3; ++k) {
    S.periodic[k] = in.pbc[k] ? 1 : 0;
    any = any || S.periodic[k];
  }
  double cell[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (any) {
    if (!in.cell) return fail(XR_EINPUT, "A cell is required when pbc is enabled");
    for (int k = 0; k < 9; ++k) cell[k] = in.cell[k];
  }
  double inv[9], det;
  inverse3(cell, inv, &det);
  if (!(std::fabs(det) > 0) || !std::isfinite(det))
    return fail(XR_EINPUT, "Periodic cells must be nonsingular and right-handed");
  double heights[3], lens[3];
  for (int k = 0; k < 3; ++k) {
    S.cell[k] = cell[k];
    S.cell[3 + k] = cell[3 + k];
    S.cell[6 + k] = cell[6 + k];
    heights[k] = 1.0 / std::sqrt(inv[k] * inv[k] + inv[3 + k] * inv[3 + k] + inv[6 + k] * inv[6 + k]);
    lens[k] = std::sqrt(cell[3 * k] * cell[3 * k] + cell[3 * k + 1] * cell[3 * k + 1] + cell[3 * k + 2] * cell[3 * k + 2]);
    if (S.periodic[k] && !(heights[k] > 2.0 * rc * (1.0 + 1e-9))) S.reach[k] = (int)std::floor(rc / heights[k] + 0.5) + 1;
  }
  for (int k = 0; k < 9; ++k) {
    S.inv[k] = inv[k];
    S.cellf[k] = (float)cell[k];
  }
  double origin[3] = {0, 0, 0}, ext = 0.0;
  for (int a = 0; a < in.natoms; ++a) {
    const double* p = in.positions + 3 * a;
    if (!std::isfinite(p[0]) || !std::isfinite(p[1]) || !std::isfinite(p[2]))
      return fail(XR_EINPUT, "positions must be a finite (N, 3) array in Angstrom");
    double wr[3], xw[3];
    for (int k = 0; k < 3; ++k) {
      const double fk = p[0] * inv[k] + p[1] * inv[3 + k] + p[2] * inv[6 + k];
      wr[k] = S.periodic[k] ? std::floor(fk) : 0.0;
    }
    for (int q = 0; q < 3; ++q) xw[q] = p[q] - (wr[0] * cell[q] + wr[1] * cell[3 + q] + wr[2] * cell[6 + q]);
    if (a == 0)
      for (int q = 0; q < 3; ++q) origin[q] = xw[q];
    for (int q = 0; q < 3; ++q) ext = std::fmax(ext, std::fabs(xw[q] - origin[q]));
  }
  double img = 0.0;
  for (int k = 0; k < 3; ++k)
    if (S.periodic[k]) img += (S.reach[k] + 2) * lens[k];
  const double C = 2.0 * ext + img + 1.0;
  const double u = 1.0 / 16777216.0;  // 2^-24
  const double delta = 8.0 * u * C;    // per-component bound on |FP32 v - FP64 v|
  const double margin = 2.0 * std::sqrt(3.0) * (rc + 2.0 * delta) * delta + 3.0 * delta * delta + 8.0 * u * rc * rc;
  S.margin = (float)(4.0 * margin + 1e-6);
  for (int q = 0; q < 3; ++q) S.origin[q] = origin[q];
  S.rc = rc;
  S.rc2 = rc * rc;
  S.bond_cut = std::fmin(5.0, rc);
  S.hb_cut = std::fmin(7.5, rc);
  S.rc2f = (float)S.rc2;
  S.bc2f = (float)(S.bond_cut * S.bond_cut);
  S.hc2f = (float)(S.hb_cut * S.hb_cut);
  return XR_OK;
}

// Writes the descriptor, packs the uploaded positions, and clears the status word (the only
// scratch the count pass accumulates into; the per-atom counts are stored, not added).
__global__ void k_static_setup(XrSystem S, XrSystem* sys, const double* xyz, double4_32a* x, int* sys_of,
                               int* status, int n) {
  const int a = blockIdx.x * blockDim.x + threadIdx.x;
  if (a == 0) {
    *sys = S;
    *status = 0;
  }
  if (a < n) {
    x[a] = make_double4_32a(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], 0.0);
    sys_of[a] = 0;
  }
}

}  // namespace

extern "C" const char* xr_static_last_error(void) { return g_err; }

extern "C" int xr_count_neighbors_static(const xr_system* sys, double cutoff, void* stream, int* counts,
                                         long long* total) {
  g_err = "";
  if (!sys || !counts || (sys->natoms > 0 && !sys->positions))
    return fail(XR_EINPUT, "sys, sys->positions and counts must be non-NULL");
  if (sys->natoms < 0) return fail(XR_EINPUT, "natoms must be non-negative");
  if (sys->natoms > kMax) return fail(XR_ECAPACITY, "natoms exceeds XR_STATIC_MAX_ATOMS (16384)");
  if (!(cutoff > 0.0) || !std::isfinite(cutoff)) return fail(XR_EINPUT, "cutoff must be positive and finite");
  if (total) *total = 0;
  const int n = sys->natoms;
  if (n == 0) return XR_OK;
  XrSystem S;
  int code = describe(*sys, cutoff, S);
  if (code != XR_OK) return code;
  unsigned char* base = nullptr;
  code = scratch_for_current_device(&base);
  if (code != XR_OK) return code;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  XrWork w;
  std::memset(&w, 0, sizeof(w));
  w.A = n;
  w.S = 1;
  w.sys = reinterpret_cast<const XrSystem*>(base + kOffSys);
  w.status = reinterpret_cast<int*>(base + kOffStatus);
  w.x = reinterpret_cast<const double4_32a*>(base + kOffX);
  w.sys_of = reinterpret_cast<const int*>(base + kOffSysOf);
  w.wrap = reinterpret_cast<int4*>(base + kOffWrap);
  w.xw = reinterpret_cast<float4*>(base + kOffXw);
  w.fw = reinterpret_cast<float4*>(base + kOffFw);
  w.cnt = reinterpret_cast<int*>(base + kOffCnt);
  double* xyz = reinterpret_cast<double*>(base + kOffXyz);

  if (cudaMemcpyAsync(xyz, sys->positions, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, st) != cudaSuccess)
    return fail(XR_ECUDA, "position upload failed");
  k_static_setup<<<(n + 255) / 256, 256, 0, st>>>(S, reinterpret_cast<XrSystem*>(base + kOffSys), xyz,
                                                   reinterpret_cast<double4_32a*>(base + kOffX),
                                                   reinterpret_cast<int*>(base + kOffSysOf), w.status, n);
  xr_launch_topology(w, st);
  if (cudaGetLastError() != cudaSuccess) return fail(XR_ECUDA, "kernel launch failed");
  int status = 0;
  // Row 0 of the [4][A + 1] count array holds the directed edges of each atom.
  if (cudaMemcpyAsync(counts, w.cnt, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&status, w.status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return fail(XR_ECUDA, "count read-back failed");
  if (status & XR_S_COINCIDENT) return fail(XR_ECOINCIDENT, "Coincident atoms are not supported");
  if (status & XR_S_SHIFT_RANGE) return fail(XR_ECAPACITY, "an image shift exceeds +-255 cells");
  if (total) {
    long long t = 0;
    for (int a = 0; a < n; ++a) t += counts[a];
    *total = t;
  }
  return XR_OK;
}
