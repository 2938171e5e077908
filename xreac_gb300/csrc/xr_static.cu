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
// make that first call before any stream capture begins. The looked-up address is kept for the
// life of the process: after cudaDeviceReset (or anything else that destroys the device's primary
// context) the array may move, so this entry point must not be used on that device again. A
// caller-supplied stream must belong to the current device.
#include <cmath>
#include <cstring>
#include <mutex>

#include "xr_common.cuh"
#include "xr_describe.h"
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
thread_local const char* g_err = "";

int fail(int code, const char* msg) {
  g_err = msg;
  return code;
}

// Device address of the scratch array on the current device, looked up on every call (a runtime table
// lookup): a cached address would go stale after a device reset re-creates the primary context.
int scratch_for_current_device(unsigned char** out) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(XR_ECUDA, "no usable current CUDA device");
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
  if (e != cudaSuccess || !p) return fail(XR_ECUDA, "cudaGetSymbolAddress of the static scratch failed");
  *out = static_cast<unsigned char*>(p);
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
  const char* msg = "";
  int code = xr_host::describe_system(*sys, 0, cutoff, S, nullptr, &msg);
  if (code != XR_OK) return fail(code, msg);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {
    // the scratch address belongs to the current device; work on another device's stream would
    // touch memory that is not this device's array
    int cur = -1, sdev = -1;
    if (cudaGetDevice(&cur) != cudaSuccess || cudaStreamGetDevice(st, &sdev) != cudaSuccess)
      return fail(XR_EINPUT, "the stream's device could not be determined");
    if (sdev != cur) return fail(XR_EINPUT, "stream belongs to another device than the current one");
  }
  unsigned char* base = nullptr;
  code = scratch_for_current_device(&base);
  if (code != XR_OK) return code;

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
