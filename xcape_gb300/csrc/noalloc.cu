// noalloc.cu -- xc_loopcape_ex_noalloc: the ordered CAPE lift for callers
// that cannot allocate device memory.
//
// Some callers may not call cudaMalloc while they work: a host framework
// that reserves the device memory up front and hands out every byte itself
// (a serving process under a fixed memory budget), or a real-time loop that
// forbids allocation after start-up.  xc_loopcape_ex wants a caller-provided
// workspace to order the columns; this entry point takes that scratch from
// a file-scope __device__ array instead, so the caller passes only its
// inputs and outputs and nothing is allocated per call.
//
// * The array holds the ordering scratch for at most XC_NOALLOC_MAX_COLUMNS
//   columns (about 6.1 MiB).  Every GPU that loads this library holds it
//   until the process exits.
// * Host code cannot use the array's name as a device address.  The first
//   call on each device looks the address up with cudaGetSymbolAddress (with
//   that device current) and keeps it; that first call should therefore come
//   before any stream capture.
// * All calls share the one array, and it keeps the last call's contents.
//   The bucket counters that must start at zero are cleared at every call.
//   Calls that overlap on the GPU (on different streams, or from several host
//   threads without ordering) race on the array: issue them one after the
//   other.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include <mutex>

#include "../../include/xcape_gb300.h"
#include "xc_kernels.h"

namespace {

// 64 KiB of bucket counters + a 16-bit bucket + a 32-bit permutation entry
// per column, each part rounded up to 256 bytes.
constexpr size_t kNoallocScratchBytes =
    65536 + 2 * (size_t)XC_NOALLOC_MAX_COLUMNS + 4 * (size_t)XC_NOALLOC_MAX_COLUMNS + 512;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
void *g_addr[kMaxDevices] = {};

// Formats the message into xc_last_error() and returns code.
int noalloc_fail(int code, const char *fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  return xc::set_error(code, msg);
}

// Device address of g_noalloc_scratch on the current device (looked up once
// per device).
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return noalloc_fail(XC_ERR_CUDA, "cudaGetDevice: %s", cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return noalloc_fail(XC_ERR_INVALID, "device %d is beyond the %d this entry point tracks", dev,
                        kMaxDevices);
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (g_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
      return noalloc_fail(XC_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return XC_OK;
}

}  // namespace

extern "C" int xc_loopcape_ex_noalloc(int grid, const void *p, const void *t3d, const void *td3d,
                                      const void *ps, const void *ts, const void *tds,
                                      int dtype, float pinc, int source, float ml_depth,
                                      int adiabat, const int *start_3d, int nk, int n2, int guess,
                                      float *cape, float *cin, int *mulvl, float *z_out,
                                      int *status, long long *counters, void *stream) {
  if (n2 > XC_NOALLOC_MAX_COLUMNS)
    return noalloc_fail(XC_ERR_INVALID,
                        "xc_loopcape_ex_noalloc takes at most %d columns (got %d): split the "
                        "batch or use xc_loopcape_ex with a workspace",
                        XC_NOALLOC_MAX_COLUMNS, n2);
  if (n2 > 0 && xc::order_workspace_bytes(n2) > kNoallocScratchBytes)
    return noalloc_fail(XC_ERR_INVALID, "ordering scratch for %d columns exceeds the static array",
                        n2);
  void *scratch = nullptr;
  if (n2 > 0) {
    const int rc = scratch_address(&scratch);
    if (rc != XC_OK) return rc;
  }
  return xc_loopcape_ex(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, source, ml_depth, adiabat,
                        start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, counters,
                        scratch, scratch ? kNoallocScratchBytes : 0, stream);
}
