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
//   columns (about 6.1 MiB).  It is created on a device when CUDA loads this
//   file's module there: at the first look-up of its address under lazy
//   module loading (CUDA_MODULE_LOADING=LAZY, the default), or when the
//   library's modules are loaded otherwise.  From then on the device holds
//   it until the context is destroyed (process exit or cudaDeviceReset).
//   A call with n2 == 0 performs only that look-up, so a caller can make the
//   one allocation CUDA does for the array at start-up, before any stream
//   capture.
// * Host code cannot use the array's name as a device address.  Every call
//   looks the address up with cudaGetSymbolAddress on the current device
//   (cheap once the module is loaded), so a context that was reset and
//   re-created, which may place the array elsewhere, gets the new address.
// * All calls share the one array, and it keeps the last call's contents.
//   The bucket counters that must start at zero are cleared at every call.
//   Calls that overlap on the GPU (on different streams, or from several host
//   threads without ordering) race on the array: issue them one after the
//   other.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>

#include "../../include/xcape_gb300.h"
#include "xc_kernels.h"

namespace {

// 64 KiB of bucket counters + a 16-bit bucket + a 32-bit permutation entry
// per column, each part rounded up to 256 bytes.
constexpr size_t kNoallocScratchBytes =
    65536 + 2 * (size_t)XC_NOALLOC_MAX_COLUMNS + 4 * (size_t)XC_NOALLOC_MAX_COLUMNS + 512;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

// Formats the message into xc_last_error() and returns code.
int noalloc_fail(int code, const char *fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  return xc::set_error(code, msg);
}

// Device address of g_noalloc_scratch on the current device, looked up on
// every call (loading this module on the device at the first one).
int scratch_address(void **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return noalloc_fail(XC_ERR_CUDA, "cudaGetSymbolAddress of the static scratch: %s",
                        cudaGetErrorString(e));
  }
  *out = p;
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
  if (n2 < 0) return noalloc_fail(XC_ERR_INVALID, "n2=%d is negative", n2);
  // Also for n2 == 0: an empty call performs the set-up (the module load
  // that creates the array on this device) and nothing else.
  void *scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != XC_OK) return rc;
  if (n2 == 0) return XC_OK;
  return xc_loopcape_ex(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, source, ml_depth, adiabat,
                        start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, counters,
                        scratch, kNoallocScratchBytes, stream);
}
