// cape_retry.cu -- the FP64 retry of the CAPE lift (XC_RETRY_FP64).
//
// The reference gives a column up after 100 iterations of its damped
// fixed point and returns CAPE = CIN = 0 (CAPE_CODE_model_lev.f90:464-474).
// In FP32 that happens on 1-3 % of warm, noisy columns: the 0.3-damped
// iteration locks into a two-value cycle one ulp wide whose step stays above
// the 2e-4 K test.  In FP64 the same iteration converges there.  The retry
// re-lifts exactly the columns the FP32 lift flagged XC_COL_NOCONV, in double
// precision with the reference's plain solver (cape_column_run with
// R = double), and overwrites their outputs; it is a second, cold kernel, so
// the hot FP32 kernels carry none of it.
//
// * retry_list_kernel compacts the flagged columns into a list (atomic
//   counter, order irrelevant: each column is still computed by one thread
//   and written to its own index), so that the FP64 lifts run in full warps;
// * cape_retry64_kernel lifts the listed columns (or, without a list, scans
//   every column's status) with a grid-stride loop, since the host does not
//   know how many were flagged.
// A retried column gets XC_COL_FP64 in its status; XC_COL_NOCONV stays set
// only if the FP64 iteration gave up as well.
#include <cuda_runtime.h>

#include "cape_column.cuh"
#include "xc_kernels.h"

namespace xc {

constexpr int COL_FP64 = 8;  // mirrors XC_COL_FP64

__global__ void retry_list_kernel(const int *status, long long n2, int *list, unsigned *count) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2 && (status[i] & COL_NOCONV)) list[atomicAdd(count, 1u)] = (int)i;
}

template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(128) cape_retry64_kernel(CapeArgs a, const int *list,
                                                           const unsigned *count) {
  const long long n = list ? (long long)*count : a.n2;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += stride) {
    const long long i = list ? (long long)list[t] : t;
    if (!list && !(a.status[i] & COL_NOCONV)) continue;
    int nsub = 0, niter = 0;
    cape_column_run<T, GRID, ICE, PSEUDO, SOLVE_PLAIN, false, double>(a, i, nsub, niter);
    a.status[i] |= COL_FP64;
  }
}

template <typename T, int GRID>
static void launch_retry_t(const CapeArgs &a, const int *list, const unsigned *count,
                           unsigned blocks, cudaStream_t s) {
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  if (ice && pseudo) cape_retry64_kernel<T, GRID, true, true><<<blocks, 128, 0, s>>>(a, list, count);
  else if (ice) cape_retry64_kernel<T, GRID, true, false><<<blocks, 128, 0, s>>>(a, list, count);
  else if (pseudo) cape_retry64_kernel<T, GRID, false, true><<<blocks, 128, 0, s>>>(a, list, count);
  else cape_retry64_kernel<T, GRID, false, false><<<blocks, 128, 0, s>>>(a, list, count);
}

cudaError_t launch_retry64(const CapeArgs &a, void *ws, cudaStream_t s) {
  if (a.n2 <= 0) return cudaSuccess;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const long long need = (a.n2 + 127) / 128;
  const unsigned blocks = (unsigned)(need < 4LL * sms ? need : 4LL * sms);
  const int *list = nullptr;
  const unsigned *count = nullptr;
  if (ws) {
    // the ordering workspace is free once the lift has run (same stream):
    // its first counter becomes the list's length, its permutation the list
    unsigned *cnt = nullptr;
    int *lst = nullptr;
    order_workspace_parts(ws, a.n2, &cnt, &lst);
    e = cudaMemsetAsync(cnt, 0, sizeof(unsigned), s);
    if (e != cudaSuccess) return e;
    retry_list_kernel<<<(unsigned)((a.n2 + 255) / 256), 256, 0, s>>>(a.status, a.n2, lst, cnt);
    list = lst;
    count = cnt;
  }
  if (a.dtype == 0) {
    if (a.grid == 1) launch_retry_t<float, 1>(a, list, count, blocks, s);
    else if (a.grid == 2) launch_retry_t<float, 2>(a, list, count, blocks, s);
    else launch_retry_t<float, 3>(a, list, count, blocks, s);
  } else {
    if (a.grid == 1) launch_retry_t<double, 1>(a, list, count, blocks, s);
    else if (a.grid == 2) launch_retry_t<double, 2>(a, list, count, blocks, s);
    else launch_retry_t<double, 3>(a, list, count, blocks, s);
  }
  return cudaGetLastError();
}

}  // namespace xc
