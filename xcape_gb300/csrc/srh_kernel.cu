// srh_kernel.cu -- storm-relative helicity kernels for sm_103a: one thread per
// column running the column routines of srh_column.cuh (the fused
// stdheight -> Bunkers -> SREH path and the three stage loops on their own).
#include <stdint.h>

#include "srh_column.cuh"
#include "xc_kernels.h"

namespace xc {

template <typename T, int GRID, bool F32>
__global__ void __launch_bounds__(128) srh_fused_kernel(SrhArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n2) srh_column_run<T, GRID, F32>(a, i);
}

__global__ void stdheight_kernel(const double *P, long long p_stride, const double *T,
                                 const double *Td, const double *Ps, const double *Ts,
                                 const double *Tds, const double *Hin, const int *start, int NK,
                                 long long NX, double *H, double *Hs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NX) stdheight_column_run(P, p_stride, T, Td, Ps, Ts, Tds, Hin, start, NK, i, H, Hs);
}

__global__ void bunkers_kernel(const float *U, const float *V, const float *Z, const float *Us,
                               const float *Vs, const float *Zs, const int *start, int nk,
                               long long n2, float *RM, float *LM, float *Mean) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2) bunkers_column_run(U, V, Z, Us, Vs, Zs, start, nk, i, RM, LM, Mean);
}

__global__ void sreh_kernel(const double *u, const double *v, const double *aglh,
                            const double *us, const double *vs, const double *aglhs,
                            const double *cu_rm, const double *cv_rm, const double *cu_lm,
                            const double *cv_lm, double top, const int *start, int nk,
                            long long n2, double *sreh_rm, double *sreh_lm) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2)
    sreh_column_run(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top, start, nk, i,
                    sreh_rm, sreh_lm);
}

static unsigned blocks_for(long long n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

template <bool F32>
static void launch_srh_p(const SrhArgs &a, unsigned blocks, cudaStream_t s) {
  if (a.dtype == 0) {
    if (a.grid == 1)
      srh_fused_kernel<float, 1, F32><<<blocks, 128, 0, s>>>(a);
    else
      srh_fused_kernel<float, 2, F32><<<blocks, 128, 0, s>>>(a);
  } else {
    if (a.grid == 1)
      srh_fused_kernel<double, 1, F32><<<blocks, 128, 0, s>>>(a);
    else
      srh_fused_kernel<double, 2, F32><<<blocks, 128, 0, s>>>(a);
  }
}

cudaError_t launch_srh(const SrhArgs &a, cudaStream_t s) {
  const unsigned blocks = blocks_for(a.n2, 128);
  if (blocks == 0) return cudaSuccess;
  if (a.precision == 1 && a.dtype == 0 && srh_seg_run(a.nk) > 0)
    return launch_srh_seg(a, s);  // srh_seg.cu
  if (a.precision == 1)
    launch_srh_p<true>(a, blocks, s);
  else
    launch_srh_p<false>(a, blocks, s);
  return cudaGetLastError();
}

cudaError_t launch_stdheight(const double *P, long long p_stride, const double *T,
                             const double *Td, const double *Ps, const double *Ts,
                             const double *Tds, const double *Hin, const int *start, int NK,
                             long long NX, double *H, double *Hs, cudaStream_t s) {
  const unsigned blocks = blocks_for(NX, 128);
  if (blocks == 0) return cudaSuccess;
  stdheight_kernel<<<blocks, 128, 0, s>>>(P, p_stride, T, Td, Ps, Ts, Tds, Hin, start, NK, NX,
                                          H, Hs);
  return cudaGetLastError();
}

cudaError_t launch_bunkers(const float *U, const float *V, const float *Z, const float *Us,
                           const float *Vs, const float *Zs, const int *start, int nk,
                           long long n2, float *RM, float *LM, float *Mean, cudaStream_t s) {
  const unsigned blocks = blocks_for(n2, 128);
  if (blocks == 0) return cudaSuccess;
  bunkers_kernel<<<blocks, 128, 0, s>>>(U, V, Z, Us, Vs, Zs, start, nk, n2, RM, LM, Mean);
  return cudaGetLastError();
}

cudaError_t launch_sreh(const double *u, const double *v, const double *aglh, const double *us,
                        const double *vs, const double *aglhs, const double *cu_rm,
                        const double *cv_rm, const double *cu_lm, const double *cv_lm,
                        double top, const int *start, int nk, long long n2, double *sreh_rm,
                        double *sreh_lm, cudaStream_t s) {
  const unsigned blocks = blocks_for(n2, 128);
  if (blocks == 0) return cudaSuccess;
  sreh_kernel<<<blocks, 128, 0, s>>>(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top,
                                     start, nk, n2, sreh_rm, sreh_lm);
  return cudaGetLastError();
}

}  // namespace xc
