// pipe_peaks.cu -- xc_measure_pipe_peaks: the FP32 and XU (MUFU) issue rates
// of the current device, measured with two short kernels of known
// instruction mix.  They are the denominators of the CAPE lift's compute
// roofline: the lift is bound by FP32 and transcendental work, not by HBM.
//
// * fp32_chain_kernel: every thread advances 8 independent chains of fused
//   multiply-adds (x = x * a + b), so the FMA pipe is never starved by
//   dependences; one FFMA is one FP32 lane operation.
// * xu_chain_kernel: every thread advances 8 independent chains of
//   ex2.approx (x = 2^-x, which stays in (0, 1]); one ex2.approx is one XU
//   lane operation (rcp.approx and lg2.approx run on the same unit).
// Both launch 8 blocks of 256 threads per SM, time themselves with CUDA
// events on the caller's stream after one warm-up launch, and keep their
// results live through a store that depends on every chain.
#include <cuda_runtime.h>

#include "../../include/xcape_gb300.h"
#include "xc_kernels.h"

namespace xc {
namespace {

constexpr int kChains = 8;
constexpr int kThreads = 256;
constexpr int kBlocksPerSm = 8;

// the kernels' store target (never written: see the kernels)
__device__ float g_sink[1];

__global__ void __launch_bounds__(kThreads) fp32_chain_kernel(float *sink, int iters, float a,
                                                              float b) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u)
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = fmaf(x[c], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678f) sink[0] = s;  // never true; keeps the chains live
}

__device__ __forceinline__ float ex2_neg(float x) {
  float y;
  asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(-x));
  return y;
}

__global__ void __launch_bounds__(kThreads) xu_chain_kernel(float *sink, int iters) {
  float x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int c = 0; c < kChains; ++c) x[c] = ex2_neg(x[c]);
  }
  float s = 0.0f;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == 12345.678f) sink[0] = s;
}

}  // namespace
}  // namespace xc

extern "C" int xc_measure_pipe_peaks(double *fp32_gops, double *xu_gops, void *stream) {
  if (!fp32_gops || !xu_gops) return xc::set_error(XC_ERR_INVALID, "NULL output");
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return xc::set_error(XC_ERR_CUDA, cudaGetErrorString(e));
  const unsigned blocks = (unsigned)(sms * xc::kBlocksPerSm);
  const double threads = (double)blocks * xc::kThreads;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  e = cudaEventCreate(&ev[0]);
  if (e == cudaSuccess) e = cudaEventCreate(&ev[1]);
  float *sink_ptr = nullptr;
  if (e == cudaSuccess) e = cudaGetSymbolAddress((void **)&sink_ptr, xc::g_sink);
  const int fp32_iters = 4096, xu_iters = 1024;
  float ms[2] = {0.0f, 0.0f};
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {  // warm-up, then timed
      if (rep == 1) e = cudaEventRecord(ev[0], s);
      if (k == 0)
        xc::fp32_chain_kernel<<<blocks, xc::kThreads, 0, s>>>(sink_ptr, fp32_iters, 0.999f, 1e-4f);
      else
        xc::xu_chain_kernel<<<blocks, xc::kThreads, 0, s>>>(sink_ptr, xu_iters);
      if (e == cudaSuccess) e = cudaGetLastError();
      if (rep == 1 && e == cudaSuccess) e = cudaEventRecord(ev[1], s);
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[1]);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms[k], ev[0], ev[1]);
  }
  for (int k = 0; k < 2; ++k)
    if (ev[k]) cudaEventDestroy(ev[k]);
  if (e != cudaSuccess) return xc::set_error(XC_ERR_CUDA, cudaGetErrorString(e));
  const double fp32_ops = threads * fp32_iters * 16.0 * xc::kChains;
  const double xu_ops = threads * xu_iters * 4.0 * xc::kChains;
  *fp32_gops = fp32_ops / (ms[0] * 1e-3) / 1e9;
  *xu_gops = xu_ops / (ms[1] * 1e-3) / 1e9;
  return XC_OK;
}
