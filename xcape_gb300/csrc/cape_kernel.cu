// cape_kernel.cu -- CAPE/CIN kernels for sm_103a: one thread per column,
// running getcape_col (cape_column.cuh).
#include "cape_column.cuh"
#include "xc_kernels.h"

namespace xc {

template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(128) cape_kernel(CapeArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nsub = 0, niter = 0;
  if (i < a.n2) cape_column_run<T, GRID, ICE, PSEUDO>(a, i, nsub, niter);
  if (a.counters) {
    // Work accounting: warp-reduce, one atomic per warp.
    long long s = nsub, it = niter;
    for (int o = 16; o > 0; o >>= 1) {
      s += __shfl_down_sync(0xffffffffu, s, o);
      it += __shfl_down_sync(0xffffffffu, it, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd((unsigned long long *)&a.counters[0], (unsigned long long)s);
      atomicAdd((unsigned long long *)&a.counters[1], (unsigned long long)it);
    }
  }
}

template <typename T>
__global__ void pres_lev_pos_kernel(const T *p1d, const T *ps, int nk, long long n2, int *start) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2) start[i] = pres_lev_pos_col<T>(p1d, __ldg(ps + i), nk);
}

// ---- launchers ---------------------------------------------------------------
template <typename T, int GRID>
static cudaError_t launch_cape_t(const CapeArgs &a, cudaStream_t s) {
  const int threads = 128;
  const unsigned blocks = (unsigned)((a.n2 + threads - 1) / threads);
  if (blocks == 0) return cudaSuccess;
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  if (ice && pseudo)
    cape_kernel<T, GRID, true, true><<<blocks, threads, 0, s>>>(a);
  else if (ice)
    cape_kernel<T, GRID, true, false><<<blocks, threads, 0, s>>>(a);
  else if (pseudo)
    cape_kernel<T, GRID, false, true><<<blocks, threads, 0, s>>>(a);
  else
    cape_kernel<T, GRID, false, false><<<blocks, threads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cape(const CapeArgs &a, cudaStream_t s) {
  if (a.dtype == 0) {
    switch (a.grid) {
      case 1: return launch_cape_t<float, 1>(a, s);
      case 2: return launch_cape_t<float, 2>(a, s);
      default: return launch_cape_t<float, 3>(a, s);
    }
  } else {
    switch (a.grid) {
      case 1: return launch_cape_t<double, 1>(a, s);
      case 2: return launch_cape_t<double, 2>(a, s);
      default: return launch_cape_t<double, 3>(a, s);
    }
  }
}

cudaError_t launch_pres_lev_pos(const void *p1d, const void *ps, int dtype, int nk, long long n2,
                                int *start, cudaStream_t s) {
  const int threads = 256;
  const unsigned blocks = (unsigned)((n2 + threads - 1) / threads);
  if (blocks == 0) return cudaSuccess;
  if (dtype == 0)
    pres_lev_pos_kernel<float><<<blocks, threads, 0, s>>>((const float *)p1d, (const float *)ps,
                                                          nk, n2, start);
  else
    pres_lev_pos_kernel<double><<<blocks, threads, 0, s>>>((const double *)p1d,
                                                           (const double *)ps, nk, n2, start);
  return cudaGetLastError();
}

}  // namespace xc
