// cape_diag.cu -- the CAPE/CIN lift with the diagnostics getcape computes
// and discards (LFC and EL pressure and height, source height and theta-e;
// cape_column.cuh, getcape_col), for the plain and the learned solvers.  A
// separate translation unit: the lift kernels of cape_kernel.cu carry none
// of the bookkeeping.
#include "cape_column.cuh"
#include "xc_kernels.h"

namespace xc {

template <typename T, int GRID, bool ICE, bool PSEUDO, int SOLVER>
__global__ void __launch_bounds__(128) cape_diag_kernel(CapeArgs a) {
  extern __shared__ __align__(16) float guess_sm[];  // packed guess network, SOLVE_LEARNED
  const float *gw = nullptr;
  if (SOLVER == SOLVE_LEARNED) {
    for (int k = threadIdx.x; k < GUESS_NPARAM; k += blockDim.x)
      guess_sm[k] = guess_packed_value(a.guess_w, k);
    __syncthreads();
    gw = guess_sm;
  }
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n2) {
    int nsub = 0, niter = 0;
    cape_column_run<T, GRID, ICE, PSEUDO, SOLVER, true>(a, i, nsub, niter, gw);
  }
}

template <typename T, int GRID, int SOLVER>
static void launch_diag_s(const CapeArgs &a, unsigned blocks, cudaStream_t s) {
  const bool ice = a.adiabat >= 3, pseudo = (a.adiabat == 1 || a.adiabat == 3);
  const size_t sm = SOLVER == SOLVE_LEARNED ? sizeof(float) * GUESS_NPARAM : 0;
  if (ice && pseudo) cape_diag_kernel<T, GRID, true, true, SOLVER><<<blocks, 128, sm, s>>>(a);
  else if (ice) cape_diag_kernel<T, GRID, true, false, SOLVER><<<blocks, 128, sm, s>>>(a);
  else if (pseudo) cape_diag_kernel<T, GRID, false, true, SOLVER><<<blocks, 128, sm, s>>>(a);
  else cape_diag_kernel<T, GRID, false, false, SOLVER><<<blocks, 128, sm, s>>>(a);
}

template <typename T, int GRID>
static void launch_diag_t(const CapeArgs &a, unsigned blocks, cudaStream_t s) {
  if (a.guess == 1) launch_diag_s<T, GRID, SOLVE_LEARNED>(a, blocks, s);
  else launch_diag_s<T, GRID, SOLVE_PLAIN>(a, blocks, s);
}

cudaError_t launch_cape_diag(const CapeArgs &a, cudaStream_t s) {
  const unsigned blocks = (unsigned)((a.n2 + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  if (a.dtype == 0) {
    if (a.grid == 1) launch_diag_t<float, 1>(a, blocks, s);
    else if (a.grid == 2) launch_diag_t<float, 2>(a, blocks, s);
    else launch_diag_t<float, 3>(a, blocks, s);
  } else {
    if (a.grid == 1) launch_diag_t<double, 1>(a, blocks, s);
    else if (a.grid == 2) launch_diag_t<double, 2>(a, blocks, s);
    else launch_diag_t<double, 3>(a, blocks, s);
  }
  return cudaGetLastError();
}

}  // namespace xc
