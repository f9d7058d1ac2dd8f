// cape_srh.cu -- calc_cape and calc_srh of the same columns in one kernel for
// sm_103a.
//
// A caller that wants both (the reference computes them with separate f2py
// chains over the same p, t, td: src/xcape/core.py:261-332 and :473-542)
// gets them from one launch: thread t lifts column perm[t] (cape_column_run,
// or learned_column for the learned solver) and then runs column t through
// the SRH chain (srh_column_run).  The lift is FP32 work and the SRH chain's
// height and helicity stages are FP64 work at the reference precision, so
// warps in one phase keep the FP32 pipes busy while warps in the other keep
// the FP64 pipe busy: with the reference precision the launch takes about
// as long as the SRH kernel alone.  The SRH walk takes the columns in their
// natural order, whose rows neighbouring lanes share; following the lift's
// order instead re-read 1.5x the bytes (the lift's lines have left L2 by
// the time its SRH walk starts).  The two results are those of the separate
// kernels: the SRH routines round every product on their own
// (srh_column.cuh, nc_mul), and the lift is the same column code with the
// same solver.
#include <stdint.h>

#include "cape_column.cuh"
#include "cape_learned.cuh"
#include "srh_column.cuh"
#include "xc_kernels.h"

namespace xc {

template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(128) cape_srh_plain_kernel(CapeArgs a, SrhArgs s) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= a.n2) return;
  const long long i = a.perm ? (long long)__ldg(a.perm + t) : t;
  int nsub = 0, niter = 0;
  cape_column_run<T, GRID, ICE, PSEUDO, SOLVE_PLAIN>(a, i, nsub, niter);
  if (s.precision == 1) srh_column_run<T, GRID, true>(s, t);
  else srh_column_run<T, GRID, false>(s, t);
}

template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(LEARNED_THREADS, 7)
    cape_srh_learned_kernel(CapeArgs a, SrhArgs s, const WarpNetSmem *img) {
  __shared__ WarpNetSmem net;
  __shared__ LearnedPrep prep[LEARNED_THREADS];
  copy_warp_net(net, img);
  __syncthreads();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nsub, niter;
  learned_column<T, GRID, ICE, PSEUDO>(a, net, prep, t, nsub, niter);
  if (t >= a.n2) return;
  if (s.precision == 1) srh_column_run<T, GRID, true>(s, t);
  else srh_column_run<T, GRID, false>(s, t);
}

template <typename T, int GRID>
static cudaError_t launch_cape_srh_t(const CapeArgs &a, const SrhArgs &s, cudaStream_t st) {
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  const unsigned blocks = (unsigned)((a.n2 + LEARNED_THREADS - 1) / LEARNED_THREADS);
  if (a.guess == 1) {
    const void *img = nullptr;
    const cudaError_t e = warp_net_image(&img);
    if (e != cudaSuccess) return e;
    const WarpNetSmem *w = (const WarpNetSmem *)img;
    if (ice && pseudo) cape_srh_learned_kernel<T, GRID, true, true><<<blocks, LEARNED_THREADS, 0, st>>>(a, s, w);
    else if (ice) cape_srh_learned_kernel<T, GRID, true, false><<<blocks, LEARNED_THREADS, 0, st>>>(a, s, w);
    else if (pseudo) cape_srh_learned_kernel<T, GRID, false, true><<<blocks, LEARNED_THREADS, 0, st>>>(a, s, w);
    else cape_srh_learned_kernel<T, GRID, false, false><<<blocks, LEARNED_THREADS, 0, st>>>(a, s, w);
  } else {
    if (ice && pseudo) cape_srh_plain_kernel<T, GRID, true, true><<<blocks, 128, 0, st>>>(a, s);
    else if (ice) cape_srh_plain_kernel<T, GRID, true, false><<<blocks, 128, 0, st>>>(a, s);
    else if (pseudo) cape_srh_plain_kernel<T, GRID, false, true><<<blocks, 128, 0, st>>>(a, s);
    else cape_srh_plain_kernel<T, GRID, false, false><<<blocks, 128, 0, st>>>(a, s);
  }
  return cudaGetLastError();
}

cudaError_t launch_cape_srh(const CapeArgs &a, const SrhArgs &s, cudaStream_t st) {
  if (a.n2 == 0) return cudaSuccess;
  if (a.dtype == 0)
    return a.grid == 1 ? launch_cape_srh_t<float, 1>(a, s, st) : launch_cape_srh_t<float, 2>(a, s, st);
  return a.grid == 1 ? launch_cape_srh_t<double, 1>(a, s, st) : launch_cape_srh_t<double, 2>(a, s, st);
}

}  // namespace xc
