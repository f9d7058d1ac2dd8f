// cape_kernel.cu -- CAPE/CIN kernels for sm_103a: one thread per column,
// running getcape_col (cape_column.cuh).
#include <cuda_bf16.h>
#include <stddef.h>
#include <stdint.h>

#include "cape_column.cuh"
#include "cape_learned.cuh"
#include "xc_kernels.h"

namespace xc {

// One thread per column.  The learned solver runs in cape_learned_kernel
// (below), which evaluates its guess network per warp on the tensor cores.
template <typename T, int GRID, bool ICE, bool PSEUDO, int SOLVER>
__global__ void __launch_bounds__(128) cape_kernel(CapeArgs a) {
  extern __shared__ __align__(16) float guess_sm[];  // packed guess network, SOLVE_LEARNED_ALL
  const float *gw = nullptr;
  if (SOLVER == SOLVE_LEARNED_ALL) {
    for (int k = threadIdx.x; k < GUESS_NPARAM; k += blockDim.x)
      guess_sm[k] = guess_packed_value(a.guess_w, k);
    __syncthreads();
    gw = guess_sm;
  }
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int nsub = 0, niter = 0;
  if (t < a.n2) {
    const long long i = a.perm ? (long long)__ldg(a.perm + t) : t;
    cape_column_run<T, GRID, ICE, PSEUDO, SOLVER>(a, i, nsub, niter, gw);
  }
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

// The shared-memory image of the guess network on this device, built from
// the parameters once per xc_guess_set_weights (build_warp_net), so that a
// block of the learned kernel copies 9.7 KB with 16-byte loads instead of
// converting and swizzling W2 from FP32 parameters.
__device__ WarpNetSmem g_warp_net;

__global__ void build_warp_net_kernel(const float *w) { load_warp_net(g_warp_net, w); }

cudaError_t build_warp_net(const float *w, cudaStream_t s) {
  build_warp_net_kernel<<<1, 256, 0, s>>>(w);
  return cudaGetLastError();
}

cudaError_t warp_net_image(const void **out) {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_warp_net);
  *out = p;
  return e;
}

// The learned solver (cape_learned.cuh): 7 resident blocks of 128 threads per SM.
template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(LEARNED_THREADS, 7) cape_learned_kernel(CapeArgs a) {
  __shared__ WarpNetSmem net;
  __shared__ LearnedPrep prep[LEARNED_THREADS];
  copy_warp_net(net, &g_warp_net);
  __syncthreads();
  int nsub, niter;
  learned_column<T, GRID, ICE, PSEUDO>(a, net, prep, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                                       nsub, niter);
  if (a.counters) {
    long long sb = nsub, it = niter;
    for (int o = 16; o > 0; o >>= 1) {
      sb += __shfl_down_sync(0xffffffffu, sb, o);
      it += __shfl_down_sync(0xffffffffu, it, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd((unsigned long long *)&a.counters[0], (unsigned long long)sb);
      atomicAdd((unsigned long long *)&a.counters[1], (unsigned long long)it);
    }
  }
}

// SOLVE_LEARNED_WARP (cape_learned.cuh): the network evaluated by each warp
// at every sub-step, in lockstep.
template <typename T, int GRID, bool ICE, bool PSEUDO>
__global__ void __launch_bounds__(LEARNED_THREADS) cape_learned_warp_kernel(CapeArgs a) {
  __shared__ WarpNetSmem net;
  copy_warp_net(net, &g_warp_net);
  __syncthreads();
  int nsub, niter;
  learned_warp_column<T, GRID, ICE, PSEUDO>(a, net, (long long)blockIdx.x * blockDim.x + threadIdx.x,
                                            nsub, niter);
  if (a.counters) {
    long long sb = nsub, it = niter;
    for (int o = 16; o > 0; o >>= 1) {
      sb += __shfl_down_sync(0xffffffffu, sb, o);
      it += __shfl_down_sync(0xffffffffu, it, o);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd((unsigned long long *)&a.counters[0], (unsigned long long)sb);
      atomicAdd((unsigned long long *)&a.counters[1], (unsigned long long)it);
    }
  }
}

template <typename T>
__global__ void pres_lev_pos_kernel(const T *p1d, const T *ps, int nk, long long n2, int *start) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2) start[i] = pres_lev_pos_col<T>(p1d, __ldg(ps + i), nk);
}

// ---- column ordering ---------------------------------------------------------
// Warps run in lockstep, so a warp pays for its slowest column at every
// sub-step and for its tallest column at the end.  Sorting the columns by
// (start level, surface dewpoint) groups columns with equal level counts and
// similar moisture -- hence similar iteration counts -- into the same warp.
// The sort is a counting sort over ORDER_BUCKETS buckets; order inside a
// bucket is whatever the atomics give, which changes no result (each column
// is still computed by one thread and written to its own index).

template <typename T, int GRID>
__device__ __forceinline__ int order_bucket(const CapeArgs &a, long long i) {
  int start = 1;
  if (GRID != 1)
    start = a.start ? __ldg(a.start + i)
                    : pres_lev_pos_col<T>((const T *)a.p, __ldg((const T *)a.ps + i), a.nk);
  start = start < 0 ? 0 : (start > ORDER_START_CAP ? ORDER_START_CAP : start);
  const float tds = ldf((const T *)a.tds + i);
  int bin = ORDER_TD_BINS - 1;  // NaN dewpoints share the last bin
  if (tds == tds) {
    const float x = (tds + 40.0f) * (ORDER_TD_BINS / 80.0f);
    bin = x <= 0.0f ? 0 : (x >= (float)(ORDER_TD_BINS - 1) ? ORDER_TD_BINS - 1 : (int)x);
  }
  return start * ORDER_TD_BINS + bin;
}

// Neighbouring columns mostly fall in the same bucket, so the lanes of a warp
// that share one add their count with a single atomic (warp-aggregated); the
// blocks are whole warps, and lanes past n2 take part with bucket -1.
template <typename T, int GRID>
__global__ void order_bucket_kernel(CapeArgs a, unsigned short *bucket, unsigned *hist) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < a.n2;
  const int b = in ? order_bucket<T, GRID>(a, i) : -1;
  if (in) bucket[i] = (unsigned short)b;
  const unsigned same = __match_any_sync(0xffffffffu, b);
  if (in && (threadIdx.x & 31) == __ffs(same) - 1) atomicAdd(hist + b, (unsigned)__popc(same));
}

// Exclusive scan of the ORDER_BUCKETS counters in place, by one block of
// ORDER_SCAN_THREADS threads: small enough to start in the slot that one
// retiring lift block frees on an SM (the host path orders a chunk while
// the lifts of earlier chunks fill the GPU).  Each thread sums its
// consecutive counters, the block scans the sums, and each thread writes
// its counters' prefixes, 16 bytes at a time.
constexpr int ORDER_SCAN_THREADS = 128;
__global__ void __launch_bounds__(ORDER_SCAN_THREADS) order_scan_kernel(unsigned *hist) {
  constexpr int PER = ORDER_BUCKETS / ORDER_SCAN_THREADS;
  static_assert(PER % 4 == 0, "whole 16-byte accesses per thread");
  __shared__ unsigned warp_tot[ORDER_SCAN_THREADS / 32];
  const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  uint4 *h4 = reinterpret_cast<uint4 *>(hist + tid * PER);
  unsigned sum = 0;
  for (int j = 0; j < PER / 4; ++j) {
    const uint4 q = h4[j];
    sum += q.x + q.y + q.z + q.w;
  }
  // inclusive scan of `sum` across the block
  unsigned x = sum;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[w] = x;
  __syncthreads();
  unsigned run = x - sum;
  for (int v = 0; v < w; ++v) run += warp_tot[v];
  for (int j = 0; j < PER / 4; ++j) {
    const uint4 q = h4[j];
    uint4 r;
    r.x = run;
    r.y = r.x + q.x;
    r.z = r.y + q.y;
    r.w = r.z + q.z;
    run = r.w + q.w;
    h4[j] = r;
  }
}

// Lanes that share a bucket take consecutive places in it, in lane order,
// from one atomic of their first lane.
__global__ void order_scatter_kernel(const unsigned short *bucket, unsigned *offs, int *perm,
                                     long long n2) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = i < n2;
  const int b = in ? (int)bucket[i] : -1;
  const unsigned same = __match_any_sync(0xffffffffu, b);
  const int lane = threadIdx.x & 31, first = __ffs(same) - 1;
  unsigned base = 0;
  if (in && lane == first) base = atomicAdd(offs + b, (unsigned)__popc(same));
  base = __shfl_sync(0xffffffffu, base, first);
  if (in) perm[base + __popc(same & ((1u << lane) - 1u))] = (int)i;
}

static size_t round256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t order_workspace_bytes(long long n2) {
  return round256(sizeof(unsigned) * ORDER_BUCKETS) + round256(sizeof(unsigned short) * n2) +
         round256(sizeof(int) * n2);
}

template <typename T, int GRID>
static void launch_bucket(const CapeArgs &a, unsigned short *bucket, unsigned *hist,
                          unsigned blocks, cudaStream_t s) {
  order_bucket_kernel<T, GRID><<<blocks, 256, 0, s>>>(a, bucket, hist);
}

void order_workspace_parts(void *ws, long long n2, unsigned **hist, int **perm) {
  char *b = (char *)ws;
  *hist = (unsigned *)b;
  *perm = (int *)(b + round256(sizeof(unsigned) * ORDER_BUCKETS) +
                  round256(sizeof(unsigned short) * n2));
}

cudaError_t launch_order(const CapeArgs &a, void *ws, const int **perm, cudaStream_t s) {
  char *b = (char *)ws;
  unsigned *hist = nullptr;
  int *pm = nullptr;
  order_workspace_parts(ws, a.n2, &hist, &pm);
  unsigned short *bucket = (unsigned short *)(b + round256(sizeof(unsigned) * ORDER_BUCKETS));
  *perm = pm;
  if (a.n2 <= 0) return cudaSuccess;
  // the scan reads and writes the counters 16 bytes at a time
  if (((uintptr_t)ws & 15) != 0) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(hist, 0, sizeof(unsigned) * ORDER_BUCKETS, s);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((a.n2 + 255) / 256);
  if (a.dtype == 0) {
    if (a.grid == 1) launch_bucket<float, 1>(a, bucket, hist, blocks, s);
    else if (a.grid == 2) launch_bucket<float, 2>(a, bucket, hist, blocks, s);
    else launch_bucket<float, 3>(a, bucket, hist, blocks, s);
  } else {
    if (a.grid == 1) launch_bucket<double, 1>(a, bucket, hist, blocks, s);
    else if (a.grid == 2) launch_bucket<double, 2>(a, bucket, hist, blocks, s);
    else launch_bucket<double, 3>(a, bucket, hist, blocks, s);
  }
  order_scan_kernel<<<1, ORDER_SCAN_THREADS, 0, s>>>(hist);
  order_scatter_kernel<<<blocks, 256, 0, s>>>(bucket, hist, pm, a.n2);
  return cudaGetLastError();
}

// ---- launchers ---------------------------------------------------------------
template <typename T, int GRID, int SOLVER>
static void launch_cape_s(const CapeArgs &a, unsigned blocks, int threads, cudaStream_t s) {
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  const size_t sm = SOLVER == SOLVE_LEARNED_ALL ? sizeof(float) * GUESS_NPARAM : 0;
  if (ice && pseudo)
    cape_kernel<T, GRID, true, true, SOLVER><<<blocks, threads, sm, s>>>(a);
  else if (ice)
    cape_kernel<T, GRID, true, false, SOLVER><<<blocks, threads, sm, s>>>(a);
  else if (pseudo)
    cape_kernel<T, GRID, false, true, SOLVER><<<blocks, threads, sm, s>>>(a);
  else
    cape_kernel<T, GRID, false, false, SOLVER><<<blocks, threads, sm, s>>>(a);
}

template <typename T, int GRID>
static void launch_learned(const CapeArgs &a, cudaStream_t s) {
  const int threads = LEARNED_THREADS;
  const unsigned blocks = (unsigned)((a.n2 + threads - 1) / threads);
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  if (ice && pseudo) cape_learned_kernel<T, GRID, true, true><<<blocks, threads, 0, s>>>(a);
  else if (ice) cape_learned_kernel<T, GRID, true, false><<<blocks, threads, 0, s>>>(a);
  else if (pseudo) cape_learned_kernel<T, GRID, false, true><<<blocks, threads, 0, s>>>(a);
  else cape_learned_kernel<T, GRID, false, false><<<blocks, threads, 0, s>>>(a);
}

template <typename T, int GRID>
static void launch_learned_warp(const CapeArgs &a, cudaStream_t s) {
  const int threads = LEARNED_THREADS;
  const unsigned blocks = (unsigned)((a.n2 + threads - 1) / threads);
  const bool ice = a.adiabat >= 3;
  const bool pseudo = (a.adiabat == 1 || a.adiabat == 3);
  if (ice && pseudo) cape_learned_warp_kernel<T, GRID, true, true><<<blocks, threads, 0, s>>>(a);
  else if (ice) cape_learned_warp_kernel<T, GRID, true, false><<<blocks, threads, 0, s>>>(a);
  else if (pseudo) cape_learned_warp_kernel<T, GRID, false, true><<<blocks, threads, 0, s>>>(a);
  else cape_learned_warp_kernel<T, GRID, false, false><<<blocks, threads, 0, s>>>(a);
}

// guess codes (include/xcape_gb300.h): 0 plain, 1 learned, 2 extrapolated,
// 3 plain first guess with secant steps, 4 the network on every saturated
// sub-step (per thread), 5 the same per warp in lockstep on the tensor cores.
template <typename T, int GRID>
static cudaError_t launch_cape_t(const CapeArgs &a, cudaStream_t s) {
  const int threads = 128;
  const unsigned blocks = (unsigned)((a.n2 + threads - 1) / threads);
  if (blocks == 0) return cudaSuccess;
  switch (a.guess) {
    case 0: launch_cape_s<T, GRID, SOLVE_PLAIN>(a, blocks, threads, s); break;
    case 1: launch_learned<T, GRID>(a, s); break;
    case 2: launch_cape_s<T, GRID, SOLVE_ACCEL>(a, blocks, threads, s); break;
    case 3: launch_cape_s<T, GRID, SOLVE_SECANT>(a, blocks, threads, s); break;
    case 5: launch_learned_warp<T, GRID>(a, s); break;
    default: launch_cape_s<T, GRID, SOLVE_LEARNED_ALL>(a, blocks, threads, s); break;
  }
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
