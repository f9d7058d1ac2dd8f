// batch.cu -- ragged batches of calc_cape requests in one persistent,
// graph-captured kernel.
//
// A batch is a list of requests (xc_cape_request): each has its own column
// count, level count, row stride, grid kind (sigma/model or pressure levels
// with below-ground levels masked per column), source, adiabat, pinc and
// ml_depth.  The executor (xc_batch) owns a device request table, a pinned
// staging copy of it, and a CUDA graph that uploads the table, clears the
// work counters and launches cape_batch_kernel.  A run writes the staging
// table and launches the graph: one graph launch per batch whatever its
// composition.
//
// In the kernel each request's columns occupy a range of a global column
// space whose start is a multiple of 32, so a warp's chunk of 32 columns
// always lies in one request: the warp takes chunks from an atomic counter
// until the space is exhausted (a persistent grid of one wave of blocks),
// finds the chunk's request by a warp-uniform binary search, and each lane
// runs one column with the column routine of the single-request kernels
// (cape_column.cuh; for the learned solver cape_learned.cuh, whose guess
// network the converged warp evaluates for its 32 columns on the tensor
// cores), selected at run time by grid kind and adiabat.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/xcape_gb300.h"
#include "cape_column.cuh"
#include "cape_learned.cuh"
#include "xc_kernels.h"

namespace xc {

namespace {

struct BatchReq {
  xc_cape_request q;
  long long col0;  // first column of the request in the batch's column space
};

struct BatchHeader {
  int nreq;
  int pad;
  long long nchunks;  // 32-column chunks in the column space
};

constexpr size_t kHeaderBytes = 64;  // keeps the request array 64-byte aligned
constexpr int kSlots = 2;            // table/graph slots used alternately

size_t table_bytes(int max_requests) {
  return kHeaderBytes + sizeof(BatchReq) * (size_t)max_requests;
}

__device__ __forceinline__ CapeArgs request_args(const xc_cape_request &q) {
  CapeArgs a;
  a.grid = q.grid;
  a.dtype = 0;
  a.p = q.p;
  a.t = q.t3d;
  a.td = q.td3d;
  a.ps = q.ps;
  a.ts = q.ts;
  a.tds = q.tds;
  a.start = nullptr;
  a.pinc = q.pinc;
  a.source = q.source;
  a.ml_depth = q.ml_depth;
  a.adiabat = q.adiabat;
  a.nk = q.nk;
  a.n2 = q.n2;
  a.ld = q.ld;
  a.guess = 0;
  a.cape = q.cape;
  a.cin = q.cin;
  a.mulvl = q.mulvl;
  a.z_out = q.z_out;
  a.status = q.status;
  a.counters = nullptr;
  a.perm = nullptr;
  a.guess_w = nullptr;
  return a;
}

template <int SOLVER>
__device__ void run_request_column(const xc_cape_request &q, long long i, int &nsub, int &niter) {
  const CapeArgs a = request_args(q);
  const float *gw = nullptr;
  const bool ice = q.adiabat >= 3, pseudo = (q.adiabat == 1 || q.adiabat == 3);
  if (q.grid == 1) {
    if (ice && pseudo) cape_column_run<float, 1, true, true, SOLVER>(a, i, nsub, niter, gw);
    else if (ice) cape_column_run<float, 1, true, false, SOLVER>(a, i, nsub, niter, gw);
    else if (pseudo) cape_column_run<float, 1, false, true, SOLVER>(a, i, nsub, niter, gw);
    else cape_column_run<float, 1, false, false, SOLVER>(a, i, nsub, niter, gw);
  } else {
    if (ice && pseudo) cape_column_run<float, 2, true, true, SOLVER>(a, i, nsub, niter, gw);
    else if (ice) cape_column_run<float, 2, true, false, SOLVER>(a, i, nsub, niter, gw);
    else if (pseudo) cape_column_run<float, 2, false, true, SOLVER>(a, i, nsub, niter, gw);
    else cape_column_run<float, 2, false, false, SOLVER>(a, i, nsub, niter, gw);
  }
}

// Column i of a request with the learned solver; every lane of the warp
// calls it (lanes past the request's n2 take part in the network's
// evaluation and write nothing).
__device__ void run_request_column_learned(const xc_cape_request &q, long long i,
                                           const WarpNetSmem &net, LearnedPrep *prep, int &nsub,
                                           int &niter) {
  const CapeArgs a = request_args(q);
  const bool ice = q.adiabat >= 3, pseudo = (q.adiabat == 1 || q.adiabat == 3);
  if (q.grid == 1) {
    if (ice && pseudo) learned_column<float, 1, true, true>(a, net, prep, i, nsub, niter);
    else if (ice) learned_column<float, 1, true, false>(a, net, prep, i, nsub, niter);
    else if (pseudo) learned_column<float, 1, false, true>(a, net, prep, i, nsub, niter);
    else learned_column<float, 1, false, false>(a, net, prep, i, nsub, niter);
  } else {
    if (ice && pseudo) learned_column<float, 2, true, true>(a, net, prep, i, nsub, niter);
    else if (ice) learned_column<float, 2, true, false>(a, net, prep, i, nsub, niter);
    else if (pseudo) learned_column<float, 2, false, true>(a, net, prep, i, nsub, niter);
    else learned_column<float, 2, false, false>(a, net, prep, i, nsub, niter);
  }
}

// counters: [0] the chunk counter, [1] sub-steps, [2] iterations.
template <int SOLVER>
__global__ void __launch_bounds__(LEARNED_THREADS) cape_batch_kernel(const unsigned char *table,
                                                                     unsigned long long *counters,
                                                                     const WarpNetSmem *net_img) {
  __shared__ WarpNetSmem net;                    // SOLVE_LEARNED only
  __shared__ LearnedPrep prep[LEARNED_THREADS];  // SOLVE_LEARNED only
  if (SOLVER == SOLVE_LEARNED) {
    copy_warp_net(net, net_img);
    __syncthreads();
  }
  const BatchHeader hdr = *reinterpret_cast<const BatchHeader *>(table);
  const BatchReq *reqs = reinterpret_cast<const BatchReq *>(table + kHeaderBytes);
  const int lane = threadIdx.x & 31;
  long long nsub_sum = 0, niter_sum = 0;
  while (true) {
    unsigned long long c = 0;
    if (lane == 0) c = atomicAdd(counters, 1ull);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= (unsigned long long)hdr.nchunks) break;
    const long long g = (long long)c * 32;
    // last request whose range starts at or before g (warp-uniform)
    int lo = 0, hi = hdr.nreq - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (reqs[mid].col0 <= g) lo = mid;
      else hi = mid - 1;
    }
    const long long i = g + lane - reqs[lo].col0;
    int nsub = 0, niter = 0;
    if (SOLVER == SOLVE_LEARNED) {
      run_request_column_learned(reqs[lo].q, i, net, prep, nsub, niter);
    } else if (i < reqs[lo].q.n2) {
      run_request_column<SOLVER>(reqs[lo].q, i, nsub, niter);
    }
    nsub_sum += nsub;
    niter_sum += niter;
  }
  for (int o = 16; o > 0; o >>= 1) {
    nsub_sum += __shfl_down_sync(0xffffffffu, nsub_sum, o);
    niter_sum += __shfl_down_sync(0xffffffffu, niter_sum, o);
  }
  if (lane == 0) {
    atomicAdd(counters + 1, (unsigned long long)nsub_sum);
    atomicAdd(counters + 2, (unsigned long long)niter_sum);
  }
}

template <int SOLVER>
cudaError_t capture_batch(cudaStream_t cs, unsigned char *dtable, const unsigned char *htable,
                          size_t bytes, unsigned long long *counters, const WarpNetSmem *gw,
                          cudaGraph_t *graph) {
  const size_t smem = 0;
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, cape_batch_kernel<SOLVER>, 128,
                                                      smem);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)(sms * (per_sm > 0 ? per_sm : 1));
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  cudaMemcpyAsync(dtable, htable, bytes, cudaMemcpyHostToDevice, cs);
  cudaMemsetAsync(counters, 0, 3 * sizeof(unsigned long long), cs);
  cape_batch_kernel<SOLVER><<<blocks, 128, smem, cs>>>(dtable, counters, gw);
  const cudaError_t le = cudaGetLastError();
  e = cudaStreamEndCapture(cs, graph);
  return le != cudaSuccess ? le : e;
}

}  // namespace

}  // namespace xc

// ---- C ABI --------------------------------------------------------------------

struct xc_batch {
  int device = 0;
  int max_requests = 0;
  long long max_columns = 0;
  int guess = 0;
  size_t bytes = 0;
  unsigned char *htable[xc::kSlots] = {};  // pinned staging tables
  unsigned char *dtable[xc::kSlots] = {};
  unsigned long long *counters[xc::kSlots] = {};  // device: chunk counter, sub-steps, iterations
  cudaGraphExec_t exec[xc::kSlots] = {};
  cudaEvent_t done[xc::kSlots] = {};
  int next = 0;       // slot of the next run
  int last = -1;      // slot of the last run
  std::mutex mu;
};

namespace xc {
int guess_weights_ptr(const float **out);                                      // capi.cu
int check_cape_options(float pinc, int source, float ml_depth, int adiabat);  // capi.cu
}  // namespace xc

namespace {

void batch_free(xc_batch *b) {
  for (int s = 0; s < xc::kSlots; ++s) {
    if (b->exec[s]) cudaGraphExecDestroy(b->exec[s]);
    if (b->done[s]) cudaEventDestroy(b->done[s]);
    if (b->dtable[s]) cudaFree(b->dtable[s]);
    if (b->counters[s]) cudaFree(b->counters[s]);
    if (b->htable[s]) cudaFreeHost(b->htable[s]);
  }
  delete b;
}

int cuda_err(cudaError_t e, const char *what) {
  char buf[256];
  snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
  return xc::set_error(XC_ERR_CUDA, buf);
}

}  // namespace

extern "C" {

int xc_batch_create(int max_requests, long long max_columns, int guess, xc_batch **out) {
  if (!out) return xc::set_error(XC_ERR_INVALID, "xc_batch_create: out is NULL");
  *out = nullptr;
  if (max_requests < 1 || max_requests > XC_BATCH_MAX_REQUESTS)
    return xc::set_error(XC_ERR_INVALID, "xc_batch_create: max_requests out of range");
  if (max_columns < 32) return xc::set_error(XC_ERR_INVALID, "xc_batch_create: max_columns < 32");
  if (guess != XC_GUESS_PLAIN && guess != XC_GUESS_LEARNED && guess != XC_GUESS_EXTRAPOLATED)
    return xc::set_error(XC_ERR_INVALID,
                          "xc_batch_create: guess must be XC_GUESS_PLAIN, _LEARNED or _EXTRAPOLATED");
  const xc::WarpNetSmem *gw = nullptr;  // the learned kernel's image of the guess network
  if (guess == XC_GUESS_LEARNED) {
    const float *w = nullptr;
    const int rc = xc::guess_weights_ptr(&w);  // fails unless a network is loaded
    if (rc) return rc;
    const void *img = nullptr;
    const cudaError_t ie = xc::warp_net_image(&img);
    if (ie != cudaSuccess) return cuda_err(ie, "xc_batch_create: the guess network's image");
    gw = (const xc::WarpNetSmem *)img;
  }
  xc_batch *b = new (std::nothrow) xc_batch();
  if (!b) return xc::set_error(XC_ERR_NOMEM, "xc_batch_create: host allocation");
  b->max_requests = max_requests;
  b->max_columns = max_columns;
  b->guess = guess;
  b->bytes = xc::table_bytes(max_requests);
  cudaError_t e = cudaGetDevice(&b->device);
  cudaStream_t cs = nullptr;
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  for (int s = 0; s < xc::kSlots && e == cudaSuccess; ++s) {
    e = xc::host_malloc((void **)&b->htable[s], b->bytes);
    if (e == cudaSuccess) e = xc::dev_malloc((void **)&b->dtable[s], b->bytes);
    if (e == cudaSuccess) e = xc::dev_malloc((void **)&b->counters[s], 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->done[s], cudaEventDisableTiming);
    if (e != cudaSuccess) break;
    memset(b->htable[s], 0, b->bytes);
    cudaGraph_t graph = nullptr;
    switch (guess) {
      case XC_GUESS_PLAIN:
        e = xc::capture_batch<xc::SOLVE_PLAIN>(cs, b->dtable[s], b->htable[s], b->bytes,
                                               b->counters[s], gw, &graph);
        break;
      case XC_GUESS_LEARNED:
        e = xc::capture_batch<xc::SOLVE_LEARNED>(cs, b->dtable[s], b->htable[s], b->bytes,
                                                 b->counters[s], gw, &graph);
        break;
      default:
        e = xc::capture_batch<xc::SOLVE_ACCEL>(cs, b->dtable[s], b->htable[s], b->bytes,
                                               b->counters[s], gw, &graph);
        break;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[s], graph, 0);
    if (graph) cudaGraphDestroy(graph);
  }
  if (cs) cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    const int rc = cuda_err(e, "xc_batch_create");
    batch_free(b);
    return rc;
  }
  *out = b;
  return XC_OK;
}

int xc_batch_run(xc_batch *b, const xc_cape_request *reqs, int nreq, void *stream) {
  if (!b) return xc::set_error(XC_ERR_INVALID, "xc_batch_run: batch is NULL");
  if (nreq < 0 || nreq > b->max_requests)
    return xc::set_error(XC_ERR_INVALID, "xc_batch_run: nreq out of range for this batch");
  if (nreq > 0 && !reqs) return xc::set_error(XC_ERR_INVALID, "xc_batch_run: reqs is NULL");
  // validate everything before touching the staging table
  long long cols = 0;
  for (int r = 0; r < nreq; ++r) {
    const xc_cape_request &q = reqs[r];
    if (q.n2 < 0) return xc::set_error(XC_ERR_INVALID, "xc_batch_run: request with n2 < 0");
    if (q.n2 == 0) continue;
    if (q.grid != 1 && q.grid != 2)
      return xc::set_error(XC_ERR_INVALID, "xc_batch_run: request grid must be 1 or 2");
    if (q.nk < 1 || q.nk > XC_MAX_LEVELS || q.ld < q.nk)
      return xc::set_error(XC_ERR_INVALID, "xc_batch_run: request needs 1 <= nk <= ld");
    if (!q.p || !q.t3d || !q.td3d || !q.ps || !q.ts || !q.tds || !q.cape || !q.cin || !q.mulvl ||
        !q.z_out)
      return xc::set_error(XC_ERR_INVALID, "xc_batch_run: NULL array in a request");
    const int rc = xc::check_cape_options(q.pinc, q.source, q.ml_depth, q.adiabat);
    if (rc) return rc;
    cols += (q.n2 + 31) / 32 * 32;
    if (cols > b->max_columns)
      return xc::set_error(XC_ERR_INVALID, "xc_batch_run: batch exceeds max_columns");
  }
  std::lock_guard<std::mutex> lk(b->mu);
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_err(e, "cudaGetDevice");
  if (dev != b->device)
    return xc::set_error(XC_ERR_INVALID, "xc_batch_run: batch belongs to another device");
  const int s = b->next;
  // the slot's staging table may still be read by the run two launches ago
  e = cudaEventSynchronize(b->done[s]);
  if (e != cudaSuccess) return cuda_err(e, "xc_batch_run: waiting for the slot");
  unsigned char *h = b->htable[s];
  xc::BatchReq *out = reinterpret_cast<xc::BatchReq *>(h + xc::kHeaderBytes);
  int n = 0;
  long long col0 = 0;
  for (int r = 0; r < nreq; ++r) {
    if (reqs[r].n2 == 0) continue;
    out[n].q = reqs[r];
    out[n].col0 = col0;
    col0 += (reqs[r].n2 + 31) / 32 * 32;
    ++n;
  }
  xc::BatchHeader hdr;
  hdr.nreq = n;
  hdr.pad = 0;
  hdr.nchunks = col0 / 32;
  memcpy(h, &hdr, sizeof(hdr));
  e = cudaGraphLaunch(b->exec[s], (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(e, "xc_batch_run: cudaGraphLaunch");
  e = cudaEventRecord(b->done[s], (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_err(e, "xc_batch_run: cudaEventRecord");
  b->last = s;
  b->next = (s + 1) % xc::kSlots;
  return XC_OK;
}

int xc_batch_work(xc_batch *b, long long *substeps, long long *iterations) {
  if (!b || !substeps || !iterations) return xc::set_error(XC_ERR_INVALID, "xc_batch_work: NULL");
  std::lock_guard<std::mutex> lk(b->mu);
  if (b->last < 0) {
    *substeps = *iterations = 0;
    return XC_OK;
  }
  unsigned long long c[3];
  cudaError_t e = cudaEventSynchronize(b->done[b->last]);
  if (e == cudaSuccess) e = cudaMemcpy(c, b->counters[b->last], sizeof(c), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_err(e, "xc_batch_work");
  *substeps = (long long)c[1];
  *iterations = (long long)c[2];
  return XC_OK;
}

int xc_batch_destroy(xc_batch *b) {
  if (!b) return XC_OK;
  for (int s = 0; s < xc::kSlots; ++s)
    if (b->done[s]) cudaEventSynchronize(b->done[s]);
  batch_free(b);
  return XC_OK;
}

int xc_copy_list(int n, void *const *dst, const void *const *src,
                 const unsigned long long *bytes, void *stream) {
  if (n < 0 || (n > 0 && (!dst || !src || !bytes)))
    return xc::set_error(XC_ERR_INVALID, "xc_copy_list: n < 0 or NULL arrays");
  for (int k = 0; k < n; ++k) {
    if (bytes[k] == 0) continue;
    if (!dst[k] || !src[k]) return xc::set_error(XC_ERR_INVALID, "xc_copy_list: NULL pointer");
    const cudaError_t e =
        cudaMemcpyAsync(dst[k], src[k], (size_t)bytes[k], cudaMemcpyDefault, (cudaStream_t)stream);
    if (e != cudaSuccess) return xc::set_error(XC_ERR_CUDA, cudaGetErrorString(e));
  }
  return XC_OK;
}

}  // extern "C"
