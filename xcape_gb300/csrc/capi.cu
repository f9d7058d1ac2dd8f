// capi.cu -- extern "C" entry points of libxcape_gb300.so (include/xcape_gb300.h).
//
// Argument checks stand in for the reference's `stop` statements and the
// Python-side ValueError/KeyError paths: every bad argument returns
// XC_ERR_INVALID with a message in xc_last_error(); nothing aborts.
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/xcape_gb300.h"
#include "xc_kernels.h"

namespace {

thread_local char g_err[512] = "";
// successful device and pinned-host allocations since the library was loaded
std::atomic<long long> g_allocs{0};

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *where) {
  return fail(XC_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

int check_common(int dtype, int nk, int n2) {
  if (dtype != XC_F32 && dtype != XC_F64) return fail(XC_ERR_INVALID, "dtype must be XC_F32 or XC_F64");
  if (nk < 1 || nk > XC_MAX_LEVELS) return fail(XC_ERR_INVALID, "nk=%d outside 1..%d", nk, XC_MAX_LEVELS);
  if (n2 < 0) return fail(XC_ERR_INVALID, "n2=%d is negative", n2);
  return XC_OK;
}

int check_cape_opts(float pinc, int source, float ml_depth, int adiabat) {
  if (source < 1 || source > 3)
    return fail(XC_ERR_INVALID, "Unknown value for source: %d (1 surface, 2 most unstable, 3 mixed layer)", source);
  if (adiabat < 1 || adiabat > 4) return fail(XC_ERR_INVALID, "Undefined adiabat: %d (1..4)", adiabat);
  if (!(pinc > 0.0f)) return fail(XC_ERR_INVALID, "pinc must be a positive pressure increment (Pa)");
  if (source == 3 && !(ml_depth > 0.0f)) return fail(XC_ERR_INVALID, "ml_depth must be positive");
  return XC_OK;
}

// Columns per chunk of the pipelined host path: at least this many, at most
// host_chunks() chunks (HOST_CHUNKS at most); the chunks' device buffers (a
// ring of slots) take at most host_ring_bytes(), and at least two slots.
constexpr int HOST_CHUNK_MIN = 131072;
constexpr int HOST_CHUNKS = 16;

// 8, or the environment's XC_HOST_CHUNKS (2..16; it changes only how the
// work is pipelined, never a result).
int host_chunks() {
  const char *e = getenv("XC_HOST_CHUNKS");
  if (e && *e) {
    const int v = atoi(e);
    if (v >= 2 && v <= HOST_CHUNKS) return v;
  }
  return 8;
}

// 4 GiB, or the environment's XC_HOST_RING_BYTES (it changes only how
// many chunks are in flight, never a result).
size_t host_ring_bytes() {
  const char *e = getenv("XC_HOST_RING_BYTES");
  if (e && *e) {
    char *end = nullptr;
    const unsigned long long v = strtoull(e, &end, 10);
    if (end && *end == '\0') return (size_t)v;
  }
  return (size_t)4 << 30;
}

// Compute streams the host path's chunks take in turn: 2, or the
// environment's XC_HOST_STREAMS (1..4; it changes only how the work overlaps
// on the GPU, never a result).  With the second source's lifts on a side
// stream, 1, 2, 3 and 4 compute streams gave 389, 403, 394 and 388 M
// columns/s end to end on 1M columns x 37 levels, two sources.
int host_streams() {
  const char *e = getenv("XC_HOST_STREAMS");
  if (e && *e) {
    const int v = atoi(e);
    if (v >= 1 && v <= 4) return v;
  }
  return 2;
}

// Host threads that move the host path's outputs from pinned staging into
// the caller's arrays: 4, or the environment's XC_HOST_COPY_THREADS (0..16;
// 0 leaves the copies to the calling thread).  One thread moves about
// 16 GB/s: for a million columns and two sources (33 MB of outputs) the
// calling thread alone took 1.4 ms longer than the GPU work it was to hide
// behind (3.15 against 1.75 ms).
int host_copy_threads() {
  const char *e = getenv("XC_HOST_COPY_THREADS");
  if (e && *e) {
    const int v = atoi(e);
    if (v >= 0 && v <= 16) return v;
  }
  return 4;
}

// A pool of those threads, started on first use and kept for the process
// (re-created in a child after fork).  A call hands its jobs in as one
// CopyBatch and waits for the batch before it returns, also on an error:
// the jobs use the call's stack.
struct CopyBatch {
  std::mutex mu;
  std::condition_variable cv;
  int left = 0;
  cudaError_t err = cudaSuccess;
  void wait() {
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return left == 0; });
  }
  ~CopyBatch() { wait(); }
};

class CopyPool {
 public:
  explicit CopyPool(int n) : pid_(getpid()) {
    for (int i = 0; i < n; ++i) std::thread([this] { loop(); }).detach();
  }
  pid_t pid() const { return pid_; }
  void submit(CopyBatch *b, std::function<cudaError_t()> job) {
    {
      std::lock_guard<std::mutex> lk(b->mu);
      ++b->left;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      q_.push_back({b, std::move(job)});
    }
    cv_.notify_one();
  }

 private:
  struct Job {
    CopyBatch *b;
    std::function<cudaError_t()> run;
  };
  void loop() {
    for (;;) {
      Job j;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return !q_.empty(); });
        j = std::move(q_.front());
        q_.pop_front();
      }
      const cudaError_t e = j.run();
      std::lock_guard<std::mutex> lk(j.b->mu);
      if (e != cudaSuccess && j.b->err == cudaSuccess) j.b->err = e;
      if (--j.b->left == 0) j.b->cv.notify_all();
    }
  }
  pid_t pid_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<Job> q_;
};

std::mutex g_pool_mu;
CopyPool *g_pool = nullptr;  // never freed: its threads outlive every call

CopyPool *copy_pool() {
  const int n = host_copy_threads();
  if (n == 0) return nullptr;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  if (!g_pool || g_pool->pid() != getpid()) g_pool = new CopyPool(n);
  return g_pool;
}

// Host calls in flight at once on one device: 4, or the environment's
// XC_HOST_CONTEXTS (1..64).  Calls beyond that wait for a context.
int host_contexts() {
  const char *e = getenv("XC_HOST_CONTEXTS");
  if (e && *e) {
    const int v = atoi(e);
    if (v >= 1 && v <= 64) return v;
  }
  return 4;
}

// Everything one host-pointer call uses on its device, owned by that call
// while it runs: two non-blocking streams for the chunks' kernels and
// output copies and one for their input copies (chunk c + 1's copies
// overlap chunk c's kernels), events, pinned output staging and the device
// workspace (grow-only).  Contexts are created on first use and kept for the
// process; calls from several host threads -- dask's threaded scheduler
// computing chunks at once -- each take their own context, so their copies
// and kernels overlap on the GPU instead of queueing behind one lock.
struct HostCtx {
  int dev = -1;
  bool busy = false;
  cudaStream_t s[4] = {};  // kernels and output copies, chunks in turn over host_streams()
  cudaStream_t copy = nullptr;             // input copies, in chunk order
  // the chunks' column orderings, at the device's highest stream priority:
  // a chunk's ordering kernels then take the SM slots that earlier chunks'
  // lift blocks free before more lift blocks do, and its lifts start sooner
  cudaStream_t ord = nullptr;
  cudaEvent_t start = nullptr;
  cudaEvent_t loaded[HOST_CHUNKS] = {};    // slot k holds its chunk's inputs
  cudaEvent_t surf[HOST_CHUNKS] = {};      // ... those the ordering reads (copied first)
  cudaEvent_t ordered[HOST_CHUNKS] = {};   // slot k's columns are ordered
  // the second and third sources' lifts of every chunk, beside the first
  // source's on the chunk's compute stream (a chunk's lifts are about one
  // wave of blocks each, and beside each other they share the SMs);
  // lifted[k][j] marks slot k's lift of source j + 1 done
  cudaStream_t side[2] = {};
  cudaEvent_t lifted[HOST_CHUNKS][2] = {};
  cudaEvent_t done[HOST_CHUNKS] = {};      // slot k's outputs are in its staging
  char *pinned = nullptr;                  // pinned output staging, grow-only
  size_t pinned_cap = 0;
  void *ws = nullptr;                      // device workspace, grow-only
  size_t ws_cap = 0;
};
std::mutex g_ctx_mu;
std::condition_variable g_ctx_cv;
std::vector<std::unique_ptr<HostCtx>> g_ctx;

// Takes a free context of the current device (creating one while fewer than
// host_contexts() exist), waiting for one otherwise; releases it on scope
// exit.
struct HostCtxLease {
  HostCtx *c = nullptr;
  int acquire() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    {
      std::unique_lock<std::mutex> lk(g_ctx_mu);
      for (;;) {
        int count = 0;
        for (auto &x : g_ctx) {
          if (x->dev != dev) continue;
          ++count;
          if (!x->busy) {
            c = x.get();
            break;
          }
        }
        if (!c && count < host_contexts()) {
          g_ctx.push_back(std::unique_ptr<HostCtx>(new HostCtx()));
          c = g_ctx.back().get();
          c->dev = dev;
        }
        if (c) {
          c->busy = true;
          break;
        }
        g_ctx_cv.wait(lk);
      }
    }
    for (int k = 0; k < 4 && e == cudaSuccess; ++k)
      if (!c->s[k]) e = cudaStreamCreateWithFlags(&c->s[k], cudaStreamNonBlocking);
    if (e == cudaSuccess && !c->copy) e = cudaStreamCreateWithFlags(&c->copy, cudaStreamNonBlocking);
    for (int j = 0; j < 2 && e == cudaSuccess; ++j)
      if (!c->side[j]) e = cudaStreamCreateWithFlags(&c->side[j], cudaStreamNonBlocking);
    if (e == cudaSuccess && !c->ord) {
      int least = 0, greatest = 0;
      e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
      if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->ord, cudaStreamNonBlocking, greatest);
    }
    for (int k = 0; k < HOST_CHUNKS && e == cudaSuccess; ++k) {
      if (!c->done[k]) e = cudaEventCreateWithFlags(&c->done[k], cudaEventDisableTiming);
      if (e == cudaSuccess && !c->ordered[k])
        e = cudaEventCreateWithFlags(&c->ordered[k], cudaEventDisableTiming);
      if (e == cudaSuccess && !c->surf[k])
        e = cudaEventCreateWithFlags(&c->surf[k], cudaEventDisableTiming);
      for (int j = 0; j < 2 && e == cudaSuccess; ++j)
        if (!c->lifted[k][j]) e = cudaEventCreateWithFlags(&c->lifted[k][j], cudaEventDisableTiming);
      if (e == cudaSuccess && !c->loaded[k])
        e = cudaEventCreateWithFlags(&c->loaded[k], cudaEventDisableTiming);
    }
    if (e == cudaSuccess && !c->start)
      e = cudaEventCreateWithFlags(&c->start, cudaEventDisableTiming);
    if (e != cudaSuccess) return cuda_fail(e, "creating the host-path streams");
    return XC_OK;
  }
  ~HostCtxLease() {
    if (!c) return;
    {
      std::lock_guard<std::mutex> lk(g_ctx_mu);
      c->busy = false;
    }
    g_ctx_cv.notify_all();
  }
};

int ctx_pinned(HostCtx *c, size_t bytes) {
  if (c->pinned_cap >= bytes) return XC_OK;
  if (c->pinned) cudaFreeHost(c->pinned);
  c->pinned = nullptr;
  c->pinned_cap = 0;
  const cudaError_t e = xc::host_malloc((void **)&c->pinned, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return fail(XC_ERR_NOMEM, "cudaMallocHost(%zu) for the host-path staging: %s", bytes,
                cudaGetErrorString(e));
  }
  c->pinned_cap = bytes;
  return XC_OK;
}

int ctx_workspace(HostCtx *c, size_t bytes, void **out) {
  if (c->ws_cap < bytes) {
    if (c->ws) {
      cudaFree(c->ws);
      c->ws = nullptr;
      c->ws_cap = 0;
    }
    const cudaError_t e = xc::dev_malloc(&c->ws, bytes);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(XC_ERR_NOMEM, "cudaMalloc(%zu) for the host-path workspace: %s", bytes,
                  cudaGetErrorString(e));
    }
    c->ws_cap = bytes;
  }
  *out = c->ws;
  return XC_OK;
}

// The guess network used by XC_GUESS_LEARNED: a static device array per
// device, filled by xc_guess_set_weights.
__device__ float g_guess_w[XC_GUESS_NPARAM];
constexpr int kMaxGuessDevices = 64;
std::mutex g_guess_mu;
bool g_guess_loaded[kMaxGuessDevices] = {};

int guess_weights(const float **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxGuessDevices) return fail(XC_ERR_INVALID, "device %d out of range", dev);
  {
    std::lock_guard<std::mutex> lk(g_guess_mu);
    if (!g_guess_loaded[dev])
      return fail(XC_ERR_INVALID, "no guess network is loaded on device %d (xc_guess_set_weights)", dev);
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_guess_w);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress");
  *out = (const float *)p;
  return XC_OK;
}

// Carves 256-byte aligned slices out of one workspace allocation.
struct Carver {
  size_t off = 0;
  size_t take(size_t bytes) {
    size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  }
};

// Side streams of xc_loopcape_multi on each device (created on first use,
// kept for the process): the second and third sources' lifts run on them,
// beside the first source's on the caller's stream, so that a lift's last
// blocks share the GPU with the next lift's first ones instead of running
// alone.  The events that fork and join them are recorded and waited on
// under g_side_mu, so that calls from several host threads each wait on
// their own records.
struct SideStreams {
  int dev = -1;
  cudaStream_t s[2] = {nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
};
std::mutex g_side_mu;
std::vector<std::unique_ptr<SideStreams>> g_side;

int side_streams(SideStreams **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  std::lock_guard<std::mutex> lk(g_side_mu);
  for (auto &x : g_side)
    if (x->dev == dev) {
      *out = x.get();
      return XC_OK;
    }
  auto x = std::make_unique<SideStreams>();
  x->dev = dev;
  for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
    e = cudaStreamCreateWithFlags(&x->s[k], cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x->join[k], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&x->fork, cudaEventDisableTiming);
  if (e != cudaSuccess) return cuda_fail(e, "side streams of the multi-source lift");
  *out = x.get();
  g_side.push_back(std::move(x));
  return XC_OK;
}

// xc_loopcape_ex (nsrc 1) and xc_loopcape_multi: the lifts of nsrc sources
// of the same device-resident columns, outputs [nsrc][n2].  With a workspace
// the columns are ordered once, and every source's lift reads that order;
// the FP64 retries, which reuse the workspace, come after all the lifts.
int lift_sources(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                 const void *ts, const void *tds, int dtype, float pinc, int nsrc,
                 const int *sources, float ml_depth, int adiabat, const int *start_3d, int nk,
                 int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out, int *status,
                 long long *counters, void *workspace, size_t workspace_bytes, void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  for (int j = 0; j < nsrc; ++j) {
    rc = check_cape_opts(pinc, sources[j], ml_depth, adiabat);
    if (rc) return rc;
  }
  if (grid < 1 || grid > 3) return fail(XC_ERR_INVALID, "grid must be 1 (sigma), 2 (pressure, 1-D p) or 3 (pressure, 3-D p)");
  if (grid == 3 && !start_3d) return fail(XC_ERR_INVALID, "grid 3 needs start_3d");
  const bool retry = (guess & XC_RETRY_FP64) != 0;
  guess &= ~XC_RETRY_FP64;
  if (guess < XC_GUESS_PLAIN || guess > XC_GUESS_LEARNED_WARP)
    return fail(XC_ERR_INVALID, "guess %d is not one of XC_GUESS_*", guess);
  if (retry && !status) return fail(XC_ERR_INVALID, "XC_RETRY_FP64 needs the status array");
  const float *guess_w = nullptr;
  if (guess == XC_GUESS_LEARNED || guess == XC_GUESS_LEARNED_EVERY ||
      guess == XC_GUESS_LEARNED_WARP) {
    rc = guess_weights(&guess_w);
    if (rc) return rc;
  }
  if (n2 == 0) return XC_OK;
  if (!p || !t3d || !td3d || !ps || !ts || !tds || !cape || !cin || !mulvl || !z_out)
    return fail(XC_ERR_INVALID, "NULL array argument");
  xc::CapeArgs a;
  a.grid = grid;
  a.dtype = dtype;
  a.p = p;
  a.t = t3d;
  a.td = td3d;
  a.ps = ps;
  a.ts = ts;
  a.tds = tds;
  a.start = grid == 1 ? nullptr : start_3d;
  a.pinc = pinc;
  a.ml_depth = ml_depth;
  a.adiabat = adiabat;
  a.nk = nk;
  a.n2 = n2;
  a.guess = guess;
  a.counters = counters;
  a.perm = nullptr;
  a.guess_w = guess_w;
  cudaError_t e = cudaSuccess;
  if (workspace) {
    if (workspace_bytes < xc::order_workspace_bytes(n2))
      return fail(XC_ERR_INVALID, "workspace of %zu bytes is smaller than the %zu needed",
                  workspace_bytes, xc::order_workspace_bytes(n2));
    if (((size_t)workspace & 255) != 0) return fail(XC_ERR_INVALID, "workspace must be 256-byte aligned");
    e = xc::launch_order(a, workspace, &a.perm, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "column ordering launch");
  }
  auto point = [&](int j) {
    const size_t o = (size_t)j * (size_t)n2;
    a.source = sources[j];
    a.cape = cape + o;
    a.cin = cin + o;
    a.mulvl = mulvl + o;
    a.z_out = z_out + o;
    a.status = status ? status + o : nullptr;
  };
  if (nsrc == 1) {
    point(0);
    e = xc::launch_cape(a, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cape kernel launch");
  } else {
    SideStreams *ss = nullptr;
    rc = side_streams(&ss);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_side_mu);
    const cudaStream_t s0 = (cudaStream_t)stream;
    e = cudaEventRecord(ss->fork, s0);  // after the ordering
    for (int j = 1; j < nsrc && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(ss->s[j - 1], ss->fork, 0);
    if (e != cudaSuccess) return cuda_fail(e, "forking the multi-source lift");
    for (int j = 0; j < nsrc; ++j) {
      point(j);
      e = xc::launch_cape(a, j == 0 ? s0 : ss->s[j - 1]);
      if (e != cudaSuccess) return cuda_fail(e, "cape kernel launch");
    }
    for (int j = 1; j < nsrc && e == cudaSuccess; ++j) {
      e = cudaEventRecord(ss->join[j - 1], ss->s[j - 1]);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(s0, ss->join[j - 1], 0);
    }
    if (e != cudaSuccess) return cuda_fail(e, "joining the multi-source lift");
  }
  for (int j = 0; retry && j < nsrc; ++j) {
    point(j);
    e = xc::launch_retry64(a, workspace, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "FP64 retry launch");
  }
  return XC_OK;
}

}  // namespace

extern "C" {

const char *xc_last_error(void) { return g_err; }

const char *xc_version(void) { return "xcape_gb300 0.1.0 (sm_103a)"; }

long long xc_alloc_count(void) { return g_allocs.load(std::memory_order_relaxed); }

int xc_release_workspace(void) {
  // frees the workspaces of the contexts no call holds
  std::lock_guard<std::mutex> lk(g_ctx_mu);
  int prev = 0;
  cudaGetDevice(&prev);
  for (auto &c : g_ctx) {
    if (c->busy || !c->ws) continue;
    cudaSetDevice(c->dev);
    cudaFree(c->ws);
    c->ws = nullptr;
    c->ws_cap = 0;
  }
  cudaSetDevice(prev);
  return XC_OK;
}

size_t xc_loopcape_workspace_bytes(int n2) {
  return n2 > 0 ? xc::order_workspace_bytes(n2) : 0;
}

int xc_loopcape_ex(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, const int *start_3d, int nk, int n2, int guess,
                   float *cape, float *cin, int *mulvl, float *z_out, int *status,
                   long long *counters, void *workspace, size_t workspace_bytes, void *stream) {
  return lift_sources(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, 1, &source, ml_depth, adiabat,
                      start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, counters,
                      workspace, workspace_bytes, stream);
}

int xc_loopcape_multi(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                      const void *ts, const void *tds, int dtype, float pinc, int nsrc,
                      const int *sources, float ml_depth, int adiabat, const int *start_3d, int nk,
                      int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out,
                      int *status, long long *counters, void *workspace, size_t workspace_bytes,
                      void *stream) {
  if (nsrc < 1 || nsrc > 3) return fail(XC_ERR_INVALID, "nsrc=%d outside 1..3", nsrc);
  if (!sources) return fail(XC_ERR_INVALID, "NULL sources");
  return lift_sources(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, nsrc, sources, ml_depth,
                      adiabat, start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, counters,
                      workspace, workspace_bytes, stream);
}

int xc_loopcape_diag(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                     const void *ts, const void *tds, int dtype, float pinc, int source,
                     float ml_depth, int adiabat, const int *start_3d, int nk, int n2, int guess,
                     float *cape, float *cin, int *mulvl, float *z_out, int *status, float *diag,
                     void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  rc = check_cape_opts(pinc, source, ml_depth, adiabat);
  if (rc) return rc;
  if (grid < 1 || grid > 3) return fail(XC_ERR_INVALID, "grid must be 1, 2 or 3");
  if (grid == 3 && !start_3d) return fail(XC_ERR_INVALID, "grid 3 needs start_3d");
  if (guess != XC_GUESS_PLAIN && guess != XC_GUESS_LEARNED)
    return fail(XC_ERR_INVALID, "xc_loopcape_diag: guess must be XC_GUESS_PLAIN or _LEARNED");
  const float *guess_w = nullptr;
  if (guess == XC_GUESS_LEARNED) {
    rc = guess_weights(&guess_w);
    if (rc) return rc;
  }
  if (n2 == 0) return XC_OK;
  if (!p || !t3d || !td3d || !ps || !ts || !tds || !cape || !cin || !mulvl || !z_out || !diag)
    return fail(XC_ERR_INVALID, "NULL array argument");
  xc::CapeArgs a;
  a.grid = grid;
  a.dtype = dtype;
  a.p = p;
  a.t = t3d;
  a.td = td3d;
  a.ps = ps;
  a.ts = ts;
  a.tds = tds;
  a.start = grid == 1 ? nullptr : start_3d;
  a.pinc = pinc;
  a.source = source;
  a.ml_depth = ml_depth;
  a.adiabat = adiabat;
  a.nk = nk;
  a.n2 = n2;
  a.guess = guess;
  a.cape = cape;
  a.cin = cin;
  a.mulvl = mulvl;
  a.z_out = z_out;
  a.status = status;
  a.counters = nullptr;
  a.perm = nullptr;
  a.guess_w = guess_w;
  a.diag = diag;
  const cudaError_t e = xc::launch_cape_diag(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cape diagnostics kernel launch");
  return XC_OK;
}

int xc_loopcape_ml(const void *p3d, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, int nk, int n2, float *cape, float *cin,
                   int *mulvl, float *z_out, int *status, void *stream) {
  return xc_loopcape_ex(1, p3d, t3d, td3d, ps, ts, tds, dtype, pinc, source, ml_depth, adiabat,
                        nullptr, nk, n2, XC_GUESS_PLAIN, cape, cin, mulvl, z_out, status, nullptr,
                        nullptr, 0, stream);
}

int xc_loopcape_pl1d(const void *t3d, const void *td3d, const void *p1d, const void *ps,
                     const void *ts, const void *tds, int dtype, float pinc, int source,
                     float ml_depth, int adiabat, const int *start_3d, int nk, int n2,
                     float *cape, float *cin, int *mulvl, float *z_out, int *status,
                     void *stream) {
  return xc_loopcape_ex(2, p1d, t3d, td3d, ps, ts, tds, dtype, pinc, source, ml_depth, adiabat,
                        start_3d, nk, n2, XC_GUESS_PLAIN, cape, cin, mulvl, z_out, status,
                        nullptr, nullptr, 0, stream);
}

int xc_loopcape_pl(const void *p3d, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, const int *start_3d, int nk, int n2,
                   float *cape, float *cin, int *mulvl, float *z_out, int *status,
                   void *stream) {
  return xc_loopcape_ex(3, p3d, t3d, td3d, ps, ts, tds, dtype, pinc, source, ml_depth, adiabat,
                        start_3d, nk, n2, XC_GUESS_PLAIN, cape, cin, mulvl, z_out, status,
                        nullptr, nullptr, 0, stream);
}


}  // extern "C"

namespace {

// The host-pointer CAPE path for nsrc sources of the same columns.  The
// columns go through in chunks.  One stream copies the chunks' inputs in
// order, once for all the sources; once a chunk's inputs are in, its
// ordering runs on the priority stream, its first source's lift and its
// output copies on one of host_streams() compute streams, in turn, and the
// other sources' lifts on the side streams.  So copies overlap lifts and
// one chunk's last warps overlap the next chunks' first.  Every chunk has
// its own device slot when the ring budget allows (the usual case), and
// then the calling thread queues the whole call without waiting.  Outputs
// come back into pinned staging (a copy into pageable memory would block
// this thread) and are moved into the caller's arrays by the copy threads
// as the chunks land, or when a slot is reused.  The column ordering depends
// only on the start level and the surface dewpoint, not on the source, so
// one ordering per chunk serves every source.  Each column is still computed
// by one thread and written to its own index, so neither the chunking nor
// the number of sources changes a result.  Outputs are [nsrc][n2].
int host_lift(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
              const void *ts, const void *tds, int dtype, float pinc, int nsrc,
              const int *sources, float ml_depth, int adiabat, const int *start_3d, int nk,
              int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out, int *status,
              void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  if (nsrc < 1 || nsrc > 3 || !sources) return fail(XC_ERR_INVALID, "nsrc must be 1..3 with a source list");
  for (int j = 0; j < nsrc; ++j) {
    rc = check_cape_opts(pinc, sources[j], ml_depth, adiabat);
    if (rc) return rc;
  }
  if (grid < 1 || grid > 3) return fail(XC_ERR_INVALID, "grid must be 1, 2 or 3");
  if (grid == 3 && !start_3d) return fail(XC_ERR_INVALID, "grid 3 needs start_3d");
  const bool retry = (guess & XC_RETRY_FP64) != 0;
  guess &= ~XC_RETRY_FP64;
  if (guess < XC_GUESS_PLAIN || guess > XC_GUESS_LEARNED_WARP)
    return fail(XC_ERR_INVALID, "guess %d is not one of XC_GUESS_*", guess);
  const float *guess_w = nullptr;
  if (guess == XC_GUESS_LEARNED || guess == XC_GUESS_LEARNED_EVERY ||
      guess == XC_GUESS_LEARNED_WARP) {
    rc = guess_weights(&guess_w);
    if (rc) return rc;
  }
  if (n2 == 0) return XC_OK;
  if (!p || !t3d || !td3d || !ps || !ts || !tds || !cape || !cin || !mulvl || !z_out)
    return fail(XC_ERR_INVALID, "NULL array argument");
  int nchunk = (n2 + HOST_CHUNK_MIN - 1) / HOST_CHUNK_MIN;
  if (nchunk > host_chunks()) nchunk = host_chunks();
  // Chunk c holds columns [bound[c], bound[c + 1]).  With three or more
  // chunks the first and the last are half-size: the first lift starts
  // after a shorter copy, and less work is left after the last copy.
  long long bound[HOST_CHUNKS + 1];
  bound[0] = 0;
  for (int c = 1; c < nchunk; ++c) {
    const double w = nchunk >= 3 ? (c - 0.5) / (nchunk - 1) : (double)c / nchunk;
    long long b = ((long long)(w * n2) + 255) / 256 * 256;
    if (b < bound[c - 1]) b = bound[c - 1];
    if (b > n2) b = n2;
    bound[c] = b;
  }
  bound[nchunk] = n2;
  int C = 256;  // columns per slot: the largest chunk
  for (int c = 0; c < nchunk; ++c)
    if (bound[c + 1] - bound[c] > C) C = (int)(bound[c + 1] - bound[c]);
  const size_t es = dtype == XC_F32 ? 4 : 8;
  const size_t c3 = (size_t)C * nk;
  const bool has_start = grid != 1 && start_3d;
  // cape, cin, mulvl, z_out (, status: the caller's, or the retry's flags) per source
  const int nout = (status || retry) ? 5 : 4;
  HostCtxLease lease;
  rc = lease.acquire();
  if (rc) return rc;
  HostCtx *pl = lease.c;
  struct Slot {
    size_t p, t, td, ps, ts, tds, st, out, ord;
  } sl[HOST_CHUNKS];
  const size_t ord_bytes = xc::order_workspace_bytes(C);
  const size_t out_bytes = (size_t)nsrc * nout * C * 4;  // [nsrc][nout][C]
  auto carve = [&](Carver &cv, Slot &q) {
    q.p = cv.take((grid == 2 ? (size_t)nk : c3) * es);
    q.t = cv.take(c3 * es);
    q.td = cv.take(c3 * es);
    q.ps = cv.take((size_t)C * es);
    q.ts = cv.take((size_t)C * es);
    q.tds = cv.take((size_t)C * es);
    q.st = has_start ? cv.take((size_t)C * 4) : 0;
    q.out = cv.take(out_bytes);
    q.ord = cv.take(ord_bytes);
  };
  size_t slot_bytes = 0;
  {
    Carver one;
    Slot q;
    carve(one, q);
    slot_bytes = one.off;
  }
  int nslot = (int)(host_ring_bytes() / slot_bytes);
  if (nslot < 2) nslot = 2;
  if (nslot > nchunk) nslot = nchunk;
  Carver cv;
  for (int k = 0; k < nslot; ++k) carve(cv, sl[k]);
  void *base = nullptr;
  rc = ctx_workspace(pl, cv.off, &base);
  if (rc) return rc;
  char *b = (char *)base;
  rc = ctx_pinned(pl, out_bytes * nslot);
  if (rc) return rc;
  // output array j of source s in a slot (device or its pinned staging)
  auto out_off = [&](int s_, int j) { return ((size_t)s_ * nout + j) * C * 4; };
  // moves columns [lo, hi) of chunk c's outputs from its slot's staging
  // into the caller's arrays, once the chunk's output copies are done
  auto copy_out = [&](int c, size_t lo, size_t hi) -> cudaError_t {
    const int k = c % nslot;
    const cudaError_t we = cudaEventSynchronize(pl->done[k]);
    if (we != cudaSuccess) return we;
    const size_t o0 = (size_t)bound[c] + lo, nb = (hi - lo) * 4;
    const char *h = pl->pinned + k * out_bytes + lo * 4;
    for (int s_ = 0; s_ < nsrc; ++s_) {
      const size_t o = (size_t)s_ * n2 + o0;
      memcpy(cape + o, h + out_off(s_, 0), nb);
      memcpy(cin + o, h + out_off(s_, 1), nb);
      memcpy(mulvl + o, h + out_off(s_, 2), nb);
      memcpy(z_out + o, h + out_off(s_, 3), nb);
      if (status) memcpy(status + o, h + out_off(s_, 4), nb);
    }
    return cudaSuccess;
  };
  // chunk c's outputs into the caller's arrays: split over the copy pool's
  // threads (finish_all waits for them), or in this thread
  CopyPool *pool = copy_pool();
  CopyBatch batch;
  const int dev = pl->dev;
  auto finish = [&](int c) -> int {
    const size_t nc = (size_t)(bound[c + 1] - bound[c]);
    if (!pool) {
      const cudaError_t we = copy_out(c, 0, nc);
      return we == cudaSuccess ? XC_OK : cuda_fail(we, "device-to-host copy");
    }
    const int parts = host_copy_threads();
    for (int j = 0; j < parts; ++j) {
      const size_t lo = nc * j / parts, hi = nc * (j + 1) / parts;
      if (hi > lo)
        pool->submit(&batch, [&copy_out, dev, c, lo, hi]() {
          cudaSetDevice(dev);
          return copy_out(c, lo, hi);
        });
    }
    return XC_OK;
  };
  auto finish_all = [&]() -> int {
    if (!pool) return XC_OK;
    batch.wait();
    return batch.err == cudaSuccess ? XC_OK : cuda_fail(batch.err, "device-to-host copy");
  };
  cudaError_t e = cudaEventRecord(pl->start, (cudaStream_t)stream);
  const int nstream = host_streams();
  for (int k = 0; k < nstream && e == cudaSuccess; ++k)
    e = cudaStreamWaitEvent(pl->s[k], pl->start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(pl->copy, pl->start, 0);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(pl->ord, pl->start, 0);
  for (int j = 0; j < 2 && e == cudaSuccess; ++j) e = cudaStreamWaitEvent(pl->side[j], pl->start, 0);
  if (e != cudaSuccess) return cuda_fail(e, "ordering the host path after the caller's stream");
  const char *hp = (const char *)p, *ht = (const char *)t3d, *htd = (const char *)td3d;
  const char *hps = (const char *)ps, *hts = (const char *)ts, *htds = (const char *)tds;
  int issued = 0;
  for (int c = 0; c < nchunk; ++c) {
    const long long c0 = bound[c];
    const int nc = (int)(bound[c + 1] - bound[c]);  // never 0: chunks of 2+ hold 65,536+
    const int k = c % nslot;
    if (c >= nslot) {
      // the slot still holds chunk c - nslot: its outputs leave the staging
      // first, and its lifts (before its output copies) are done with the inputs
      rc = finish(c - nslot);
      if (!rc) rc = finish_all();
      if (rc) return rc;
    }
    const Slot &q = sl[k];
    cudaStream_t s = pl->s[c % nstream];
    const size_t r3 = (size_t)nc * nk * es, off3 = (size_t)c0 * nk * es, off1 = (size_t)c0 * es;
#define H2D(off, src, bytes)                                                         \
    if (e == cudaSuccess)                                                            \
      e = cudaMemcpyAsync(b + (off), (src), (bytes), cudaMemcpyHostToDevice, pl->copy)
    // first what the ordering reads (the surface values, the start levels,
    // the 1-D pressures), so that the chunk's ordering runs while its
    // profiles are still crossing
    if (grid == 2) H2D(q.p, hp, (size_t)nk * es);
    H2D(q.ps, hps + off1, (size_t)nc * es);
    H2D(q.ts, hts + off1, (size_t)nc * es);
    H2D(q.tds, htds + off1, (size_t)nc * es);
    if (has_start) H2D(q.st, start_3d + c0, (size_t)nc * 4);
    if (e == cudaSuccess) e = cudaEventRecord(pl->surf[k], pl->copy);
    if (grid != 2) H2D(q.p, hp + off3, r3);
    H2D(q.t, ht + off3, r3);
    H2D(q.td, htd + off3, r3);
#undef H2D
    if (e == cudaSuccess) e = cudaEventRecord(pl->loaded[k], pl->copy);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(pl->ord, pl->surf[k], 0);
    if (e != cudaSuccess) return cuda_fail(e, "host-to-device copy");
    xc::CapeArgs a;
    a.grid = grid;
    a.dtype = dtype;
    a.p = b + q.p;
    a.t = b + q.t;
    a.td = b + q.td;
    a.ps = b + q.ps;
    a.ts = b + q.ts;
    a.tds = b + q.tds;
    a.start = has_start ? (const int *)(b + q.st) : nullptr;
    a.pinc = pinc;
    a.ml_depth = ml_depth;
    a.adiabat = adiabat;
    a.nk = nk;
    a.n2 = nc;
    a.guess = guess;
    a.counters = nullptr;
    a.perm = nullptr;
    a.guess_w = guess_w;
    e = xc::launch_order(a, b + q.ord, &a.perm, pl->ord);
    if (e == cudaSuccess) e = cudaEventRecord(pl->ordered[k], pl->ord);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, pl->ordered[k], 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, pl->loaded[k], 0);
    if (e != cudaSuccess) return cuda_fail(e, "column ordering launch");
    auto point = [&](int s_) {
      char *o = b + q.out;
      a.source = sources[s_];
      a.cape = (float *)(o + out_off(s_, 0));
      a.cin = (float *)(o + out_off(s_, 1));
      a.mulvl = (int *)(o + out_off(s_, 2));
      a.z_out = (float *)(o + out_off(s_, 3));
      a.status = nout == 5 ? (int *)(o + out_off(s_, 4)) : nullptr;
    };
    for (int s_ = 1; s_ < nsrc && e == cudaSuccess; ++s_) {
      e = cudaStreamWaitEvent(pl->side[s_ - 1], pl->ordered[k], 0);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(pl->side[s_ - 1], pl->loaded[k], 0);
    }
    for (int s_ = 0; s_ < nsrc && e == cudaSuccess; ++s_) {
      point(s_);
      e = xc::launch_cape(a, s_ == 0 ? s : pl->side[s_ - 1]);
      if (e == cudaSuccess && s_ > 0) e = cudaEventRecord(pl->lifted[k][s_ - 1], pl->side[s_ - 1]);
      if (e == cudaSuccess && s_ > 0) e = cudaStreamWaitEvent(s, pl->lifted[k][s_ - 1], 0);
    }
    if (e != cudaSuccess) return cuda_fail(e, "cape kernel launch");
    // the FP64 retries come after every source's lift: each reuses the
    // ordering workspace, which the lifts read
    for (int s_ = 0; retry && s_ < nsrc; ++s_) {
      point(s_);
      e = xc::launch_retry64(a, b + q.ord, s);
      if (e != cudaSuccess) return cuda_fail(e, "FP64 retry launch");
    }
    // copies of the slot's outputs: [nsrc][nout][C], of which the first nc
    // entries of each array are this chunk's (the status only if asked for)
    char *h = pl->pinned + k * out_bytes;
    for (int j = 0; j < nsrc * nout && e == cudaSuccess; ++j)
      if (j % nout < 4 || status)
        e = cudaMemcpyAsync(h + (size_t)j * C * 4, b + q.out + (size_t)j * C * 4,
                            (size_t)nc * 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaEventRecord(pl->done[k], s);
    if (e != cudaSuccess) return cuda_fail(e, "device-to-host copy");
    issued = c + 1;
  }
  for (int c = issued - nslot < 0 ? 0 : issued - nslot; c < issued; ++c) {
    rc = finish(c);
    if (rc) return rc;
  }
  return finish_all();
}

}  // namespace

extern "C" {

int xc_loopcape_ex_host(int grid, const void *p, const void *t3d, const void *td3d,
                        const void *ps, const void *ts, const void *tds, int dtype, float pinc,
                        int source, float ml_depth, int adiabat, const int *start_3d, int nk,
                        int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out,
                        int *status, void *stream) {
  return host_lift(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, 1, &source, ml_depth, adiabat,
                   start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, stream);
}

int xc_loopcape_multi_host(int grid, const void *p, const void *t3d, const void *td3d,
                           const void *ps, const void *ts, const void *tds, int dtype, float pinc,
                           int nsrc, const int *sources, float ml_depth, int adiabat,
                           const int *start_3d, int nk, int n2, int guess, float *cape,
                           float *cin, int *mulvl, float *z_out, int *status, void *stream) {
  return host_lift(grid, p, t3d, td3d, ps, ts, tds, dtype, pinc, nsrc, sources, ml_depth, adiabat,
                   start_3d, nk, n2, guess, cape, cin, mulvl, z_out, status, stream);
}

int xc_calc_srh(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                const void *v3d, const void *ps, const void *ts, const void *tds,
                const void *us, const void *vs, int dtype, const int *start_3d, double depth,
                double aglh0, int nk, int n2, double *srh_rm, double *srh_lm, float *rm,
                float *lm, float *mean6, void *stream) {
  return xc_calc_srh_ex(grid, p, t3d, td3d, u3d, v3d, ps, ts, tds, us, vs, dtype, start_3d, depth,
                        aglh0, nk, n2, XC_SRH_REFERENCE, srh_rm, srh_lm, rm, lm, mean6, stream);
}

int xc_calc_srh_ex(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                   const void *v3d, const void *ps, const void *ts, const void *tds,
                   const void *us, const void *vs, int dtype, const int *start_3d, double depth,
                   double aglh0, int nk, int n2, int precision, double *srh_rm, double *srh_lm,
                   float *rm, float *lm, float *mean6, void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  if (grid != 1 && grid != 2) return fail(XC_ERR_INVALID, "grid must be 1 (sigma) or 2 (pressure, 1-D p)");
  if (precision != XC_SRH_REFERENCE && precision != XC_SRH_FP32)
    return fail(XC_ERR_INVALID, "precision must be XC_SRH_REFERENCE or XC_SRH_FP32");
  if ((rm == nullptr) != (lm == nullptr) || (rm == nullptr) != (mean6 == nullptr))
    return fail(XC_ERR_INVALID, "rm, lm and mean6 must be all NULL or all set");
  if (n2 == 0) return XC_OK;
  if (!p || !t3d || !td3d || !u3d || !v3d || !ps || !ts || !tds || !us || !vs || !srh_rm || !srh_lm)
    return fail(XC_ERR_INVALID, "NULL array argument");
  xc::SrhArgs a;
  a.grid = grid;
  a.dtype = dtype;
  a.p = p;
  a.t = t3d;
  a.td = td3d;
  a.u = u3d;
  a.v = v3d;
  a.ps = ps;
  a.ts = ts;
  a.tds = tds;
  a.us = us;
  a.vs = vs;
  a.start = grid == 2 ? start_3d : nullptr;
  a.depth = depth;
  a.aglh0 = aglh0;
  a.nk = nk;
  a.n2 = n2;
  a.srh_rm = srh_rm;
  a.srh_lm = srh_lm;
  a.rm = rm;
  a.lm = lm;
  a.mean6 = mean6;
  a.precision = precision;
  cudaError_t e = xc::launch_srh(a, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "srh kernel launch");
  return XC_OK;
}

int xc_cape_srh(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                const void *v3d, const void *ps, const void *ts, const void *tds, const void *us,
                const void *vs, int dtype, float pinc, int source, float ml_depth, int adiabat,
                const int *start_3d, double depth, double aglh0, int nk, int n2, int guess,
                int precision, float *cape, float *cin, int *mulvl, float *z_out, int *status,
                double *srh_rm, double *srh_lm, float *rm, float *lm, float *mean6,
                void *workspace, size_t workspace_bytes, void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  rc = check_cape_opts(pinc, source, ml_depth, adiabat);
  if (rc) return rc;
  if (grid != 1 && grid != 2) return fail(XC_ERR_INVALID, "grid must be 1 (sigma) or 2 (pressure, 1-D p)");
  if (guess != XC_GUESS_PLAIN && guess != XC_GUESS_LEARNED)
    return fail(XC_ERR_INVALID, "xc_cape_srh: guess must be XC_GUESS_PLAIN or XC_GUESS_LEARNED");
  if (precision != XC_SRH_REFERENCE && precision != XC_SRH_FP32)
    return fail(XC_ERR_INVALID, "precision must be XC_SRH_REFERENCE or XC_SRH_FP32");
  if ((rm == nullptr) != (lm == nullptr) || (rm == nullptr) != (mean6 == nullptr))
    return fail(XC_ERR_INVALID, "rm, lm and mean6 must be all NULL or all set");
  const float *guess_w = nullptr;
  if (guess == XC_GUESS_LEARNED) {
    rc = guess_weights(&guess_w);
    if (rc) return rc;
  }
  if (n2 == 0) return XC_OK;
  if (!p || !t3d || !td3d || !u3d || !v3d || !ps || !ts || !tds || !us || !vs || !cape || !cin ||
      !mulvl || !z_out || !srh_rm || !srh_lm)
    return fail(XC_ERR_INVALID, "NULL array argument");
  xc::CapeArgs a;
  a.grid = grid;
  a.dtype = dtype;
  a.p = p;
  a.t = t3d;
  a.td = td3d;
  a.ps = ps;
  a.ts = ts;
  a.tds = tds;
  a.start = grid == 2 ? start_3d : nullptr;
  a.pinc = pinc;
  a.source = source;
  a.ml_depth = ml_depth;
  a.adiabat = adiabat;
  a.nk = nk;
  a.n2 = n2;
  a.guess = guess;
  a.cape = cape;
  a.cin = cin;
  a.mulvl = mulvl;
  a.z_out = z_out;
  a.status = status;
  a.counters = nullptr;
  a.perm = nullptr;
  a.guess_w = guess_w;
  xc::SrhArgs h;
  h.grid = grid;
  h.dtype = dtype;
  h.p = p;
  h.t = t3d;
  h.td = td3d;
  h.u = u3d;
  h.v = v3d;
  h.ps = ps;
  h.ts = ts;
  h.tds = tds;
  h.us = us;
  h.vs = vs;
  h.start = a.start;
  h.depth = depth;
  h.aglh0 = aglh0;
  h.nk = nk;
  h.n2 = n2;
  h.srh_rm = srh_rm;
  h.srh_lm = srh_lm;
  h.rm = rm;
  h.lm = lm;
  h.mean6 = mean6;
  h.precision = precision;
  cudaError_t e = cudaSuccess;
  if (workspace) {
    if (workspace_bytes < xc::order_workspace_bytes(n2))
      return fail(XC_ERR_INVALID, "workspace of %zu bytes is smaller than the %zu needed",
                  workspace_bytes, xc::order_workspace_bytes(n2));
    if (((size_t)workspace & 255) != 0) return fail(XC_ERR_INVALID, "workspace must be 256-byte aligned");
    e = xc::launch_order(a, workspace, &a.perm, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "column ordering launch");
  }
  if (precision == XC_SRH_FP32 && dtype == XC_F32) {
    // With the FP32 SRH stages and f32 inputs the SRH part runs the
    // level-parallel kernel of calc_srh (eight lanes per column, coalesced
    // reads, no staging), which a fused kernel's one-thread walk of the
    // ordered (scattered) columns cannot match: the lift and that kernel run
    // back to back, and their results are those of the two calls.  With the
    // FP64 SRH stages, or f64 inputs, the fused kernel lets the lift and the
    // FP64 stages share the SMs.
    e = xc::launch_cape(a, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cape kernel launch");
    e = xc::launch_srh(h, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "srh kernel launch");
    return XC_OK;
  }
  e = xc::launch_cape_srh(a, h, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cape + srh kernel launch");
  return XC_OK;
}

int xc_calc_srh_host(int grid, const void *p, const void *t3d, const void *td3d,
                     const void *u3d, const void *v3d, const void *ps, const void *ts,
                     const void *tds, const void *us, const void *vs, int dtype,
                     const int *start_3d, double depth, double aglh0, int nk, int n2,
                     int precision, double *srh_rm, double *srh_lm, float *rm, float *lm,
                     float *mean6, void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  if (grid != 1 && grid != 2) return fail(XC_ERR_INVALID, "grid must be 1 or 2");
  if ((rm == nullptr) != (lm == nullptr) || (rm == nullptr) != (mean6 == nullptr))
    return fail(XC_ERR_INVALID, "rm, lm and mean6 must be all NULL or all set");
  if (n2 == 0) return XC_OK;
  const size_t es = dtype == XC_F32 ? 4 : 8;
  const size_t n3 = (size_t)n2 * nk;
  const size_t p_bytes = (grid == 2 ? (size_t)nk : n3) * es;
  HostCtxLease lease;
  rc = lease.acquire();
  if (rc) return rc;
  Carver cv;
  const size_t o_p = cv.take(p_bytes), o_t = cv.take(n3 * es), o_td = cv.take(n3 * es),
               o_u = cv.take(n3 * es), o_v = cv.take(n3 * es);
  const size_t o_ps = cv.take(n2 * es), o_ts = cv.take(n2 * es), o_tds = cv.take(n2 * es),
               o_us = cv.take(n2 * es), o_vs = cv.take(n2 * es);
  const size_t o_st = (grid == 2 && start_3d) ? cv.take(n2 * 4) : 0;
  const size_t o_srm = cv.take(n2 * 8), o_slm = cv.take(n2 * 8);
  const size_t o_rm = rm ? cv.take(n2 * 8) : 0, o_lm = rm ? cv.take(n2 * 8) : 0,
               o_mean = rm ? cv.take(n2 * 8) : 0;
  void *base = nullptr;
  rc = ctx_workspace(lease.c, cv.off, &base);
  if (rc) return rc;
  char *b = (char *)base;
  // on the context's first stream, after the caller's stream, so that
  // concurrent calls from several threads overlap on the GPU
  cudaStream_t s = lease.c->s[0];
  cudaError_t e0 = cudaEventRecord(lease.c->start, (cudaStream_t)stream);
  if (e0 == cudaSuccess) e0 = cudaStreamWaitEvent(s, lease.c->start, 0);
  if (e0 != cudaSuccess) return cuda_fail(e0, "ordering the host path after the caller's stream");
  cudaError_t e = cudaSuccess;
#define H2D(off, src, bytes)                                                         \
  if (e == cudaSuccess) e = cudaMemcpyAsync(b + (off), (src), (bytes), cudaMemcpyHostToDevice, s)
  H2D(o_p, p, p_bytes);
  H2D(o_t, t3d, n3 * es);
  H2D(o_td, td3d, n3 * es);
  H2D(o_u, u3d, n3 * es);
  H2D(o_v, v3d, n3 * es);
  H2D(o_ps, ps, n2 * es);
  H2D(o_ts, ts, n2 * es);
  H2D(o_tds, tds, n2 * es);
  H2D(o_us, us, n2 * es);
  H2D(o_vs, vs, n2 * es);
  if (grid == 2 && start_3d) H2D(o_st, start_3d, n2 * 4);
#undef H2D
  if (e != cudaSuccess) return cuda_fail(e, "host-to-device copy");
  rc = xc_calc_srh_ex(grid, b + o_p, b + o_t, b + o_td, b + o_u, b + o_v, b + o_ps, b + o_ts,
                      b + o_tds, b + o_us, b + o_vs, dtype,
                      (grid == 2 && start_3d) ? (const int *)(b + o_st) : nullptr, depth, aglh0,
                      nk, n2, precision, (double *)(b + o_srm), (double *)(b + o_slm),
                      rm ? (float *)(b + o_rm) : nullptr, rm ? (float *)(b + o_lm) : nullptr,
                      rm ? (float *)(b + o_mean) : nullptr, s);
  if (rc) return rc;
#define D2H(dst, off, bytes)                                                         \
  if (e == cudaSuccess) e = cudaMemcpyAsync((dst), b + (off), (bytes), cudaMemcpyDeviceToHost, s)
  D2H(srh_rm, o_srm, n2 * 8);
  D2H(srh_lm, o_slm, n2 * 8);
  if (rm) {
    D2H(rm, o_rm, n2 * 8);
    D2H(lm, o_lm, n2 * 8);
    D2H(mean6, o_mean, n2 * 8);
  }
#undef D2H
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "device-to-host copy");
  return XC_OK;
}

int xc_loop_stdheight_ml(const double *P, const double *T, const double *Td, const double *Ps,
                         const double *Ts, const double *Tds, const double *Hin, int NK, int NX,
                         double *H, double *Hs, void *stream) {
  int rc = check_common(XC_F64, NK, NX);
  if (rc) return rc;
  cudaError_t e = xc::launch_stdheight(P, NK, T, Td, Ps, Ts, Tds, Hin, nullptr, NK, NX, H, Hs,
                                       (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "stdheight kernel launch");
}

int xc_loop_stdheight_pl1d(const double *T, const double *Td, const double *P, const double *Ps,
                           const double *Ts, const double *Tds, const double *Hin,
                           const int *start_3d, int NK, int NX, double *H, double *Hs,
                           void *stream) {
  int rc = check_common(XC_F64, NK, NX);
  if (rc) return rc;
  if (!start_3d) return fail(XC_ERR_INVALID, "start_3d is required");
  cudaError_t e = xc::launch_stdheight(P, 0, T, Td, Ps, Ts, Tds, Hin, start_3d, NK, NX, H, Hs,
                                       (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "stdheight kernel launch");
}

int xc_loop_stdheight_pl(const double *P, const double *T, const double *Td, const double *Ps,
                         const double *Ts, const double *Tds, const double *Hin,
                         const int *start_3d, int NK, int NX, double *H, double *Hs,
                         void *stream) {
  int rc = check_common(XC_F64, NK, NX);
  if (rc) return rc;
  if (!start_3d) return fail(XC_ERR_INVALID, "start_3d is required");
  cudaError_t e = xc::launch_stdheight(P, NK, T, Td, Ps, Ts, Tds, Hin, start_3d, NK, NX, H, Hs,
                                       (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "stdheight kernel launch");
}

int xc_bunkers_loop_ml(const float *U3d, const float *V3d, const float *AGLH3d, const float *Us,
                       const float *Vs, const float *AGLHs, int nk, int n2, float *RM, float *LM,
                       float *Mean6kmwind, void *stream) {
  int rc = check_common(XC_F32, nk, n2);
  if (rc) return rc;
  cudaError_t e = xc::launch_bunkers(U3d, V3d, AGLH3d, Us, Vs, AGLHs, nullptr, nk, n2, RM, LM,
                                     Mean6kmwind, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "bunkers kernel launch");
}

int xc_bunkers_loop_pl(const float *U3d, const float *V3d, const float *AGLH3d, const float *Us,
                       const float *Vs, const float *AGLHs, const int *start_3d, int nk, int n2,
                       float *RM, float *LM, float *Mean6kmwind, void *stream) {
  int rc = check_common(XC_F32, nk, n2);
  if (rc) return rc;
  if (!start_3d) return fail(XC_ERR_INVALID, "start_3d is required");
  cudaError_t e = xc::launch_bunkers(U3d, V3d, AGLH3d, Us, Vs, AGLHs, start_3d, nk, n2, RM, LM,
                                     Mean6kmwind, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "bunkers kernel launch");
}

int xc_loop_sreh_ml(const double *u, const double *v, const double *aglh, const double *us,
                    const double *vs, const double *aglhs, const double *cu_rm,
                    const double *cv_rm, const double *cu_lm, const double *cv_lm, double top,
                    int nk, int n2, double *sreh_rm, double *sreh_lm, void *stream) {
  int rc = check_common(XC_F64, nk, n2);
  if (rc) return rc;
  cudaError_t e = xc::launch_sreh(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top,
                                  nullptr, nk, n2, sreh_rm, sreh_lm, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "sreh kernel launch");
}

int xc_loop_sreh_pl(const double *u, const double *v, const double *aglh, const double *us,
                    const double *vs, const double *aglhs, const double *cu_rm,
                    const double *cv_rm, const double *cu_lm, const double *cv_lm, double top,
                    const int *start_3d, int nk, int n2, double *sreh_rm, double *sreh_lm,
                    void *stream) {
  int rc = check_common(XC_F64, nk, n2);
  if (rc) return rc;
  if (!start_3d) return fail(XC_ERR_INVALID, "start_3d is required");
  cudaError_t e = xc::launch_sreh(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top,
                                  start_3d, nk, n2, sreh_rm, sreh_lm, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "sreh kernel launch");
}

int xc_pres_lev_pos(const void *p1d, const void *ps, int dtype, int nk, int n2, int *start_3d,
                    void *stream) {
  int rc = check_common(dtype, nk, n2);
  if (rc) return rc;
  if (n2 == 0) return XC_OK;
  cudaError_t e = xc::launch_pres_lev_pos(p1d, ps, dtype, nk, n2, start_3d, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "pres_lev_pos kernel launch");
}

}  // extern "C"

extern "C" {

int xc_guess_set_weights(const float *weights, int on_device, void *stream) {
  if (!weights) return fail(XC_ERR_INVALID, "NULL weights");
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxGuessDevices) return fail(XC_ERR_INVALID, "device %d out of range", dev);
  e = cudaMemcpyToSymbolAsync(g_guess_w, weights, sizeof(float) * XC_GUESS_NPARAM, 0,
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              (cudaStream_t)stream);
  void *gw = nullptr;
  if (e == cudaSuccess) e = cudaGetSymbolAddress(&gw, g_guess_w);
  if (e == cudaSuccess) e = xc::build_warp_net((const float *)gw, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "loading the guess network");
  std::lock_guard<std::mutex> lk(g_guess_mu);
  g_guess_loaded[dev] = true;
  return XC_OK;
}

int xc_guess_pairs(long long n, unsigned long long seed, float *feats, float *targets, int *iters,
                   void *stream) {
  if (n < 0) return fail(XC_ERR_INVALID, "n is negative");
  if (n > 0 && (!feats || !targets || !iters)) return fail(XC_ERR_INVALID, "NULL array argument");
  cudaError_t e = xc::launch_guess_pairs(n, seed, feats, targets, iters, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "guess pair kernel launch");
}

int xc_guess_grad(const float *weights, const float *feats, const float *targets, long long n,
                  float *grad, float *loss, void *stream) {
  if (n < 0) return fail(XC_ERR_INVALID, "n is negative");
  if (n > 0 && (!weights || !feats || !targets || !grad || !loss))
    return fail(XC_ERR_INVALID, "NULL array argument");
  cudaError_t e = xc::launch_guess_grad(weights, feats, targets, 0, n, grad, loss,
                                        (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "guess training kernel launch");
}

int xc_guess_grad_tc(const float *weights, const float *feats, const float *targets,
                     long long n, float *grad, float *loss, int *status, void *stream) {
  if (n < 0) return fail(XC_ERR_INVALID, "n is negative");
  if (n > 0 && (!weights || !feats || !targets || !grad || !loss))
    return fail(XC_ERR_INVALID, "NULL array argument");
  cudaError_t e = xc::launch_guess_grad_tc(weights, feats, targets, 0, n, grad, loss, status,
                                           (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "guess training kernel (tcgen05) launch");
}

int xc_guess_adam(float *weights, float *grad, float *m, float *v, float lr, int step,
                  void *stream) {
  if (!weights || !grad || !m || !v || step < 1) return fail(XC_ERR_INVALID, "bad Adam arguments");
  cudaError_t e = xc::launch_guess_adam(weights, grad, m, v, lr, step, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "Adam kernel launch");
}

int xc_guess_eval(const float *weights, const float *feats, long long n, float *out,
                  void *stream) {
  if (n < 0) return fail(XC_ERR_INVALID, "n is negative");
  if (n > 0 && (!weights || !feats || !out)) return fail(XC_ERR_INVALID, "NULL array argument");
  cudaError_t e = xc::launch_guess_eval(weights, feats, n, out, (cudaStream_t)stream);
  return e == cudaSuccess ? XC_OK : cuda_fail(e, "guess inference kernel launch");
}

}  // extern "C"

namespace xc {
// Records `msg` as the calling thread's xc_last_error() text; returns code.
int set_error(int code, const char *msg) {
  snprintf(g_err, sizeof(g_err), "%s", msg);
  return code;
}
cudaError_t dev_malloc(void **p, size_t bytes) {
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e == cudaSuccess) g_allocs.fetch_add(1, std::memory_order_relaxed);
  return e;
}
cudaError_t host_malloc(void **p, size_t bytes) {
  const cudaError_t e = cudaMallocHost(p, bytes);
  if (e == cudaSuccess) g_allocs.fetch_add(1, std::memory_order_relaxed);
  return e;
}
// For the batch executor (batch.cu): the loaded guess network, and the
// option checks of the single-request entry points.
int guess_weights_ptr(const float **out) { return guess_weights(out); }
int check_cape_options(float pinc, int source, float ml_depth, int adiabat) {
  return check_cape_opts(pinc, source, ml_depth, adiabat);
}
}  // namespace xc
