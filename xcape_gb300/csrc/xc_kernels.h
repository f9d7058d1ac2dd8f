// xc_kernels.h -- launch interface between the C ABI (capi.cu) and the kernels.
#pragma once
#include <atomic>
#include <cuda_runtime.h>

namespace xc {

struct CapeArgs {
  int grid;   // 1 sigma/model (p per column), 2 pressure with shared p1d, 3 pressure per column
  int dtype;  // 0 f32 inputs, 1 f64 inputs
  const void *p, *t, *td, *ps, *ts, *tds;
  const int *start;  // nullable for grid 2 (derived in the kernel)
  float pinc;
  int source;
  float ml_depth;
  int adiabat;
  int nk;
  long long n2;
  long long ld = 0;        // elements between consecutive columns of p (3-D), t, td; 0: nk
  int guess;
  float *cape, *cin;
  int *mulvl;
  float *z_out;
  int *status;             // nullable
  long long *counters;     // nullable: [0] += sub-steps, [1] += iterations
  const int *perm;         // nullable: thread t computes column perm[t]
  const float *guess_w;    // guess network parameters (device), guess == XC_GUESS_LEARNED
  float *diag = nullptr;   // nullable: [n2][6] diagnostics (cape_column.cuh, getcape_col)
};

// Guess network (guess_mlp.cu).
size_t guess_smem_bytes();
cudaError_t launch_guess_pairs(long long n, unsigned long long seed, float *feats,
                               float *targets, int *iters, cudaStream_t s);
cudaError_t launch_guess_grad(const float *w, const float *feats, const float *targets,
                              long long batch0, long long nb, float *grad, float *loss,
                              cudaStream_t s);
// The same gradient with the three products on tcgen05 (guess_train_tc_kernel);
// *status (device, may be NULL) is set to 1 if a tensor-core wait ran out.
cudaError_t launch_guess_grad_tc(const float *w, const float *feats, const float *targets,
                                 long long batch0, long long nb, float *grad, float *loss,
                                 int *status, cudaStream_t s);
cudaError_t launch_guess_adam(float *w, float *grad, float *m, float *v, float lr, int step,
                              cudaStream_t s);
cudaError_t launch_guess_eval(const float *w, const float *feats, long long n, float *out,
                              cudaStream_t s);

cudaError_t launch_cape(const CapeArgs &a, cudaStream_t s);
// Rebuilds the learned kernel's shared-memory image of the guess network
// from the parameters w (device) on this device (cape_kernel.cu).
cudaError_t build_warp_net(const float *w, cudaStream_t s);
// Device address of that image on this device (for kernels in other files).
cudaError_t warp_net_image(const void **out);
cudaError_t launch_cape_diag(const CapeArgs &a, cudaStream_t s);  // cape_diag.cu

// Column ordering (cape_kernel.cu): a counting sort of the columns by
// (start level, surface dewpoint) so that the 32 columns of a warp need
// similar numbers of levels and iterations.  Scratch: ORDER_BUCKETS counters
// plus a 16-bit bucket and a 32-bit permutation entry per column.
constexpr int ORDER_START_CAP = 63;
constexpr int ORDER_TD_BINS = 256;
constexpr int ORDER_BUCKETS = (ORDER_START_CAP + 1) * ORDER_TD_BINS;
size_t order_workspace_bytes(long long n2);
// Carves `ws` (order_workspace_bytes(n2) bytes, 256-byte aligned) and
// launches the three ordering kernels; on return *perm points into ws.
cudaError_t launch_order(const CapeArgs &a, void *ws, const int **perm, cudaStream_t s);
// The first bucket counter and the permutation of an ordering workspace.
void order_workspace_parts(void *ws, long long n2, unsigned **hist, int **perm);

// FP64 retry of the columns whose status has COL_NOCONV (cape_retry.cu), on
// `s` after the lift; ws (nullable) is the lift's ordering workspace, reused
// for the list of those columns.  a.status must be set.
cudaError_t launch_retry64(const CapeArgs &a, void *ws, cudaStream_t s);

// Records msg as the calling thread's xc_last_error() text (capi.cu).
int set_error(int code, const char *msg);

// Every device or pinned-host allocation the library makes goes through
// these two (capi.cu), which count the successful ones for xc_alloc_count().
cudaError_t dev_malloc(void **p, size_t bytes);
cudaError_t host_malloc(void **p, size_t bytes);

// Raises `func`'s dynamic shared-memory limit to `bytes` on the current
// device, once per device (the attribute is per device; setting it again is
// harmless, so concurrent first calls need no lock).  done: a per-call-site
// array of kMaxAttrDevices flags.
constexpr int kMaxAttrDevices = 64;
inline cudaError_t smem_attr_once(const void *func, int bytes, std::atomic<int> *done) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxAttrDevices && done[dev].load(std::memory_order_acquire))
    return cudaSuccess;
  e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxAttrDevices)
    done[dev].store(1, std::memory_order_release);
  return e;
}
cudaError_t launch_pres_lev_pos(const void *p1d, const void *ps, int dtype, int nk, long long n2,
                                int *start, cudaStream_t s);

struct SrhArgs {
  int grid;   // 1 sigma/model, 2 pressure with shared p1d
  int dtype;
  const void *p, *t, *td, *u, *v, *ps, *ts, *tds, *us, *vs;
  const int *start;  // nullable for grid 2
  double depth, aglh0;
  int nk;
  long long n2;
  double *srh_rm, *srh_lm;
  float *rm, *lm, *mean6;  // nullable, [n2][2]
  int precision;           // 0: reference precisions (FP64 stdheight/SREH), 1: FP32
  int seg_colmap = 0;      // FP32 level-parallel kernel: which columns share a warp (srh_seg.cu)
};

cudaError_t launch_srh(const SrhArgs &a, cudaStream_t s);
// The FP32 level-parallel kernel for float inputs (srh_seg.cu), and its run
// length for nk input levels (0: fewer than 5 levels, which it does not take).
cudaError_t launch_srh_seg(const SrhArgs &a, cudaStream_t s);
int srh_seg_run(int levels);
// CAPE (guess 0 or 1) and SRH of the same columns in one kernel (cape_srh.cu).
cudaError_t launch_cape_srh(const CapeArgs &a, const SrhArgs &s, cudaStream_t st);

// Stage kernels mirroring the reference's individual Fortran loops.
cudaError_t launch_stdheight(const double *P, long long p_stride, const double *T,
                             const double *Td, const double *Ps, const double *Ts,
                             const double *Tds, const double *Hin, const int *start, int NK,
                             long long NX, double *H, double *Hs, cudaStream_t s);
cudaError_t launch_bunkers(const float *U, const float *V, const float *Z, const float *Us,
                           const float *Vs, const float *Zs, const int *start, int nk,
                           long long n2, float *RM, float *LM, float *Mean, cudaStream_t s);
cudaError_t launch_sreh(const double *u, const double *v, const double *aglh, const double *us,
                        const double *vs, const double *aglhs, const double *cu_rm,
                        const double *cv_rm, const double *cu_lm, const double *cv_lm,
                        double top, const int *start, int nk, long long n2, double *sreh_rm,
                        double *sreh_lm, cudaStream_t s);

}  // namespace xc
