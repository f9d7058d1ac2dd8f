/*
 * xcape_gb300.h -- C ABI of libxcape_gb300.so, the GB300 (sm_103a) column
 * kernels behind xcape's calc_cape / calc_srh.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, and
 * returns an int status (XC_OK == 0).  No entry point aborts the process:
 * where the reference Fortran executes `stop` (unknown source / adiabat) the
 * call returns XC_ERR_INVALID instead.
 *
 * Array layout is the one the reference's f2py interfaces bind: a Fortran
 * (nk, n2) array, which is the C array [n2][nk] -- the levels of one column
 * are contiguous, exactly as a user's (..., nlev) numpy array is laid out.
 * Outputs declared (2, n2) in Fortran are [n2][2] here.
 *
 * Two families of entry points:
 *   xc_*          DEVICE pointers; asynchronous on `stream` (a cudaStream_t,
 *                 NULL = the legacy default stream).  Nothing is allocated.
 *   xc_*_host     HOST pointers (pageable or pinned); the library stages the
 *                 arrays through a device workspace that it owns (grown on
 *                 demand, released by xc_release_workspace), runs the same
 *                 kernels and returns when the outputs are back in host memory.
 *
 * Input element type: `dtype` selects XC_F32 or XC_F64 for every
 * floating-point input of a call.  The CAPE kernels round f64 inputs to f32
 * on load, which is what f2py does when it passes a float64 array to a
 * `real` argument.
 */
#ifndef XCAPE_GB300_H
#define XCAPE_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Return codes. */
#define XC_OK 0
#define XC_ERR_INVALID 1  /* bad argument: sizes, option codes, dtype, NULL   */
#define XC_ERR_CUDA 2     /* a CUDA runtime call failed (see xc_last_error)    */
#define XC_ERR_NOMEM 3    /* device workspace could not be allocated           */
#define XC_ERR_NODEVICE 4 /* no CUDA device                                    */

/* Input element types. */
#define XC_F32 0
#define XC_F64 1

/* Option codes, identical to the reference's integer encodings
 * (src/xcape/core.py:302-311). */
#define XC_SOURCE_SURFACE 1
#define XC_SOURCE_MOST_UNSTABLE 2
#define XC_SOURCE_MIXED_LAYER 3
#define XC_ADIABAT_PSEUDO_LIQUID 1
#define XC_ADIABAT_REVERSIBLE_LIQUID 2
#define XC_ADIABAT_PSEUDO_ICE 3
#define XC_ADIABAT_REVERSIBLE_ICE 4

/* Per-column status bits (optional `status` output). */
#define XC_COL_NOCONV 1   /* moist-adiabat iteration passed 100 steps: cape=cin=0 */
#define XC_COL_BADSTART 2 /* start_3d outside 1..nk: outputs zero              */
#define XC_COL_TOOMANYSTEPS 4 /* the ascent would take more than 2^22 sub-steps, or
                                 a pressure step is not finite: cape = cin = 0   */
#define XC_COL_FP64 8     /* recomputed in double precision by the FP64 retry      */

/* Moist-adiabat solver of xc_loopcape_ex (`guess` argument).
 * XC_GUESS_PLAIN is the reference's iteration: first guess thlast = th1,
 * damped step 0.3 * (F(x) - x), stop when |F(x) - x| <= 2e-4 K, give up after
 * 100 steps (CAPE_CODE_model_lev.f90:431-480).  The other modes keep the map
 * F, the stopping test and the result th2 = F(x), and change how x moves:
 * a better first guess, then secant steps on F(x) - x; they evaluate F with
 * one logarithm per sub-step for pi2 and ln(p2/p1) and one approximate (a few
 * ulp) divide in its exponent, and agree with the FP64 run within tolerance. */
#define XC_GUESS_PLAIN 0
#define XC_GUESS_LEARNED 1      /* extrapolated, with the guess network's guess on the
                                   first sub-step that starts saturated */
#define XC_GUESS_EXTRAPOLATED 2 /* first guess extrapolates the previous step  */
#define XC_GUESS_SECANT 3       /* first guess th1 (the reference's), secant steps */
#define XC_GUESS_LEARNED_EVERY 4 /* the network's guess on every sub-step that starts
                                    saturated, th1 on the others; secant steps */
#define XC_GUESS_LEARNED_WARP 5 /* the network's guess on every sub-step that starts
                                   saturated, the extrapolated one on the others;
                                   Newton then secant steps; each warp evaluates the
                                   network for its 32 columns in lockstep at every
                                   sub-step on the tensor cores */

/* Flag OR'ed into `guess` (xc_loopcape_ex, xc_loopcape_ex_host,
 * xc_loopcape_multi_host, xc_loopcape_ex_noalloc): after the FP32 lift, the
 * columns it flagged XC_COL_NOCONV -- the reference's give-up after 100
 * iterations, CAPE = CIN = 0 (CAPE_CODE_model_lev.f90:464-474), which FP32
 * rounding can cause where the iteration converges in FP64 -- are lifted
 * again in double precision with the reference's iteration, in a second
 * kernel, and their outputs replaced.  Their status gains XC_COL_FP64 and
 * keeps XC_COL_NOCONV only if the FP64 iteration gave up too.  The device
 * entry points need the status array for it. */
#define XC_RETRY_FP64 256

/* Parameters of the guess network (3 -> 64 -> 64 -> 1, ReLU), flat:
 * W1[64][3] b1[64] W2[64][64] b2[64] w3[64] b3. */
#define XC_GUESS_NPARAM 4481

/* Largest supported level count of one column (without the surface). */
#define XC_MAX_LEVELS 4096

/* ---------------------------------------------------------------------- */
/* CAPE / CIN                                                             */
/* ---------------------------------------------------------------------- */

/* Replaces loopcape_ml: CAPE_CODE_model_lev.pyf:6-24,
 * CAPE_CODE_model_lev.f90:4-91 (+ getcape_ml :97-564).
 * p3d/t3d/td3d [n2][nk] (hPa, degC, degC), ps/ts/tds [n2].
 * Outputs [n2]: cape, cin (J/kg), mulvl (1-based level of the most-unstable
 * parcel, surface = 1; -999999 unless source == 2), z_out (height of the last
 * level reached, m).  status may be NULL. */
int xc_loopcape_ml(const void *p3d, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, int nk, int n2, float *cape, float *cin,
                   int *mulvl, float *z_out, int *status, void *stream);

/* Replaces loopcape_pl1d: CAPE_CODE_pressure_lev.pyf:26-45 (the routine named
 * loopcape_pl1d there), CAPE_CODE_pressure_lev.f90:88-169.  p1d [nk] is shared
 * by all columns.  start_3d [n2] is the 1-based first level at or above the
 * surface; when start_3d is NULL it is derived in the kernel with the
 * reference's rule (src/xcape/core.py:286-289: masked argmin of ps - p). */
int xc_loopcape_pl1d(const void *t3d, const void *td3d, const void *p1d, const void *ps,
                     const void *ts, const void *tds, int dtype, float pinc, int source,
                     float ml_depth, int adiabat, const int *start_3d, int nk, int n2,
                     float *cape, float *cin, int *mulvl, float *z_out, int *status,
                     void *stream);

/* Replaces loopcape_pl: CAPE_CODE_pressure_lev.pyf:6-25,
 * CAPE_CODE_pressure_lev.f90:4-84 (per-column pressure, per-column start;
 * start_3d must not be NULL). */
int xc_loopcape_pl(const void *p3d, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, const int *start_3d, int nk, int n2,
                   float *cape, float *cin, int *mulvl, float *z_out, int *status,
                   void *stream);

/* Generalised CAPE entry point used by the Python layer: one call for the
 * three grid kinds.  grid: 1 = sigma/model (p3d per column), 2 = pressure
 * with shared p1d (start_3d optional), 3 = pressure with per-column p3d
 * (start_3d required).  guess: XC_GUESS_*.  counters (nullable, 2 x int64 on
 * the device) receives the total sub-steps and iterations, atomically added.
 * workspace (nullable, device memory of at least
 * xc_loopcape_workspace_bytes(n2) bytes, 256-byte aligned) lets the call
 * reorder the columns by level count and surface dewpoint before the lift,
 * so that each warp's columns need similar work; the results do not depend
 * on it.  The call keeps using the workspace until the stream reaches the
 * end of the launch. */
int xc_loopcape_ex(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                   const void *ts, const void *tds, int dtype, float pinc, int source,
                   float ml_depth, int adiabat, const int *start_3d, int nk, int n2, int guess,
                   float *cape, float *cin, int *mulvl, float *z_out, int *status,
                   long long *counters, void *workspace, size_t workspace_bytes, void *stream);

/* xc_loopcape_ex for nsrc (1..3) sources of the same device-resident
 * columns in one call: with a workspace the columns are ordered once, and
 * every source's lift reads that order.  No counterpart in the reference,
 * where each source is its own calc_cape call (src/xcape/core.py:130-235).
 * sources [nsrc] holds XC_SOURCE_* codes; the outputs are [nsrc][n2]
 * (source j's result of column i at j * n2 + i; status may be NULL) and
 * equal those of nsrc xc_loopcape_ex calls.  counters, when given, sums the
 * work of all the sources.  With XC_RETRY_FP64 the retries of every source
 * follow all the lifts. */
int xc_loopcape_multi(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                      const void *ts, const void *tds, int dtype, float pinc, int nsrc,
                      const int *sources, float ml_depth, int adiabat, const int *start_3d, int nk,
                      int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out,
                      int *status, long long *counters, void *workspace, size_t workspace_bytes,
                      void *stream);

/* xc_loopcape_ex (natural column order, no counters) with the diagnostics
 * that getcape computes and discards -- the crossing pressure of its
 * buoyancy sign changes (CAPE_CODE_model_lev.f90:511, :526) and the parcel
 * theta-e (:505).  No counterpart entry point in the reference.
 * diag [n2][6] (device, float):
 *   0 LFC pressure (hPa), 1 LFC height (m): the lowest point of the first
 *     layer with positive area -- the negative-to-positive crossing, or the
 *     layer's base when the parcel is already buoyant there;
 *   2 EL pressure (hPa), 3 EL height (m): the highest positive-to-negative
 *     crossing, or the last level reached when the parcel is still buoyant;
 *   4 height (m) and 5 theta-e (K, getthe) of the source parcel.
 * Each is -999999 where undefined: no positive area (0-3), no ascent, or a
 * column whose iteration gave up.  guess: XC_GUESS_PLAIN or
 * XC_GUESS_LEARNED. */
int xc_loopcape_diag(int grid, const void *p, const void *t3d, const void *td3d, const void *ps,
                     const void *ts, const void *tds, int dtype, float pinc, int source,
                     float ml_depth, int adiabat, const int *start_3d, int nk, int n2, int guess,
                     float *cape, float *cin, int *mulvl, float *z_out, int *status, float *diag,
                     void *stream);

/* Device workspace that lets xc_loopcape_ex order n2 columns. */
size_t xc_loopcape_workspace_bytes(int n2);

/* Largest n2 that xc_loopcape_ex_noalloc accepts. */
#define XC_NOALLOC_MAX_COLUMNS 1048576

/* xc_loopcape_ex for callers that cannot allocate device memory -- a host
 * framework that owns every byte of the device's memory, a serving process
 * under a fixed memory budget, a real-time loop that forbids allocation after
 * start-up.  No counterpart in the reference (its Fortran runs on the host).
 * Same arguments and results as xc_loopcape_ex (device pointers, columns
 * ordered before the lift), but the ordering scratch lives in a static
 * device array inside the library (about 6.1 MiB), so the call allocates
 * nothing.  n2 above XC_NOALLOC_MAX_COLUMNS is rejected with XC_ERR_INVALID.
 * CUDA creates the array on a device when it loads the library's module
 * that holds it: under lazy module loading (the default) at the first call
 * on that device, and the device then keeps it until its context is
 * destroyed.  A call with n2 == 0 does only that set-up, so make one at
 * start-up on each device, before any stream capture.  Every call looks the
 * array's address up again, so it stays valid after cudaDeviceReset.  All
 * calls share the array: calls that overlap on the GPU race and must be
 * issued one after the other. */
int xc_loopcape_ex_noalloc(int grid, const void *p, const void *t3d, const void *td3d,
                           const void *ps, const void *ts, const void *tds, int dtype,
                           float pinc, int source, float ml_depth, int adiabat,
                           const int *start_3d, int nk, int n2, int guess, float *cape,
                           float *cin, int *mulvl, float *z_out, int *status,
                           long long *counters, void *stream);

/* Host-pointer form of xc_loopcape_ex (see the family note above).  The
 * columns go through in up to 8 chunks whose device buffers take at most
 * 4 GiB (at least two chunks' worth; the environment variable
 * XC_HOST_RING_BYTES sets another limit, in bytes); chunks beyond that
 * reuse buffers, which changes no result.  The outputs reach the caller's
 * arrays through pinned staging, moved by a pool of host threads that the
 * library starts on first use and keeps (XC_HOST_COPY_THREADS, 0..16,
 * default 4; 0 moves them in the calling thread).  XC_HOST_CHUNKS (2..16,
 * default 8) and XC_HOST_STREAMS (1..4, default 2) set the chunk count and
 * the compute streams; none of these changes a result. */
int xc_loopcape_ex_host(int grid, const void *p, const void *t3d, const void *td3d,
                        const void *ps, const void *ts, const void *tds, int dtype, float pinc,
                        int source, float ml_depth, int adiabat, const int *start_3d, int nk,
                        int n2, int guess, float *cape, float *cin, int *mulvl, float *z_out,
                        int *status, void *stream);

/* xc_loopcape_ex_host for nsrc (1..3) sources of the same columns: the
 * inputs cross to the device once and every source is lifted from them.
 * No counterpart in the reference, where each source is its own calc_cape
 * call (src/xcape/core.py:130-235), each handing the same p, t, td to the
 * Fortran again.  sources [nsrc] holds XC_SOURCE_* codes; the outputs are
 * [nsrc][n2] (source j's results of column i at j * n2 + i) and equal those
 * of nsrc xc_loopcape_ex_host calls. */
int xc_loopcape_multi_host(int grid, const void *p, const void *t3d, const void *td3d,
                           const void *ps, const void *ts, const void *tds, int dtype, float pinc,
                           int nsrc, const int *sources, float ml_depth, int adiabat,
                           const int *start_3d, int nk, int n2, int guess, float *cape,
                           float *cin, int *mulvl, float *z_out, int *status, void *stream);

/* ---------------------------------------------------------------------- */
/* Storm-relative helicity                                                 */
/* ---------------------------------------------------------------------- */

/* Fused replacement of src/xcape/core.py:_calc_srh_numpy :473-542, i.e. the
 * chain loop_stdheight_{ml,pl1d} -> bunkers_loop_{ml,pl} -> loop_sreh_{ml,pl}
 * in one pass per column.  grid: 1 = sigma/model (p [n2][nk]), 2 = pressure
 * with shared p [nk] (start_3d optional as for xc_loopcape_pl1d).
 * depth (m) is `top` of loop_sreh; aglh0 is the surface height (2 m in the
 * reference, core.py:519).  srh_rm/srh_lm [n2] (f64, like loop_sreh);
 * rm/lm/mean6 [n2][2] (f32, like bunkers_loop) may be NULL. */
int xc_calc_srh(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                const void *v3d, const void *ps, const void *ts, const void *tds,
                const void *us, const void *vs, int dtype, const int *start_3d, double depth,
                double aglh0, int nk, int n2, double *srh_rm, double *srh_lm, float *rm,
                float *lm, float *mean6, void *stream);

/* Precision of the stdheight and SREH stages (xc_calc_srh_ex). */
#define XC_SRH_REFERENCE 0 /* as the reference: FP64 stdheight and SREH, FP32 Bunkers */
#define XC_SRH_FP32 1      /* FP32 throughout, Kahan-compensated height and helicity sums */

/* xc_calc_srh with a choice of precision for the height and helicity stages
 * (xc_calc_srh uses XC_SRH_REFERENCE).  XC_SRH_FP32 trades the FP64 stages
 * for FP32 ones with compensated sums; its difference from the reference is
 * stated in the test suite (tests/test_gpu_srh.py) and is far inside
 * 0.5 m^2/s^2. */
int xc_calc_srh_ex(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                   const void *v3d, const void *ps, const void *ts, const void *tds,
                   const void *us, const void *vs, int dtype, const int *start_3d, double depth,
                   double aglh0, int nk, int n2, int precision, double *srh_rm, double *srh_lm,
                   float *rm, float *lm, float *mean6, void *stream);

/* Host-pointer form of xc_calc_srh_ex. */
int xc_calc_srh_host(int grid, const void *p, const void *t3d, const void *td3d,
                     const void *u3d, const void *v3d, const void *ps, const void *ts,
                     const void *tds, const void *us, const void *vs, int dtype,
                     const int *start_3d, double depth, double aglh0, int nk, int n2,
                     int precision, double *srh_rm, double *srh_lm, float *rm, float *lm,
                     float *mean6, void *stream);

/* ---------------------------------------------------------------------- */
/* CAPE and SRH of the same columns in one pass                            */
/* ---------------------------------------------------------------------- */

/* xc_loopcape_ex and xc_calc_srh_ex on the same columns in one kernel: the
 * FP32 lift (CAPE/CIN) and the SRH chain, whose FP64 stages then run on the
 * FP64 pipe while other warps lift.  No counterpart in the reference, which
 * computes the two with separate f2py chains over the same inputs
 * (src/xcape/core.py:261-332 and :473-542); the results are those of the
 * two separate calls.  Device pointers.
 * grid: 1 (sigma, p [n2][nk]) or 2 (pressure, shared p [nk], start_3d
 * optional).  CAPE options and outputs as xc_loopcape_ex, with guess
 * XC_GUESS_PLAIN or XC_GUESS_LEARNED; depth, aglh0, precision and the SRH
 * outputs as xc_calc_srh_ex.  workspace (nullable, as xc_loopcape_ex)
 * orders the columns for the lift.  With precision XC_SRH_FP32 and f32
 * inputs the call runs the lift and calc_srh's level-parallel FP32 kernel
 * back to back instead, which is faster there (that kernel reads each
 * column's rows coalesced with eight lanes per column). */
int xc_cape_srh(int grid, const void *p, const void *t3d, const void *td3d, const void *u3d,
                const void *v3d, const void *ps, const void *ts, const void *tds, const void *us,
                const void *vs, int dtype, float pinc, int source, float ml_depth, int adiabat,
                const int *start_3d, double depth, double aglh0, int nk, int n2, int guess,
                int precision, float *cape, float *cin, int *mulvl, float *z_out, int *status,
                double *srh_rm, double *srh_lm, float *rm, float *lm, float *mean6,
                void *workspace, size_t workspace_bytes, void *stream);

/* Replaces loop_stdheight_ml: stdheight_2D_model_lev.pyf:6-19,
 * stdheight_2D_model_lev.f90:4-34 (+ stdheight_ml :74-160).  All f64. */
int xc_loop_stdheight_ml(const double *P, const double *T, const double *Td, const double *Ps,
                         const double *Ts, const double *Tds, const double *Hin, int NK, int NX,
                         double *H, double *Hs, void *stream);

/* Replaces loop_stdheight_pl1d: stdheight_2D_pressure_lev.pyf:20-33,
 * stdheight_2D_pressure_lev.f90:65-93.  Levels below start get -999999. */
int xc_loop_stdheight_pl1d(const double *T, const double *Td, const double *P, const double *Ps,
                           const double *Ts, const double *Tds, const double *Hin,
                           const int *start_3d, int NK, int NX, double *H, double *Hs,
                           void *stream);

/* Replaces loop_stdheight_pl: stdheight_2D_pressure_lev.pyf:6-19,
 * stdheight_2D_pressure_lev.f90:5-47. */
int xc_loop_stdheight_pl(const double *P, const double *T, const double *Td, const double *Ps,
                         const double *Ts, const double *Tds, const double *Hin,
                         const int *start_3d, int NK, int NX, double *H, double *Hs,
                         void *stream);

/* Replaces bunkers_loop_ml: Bunkers_model_lev.pyf:8-21,
 * Bunkers_model_lev.f90:4-69 (+ bunkers_calc_ml :75-180, DINTERP2DZ :188-236).
 * All f32; RM/LM/Mean6kmwind [n2][2]. */
int xc_bunkers_loop_ml(const float *U3d, const float *V3d, const float *AGLH3d, const float *Us,
                       const float *Vs, const float *AGLHs, int nk, int n2, float *RM, float *LM,
                       float *Mean6kmwind, void *stream);

/* Replaces bunkers_loop_pl: Bunkers_pressure_lev.pyf:7-21,
 * Bunkers_pressure_lev.f90:4-78. */
int xc_bunkers_loop_pl(const float *U3d, const float *V3d, const float *AGLH3d, const float *Us,
                       const float *Vs, const float *AGLHs, const int *start_3d, int nk, int n2,
                       float *RM, float *LM, float *Mean6kmwind, void *stream);

/* Replaces loop_sreh_ml: SREH_model_lev.pyf:6-23, SREH_model_lev.f90:4-55
 * (+ DCALRELHL_ml :61-118, INTERP1 :123-129).  All f64. */
int xc_loop_sreh_ml(const double *u, const double *v, const double *aglh, const double *us,
                    const double *vs, const double *aglhs, const double *cu_rm,
                    const double *cv_rm, const double *cu_lm, const double *cv_lm, double top,
                    int nk, int n2, double *sreh_rm, double *sreh_lm, void *stream);

/* Replaces loop_sreh_pl: SREH_pressure_lev.pyf:6-24, SREH_pressure_lev.f90:4-63. */
int xc_loop_sreh_pl(const double *u, const double *v, const double *aglh, const double *us,
                    const double *vs, const double *aglhs, const double *cu_rm,
                    const double *cv_rm, const double *cu_lm, const double *cv_lm, double top,
                    const int *start_3d, int nk, int n2, double *sreh_rm, double *sreh_lm,
                    void *stream);

/* Derives start_3d [n2] for a shared 1-D pressure axis with the reference's
 * rule (core.py:286-289).  No counterpart entry point in the reference: there
 * it is host numpy code. */
int xc_pres_lev_pos(const void *p1d, const void *ps, int dtype, int nk, int n2, int *start_3d,
                    void *stream);

/* ---------------------------------------------------------------------- */
/* Learned first guess (no counterpart in the reference)                  */
/* ---------------------------------------------------------------------- */
/* The network maps a saturated parcel's (target pressure, theta-e, total
 * water) to its temperature at the end of a sub-step.  All pointers below are
 * device memory except where stated; calls are asynchronous on `stream`. */

/* Loads the network that XC_GUESS_LEARNED uses on the current device
 * (weights: XC_GUESS_NPARAM floats, host memory if on_device == 0).
 * Synchronises `stream`. */
int xc_guess_set_weights(const float *weights, int on_device, void *stream);

/* n training pairs drawn with `seed`: saturated parcels, p 100..1050 hPa,
 * T -80..40 degC, pressure steps 1..25 hPa, each solved with the plain
 * (reference) iteration.  feats [n][3], targets [n] (normalised end
 * temperature), iters [n] (iterations used, negative if it gave up). */
int xc_guess_pairs(long long n, unsigned long long seed, float *feats, float *targets, int *iters,
                   void *stream);

/* Adds the gradient of the mean squared error over the n pairs to grad
 * [XC_GUESS_NPARAM] and the loss to *loss (both must be zeroed first).  The
 * three 64-wide products run on the tensor cores with mma.sync (BF16
 * operands, FP32 accumulation). */
int xc_guess_grad(const float *weights, const float *feats, const float *targets, long long n,
                  float *grad, float *loss, void *stream);

/* xc_guess_grad with the three products on the 5th-generation tensor cores
 * (tcgen05.mma, BF16 operands in shared memory, FP32 accumulators in tensor
 * memory; dW2 stays in tensor memory over a block's tiles).  status: a
 * device int (may be NULL) set to 1 if a wait for the tensor cores ran out,
 * in which case grad and loss are incomplete; the caller zeroes it. */
int xc_guess_grad_tc(const float *weights, const float *feats, const float *targets,
                     long long n, float *grad, float *loss, int *status, void *stream);

/* One Adam step (step >= 1) on the FP32 weights; zeroes grad. */
int xc_guess_adam(float *weights, float *grad, float *m, float *v, float lr, int step,
                  void *stream);

/* Batched inference: out [n] = network(feats [n][3]). */
int xc_guess_eval(const float *weights, const float *feats, long long n, float *out,
                  void *stream);

/* ---------------------------------------------------------------------- */
/* Library services                                                       */
/* ---------------------------------------------------------------------- */

/* Frees the device workspace of the *_host entry points (all devices). */
int xc_release_workspace(void);

/* Text of the last error raised on the calling thread ("" if none). */
const char *xc_last_error(void);

/* Library version string. */
const char *xc_version(void);

/* Device and pinned-host allocations (cudaMalloc, cudaMallocHost) the library
 * has made since it was loaded; it does not count CUDA's own allocations
 * (module loads, graphs, streams).  For checking that a path allocates
 * nothing, e.g. xc_loopcape_ex_noalloc. */
long long xc_alloc_count(void);

/* Measures the current device's FP32 and XU (transcendental unit) issue
 * rates with two short kernels of known instruction mix -- 8 independent
 * fused multiply-add chains per thread, and 8 independent ex2.approx chains
 * per thread -- timed with CUDA events on `stream` after a warm-up launch.
 * Outputs are lane operations per second, in units of 1e9 (one FFMA or one
 * ex2.approx of one thread is one operation).  They are the denominators of
 * the CAPE lift's compute roofline.  No counterpart in the reference.
 * Synchronises `stream`; takes a few milliseconds. */
int xc_measure_pipe_peaks(double *fp32_gops, double *xu_gops, void *stream);

/* ------------------------------------------------------------------------ */
/* Ragged batches in one persistent, graph-captured kernel.  No counterpart  */
/* in the reference, whose unit of work is one f2py call on one array         */
/* (loopcape_ml, CAPE_CODE_model_lev.f90:4-91; loopcape_pl1d,                 */
/* CAPE_CODE_pressure_lev.f90:88-169): a batch runs many such calls, each     */
/* with its own sizes and options, in one launch.                             */
/* ------------------------------------------------------------------------ */

/* One calc_cape request: float32 DEVICE arrays.
 *   grid 1 (sigma / model levels): p, t3d, td3d are [n2][ld];
 *   grid 2 (pressure levels): p is [nk], shared by the request's columns,
 *          t3d and td3d are [n2][ld]; each column's start level is derived
 *          from its ps (below-ground levels masked, core.py:286-289).
 * The first nk of every ld values are a column's levels (ld >= nk; ld = nk
 * for a dense array).  ps, ts, tds, cape, cin, mulvl, z_out, status: [n2].
 * pinc, source, ml_depth, adiabat: as xc_loopcape_ml. */
typedef struct xc_cape_request {
  int grid;
  int nk;
  long long n2;
  long long ld;
  const float *p, *t3d, *td3d, *ps, *ts, *tds;
  float pinc;
  int source;
  float ml_depth;
  int adiabat;
  float *cape, *cin;
  int *mulvl;
  float *z_out;
  int *status; /* nullable */
} xc_cape_request;

#define XC_BATCH_MAX_REQUESTS 65536

typedef struct xc_batch xc_batch; /* opaque batch executor */

/* Creates an executor on the current device for batches of up to
 * max_requests requests and max_columns columns, each request's column
 * count rounded up to a multiple of 32.  guess: XC_GUESS_PLAIN,
 * XC_GUESS_LEARNED (needs xc_guess_set_weights first) or
 * XC_GUESS_EXTRAPOLATED.  It allocates two request tables on the device,
 * two pinned staging tables, and instantiates two CUDA graphs.  Each graph
 * uploads a table, clears the work counters and launches the persistent
 * kernel (one wave of blocks that take 32-column chunks from an atomic
 * counter). */
int xc_batch_create(int max_requests, long long max_columns, int guess, xc_batch **out);
/* Runs one batch: reqs is a HOST array of nreq descriptors.  Every request
 * is validated first; an invalid request or a batch over the executor's
 * capacity returns XC_ERR_INVALID with nothing launched.  Otherwise the
 * descriptors are written to a staging table and its graph is launched on
 * `stream`.  The outputs are complete when `stream` reaches this point.
 * Runs alternate between the two tables; a run first waits for the run
 * before the previous one. */
int xc_batch_run(xc_batch *b, const xc_cape_request *reqs, int nreq, void *stream);
/* Sub-steps and fixed-point iterations of the last run (waits for it). */
int xc_batch_work(xc_batch *b, long long *substeps, long long *iterations);
/* Waits for the executor's runs and frees it (NULL is a no-op). */
int xc_batch_destroy(xc_batch *b);

/* Queues n copies on `stream` in order, dst[k] <- src[k] of bytes[k] bytes,
 * one cudaMemcpyAsync each with the direction taken from the pointers
 * (unified addressing): the inputs of a service loop's batch into its
 * device arena, or its results back, in one call from the host language
 * instead of one call per array.  Copies from or to pinned host memory are
 * asynchronous; the caller keeps the buffers alive and unchanged until the
 * stream has passed them.  Zero-byte entries are skipped. */
int xc_copy_list(int n, void *const *dst, const void *const *src,
                 const unsigned long long *bytes, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* XCAPE_GB300_H */
