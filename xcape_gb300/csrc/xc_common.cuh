// xc_common.cuh -- shared device helpers for the xcape GB300 column kernels.
//
// Thermodynamic constants and helper functions follow the reference Fortran
// (src/xcape/fortran/CAPE_CODE_model_lev.f90:188-211 for the constants,
// :570-620 for getqvs/getqvi/getthe).  Single-precision constants are
// evaluated in float at compile time exactly as gfortran folds `real,
// parameter` expressions.
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define XC_HD __host__ __device__ __forceinline__
#else
#define XC_HD inline
#endif

namespace xc {

// ---- CAPE constants (CAPE_CODE_model_lev.f90:188-211) ---------------------
constexpr float G = 9.81f;
constexpr float P00 = 100000.0f;
constexpr float CP = 1005.7f;
constexpr float RD = 287.04f;
constexpr float RV = 461.5f;
constexpr float XLV = 2501000.0f;
constexpr float XLS = 2836017.0f;
constexpr float T0 = 273.15f;
constexpr float CPV = 1875.0f;
constexpr float CPL = 4190.0f;
constexpr float CPI = 2118.636f;
constexpr float LV1 = XLV + (CPL - CPV) * T0;
constexpr float LV2 = CPL - CPV;
constexpr float LS1 = XLS + (CPI - CPV) * T0;
constexpr float LS2 = CPI - CPV;
constexpr float RP00 = 1.0f / P00;
constexpr float REPS = RV / RD;
constexpr float RDDCP = RD / CP;
constexpr float CPDG = CP / G;
constexpr float CONVERGE = 0.0002f;
constexpr float LN_P00 = 11.5129254649702f;  // ln(P00), for the accelerated solvers
constexpr float QEPS = 287.04f / 461.5f;  // eps inside getqvs/getqvi

// Column status bits (mirrors include/xcape_gb300.h).
constexpr int COL_NOCONV = 1;
constexpr int COL_BADSTART = 2;
constexpr int COL_TOOMANYSTEPS = 4;

// Sub-step budget of one column: bounds the work of any input (a column
// that would need more is flagged and zeroed instead of running on).
constexpr long long MAX_SUBSTEPS = 1LL << 22;

// ---- getqvs / getqvi / getthe ----------------------------------------------
// CAPE_CODE_model_lev.f90:570-581
XC_HD float getqvs(float p, float t) {
  float es = 611.2f * expf(17.67f * (t - 273.15f) / (t - 29.65f));
  return QEPS * es / (p - es);
}
// CAPE_CODE_model_lev.f90:587-598
XC_HD float getqvi(float p, float t) {
  float es = 611.2f * expf(21.8745584f * (t - 273.15f) / (t - 7.66f));
  return QEPS * es / (p - es);
}
// CAPE_CODE_model_lev.f90:604-620 (x**(-1) is 1/x)
XC_HD float getthe(float p, float t, float td, float q) {
  float tlcl;
  if ((td - t) >= -0.1f) {
    tlcl = t;
  } else {
    tlcl = 56.0f + 1.0f / (1.0f / (td - 56.0f) + 0.00125f * logf(t / td));
  }
  return t * powf(100000.0f / p, 0.2854f * (1.0f - 0.28f * q)) *
         expf(((3376.0f / tlcl) - 2.54f) * q * (1.0f + 0.81f * q));
}

// Approximate divide (a few ulp) for the accelerated solvers: their secant
// quotients, the saturation mixing ratio and the exponent of their map, whose
// contract is agreement with the FP64 run within tolerance rather than
// bit-faithfulness to the FP32 Fortran.  On the device a times the PTX
// reciprocal approximation; this and the approximate functions below use the
// flush-to-zero forms, which skip the handling of subnormal operands and
// results: the quantities they see (pressures, temperatures, mixing ratios
// and their ratios) are far from the subnormal range, where a result would
// only be flushed to zero.  Exact on the host.
XC_HD float fast_div(float a, float b) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(b));
  return a * r;
#else
  return a / b;
#endif
}
// Approximate exp for the same solvers: ex2.approx of x log2(e), a relative
// error of a few ulp plus the rounding of x log2(e).  expf on the host.
XC_HD float fast_exp(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x * 1.4426950408889634f));
  return y;
#else
  return expf(x);
#endif
}

// Approximate natural log: lg2.approx of x times ln 2 (a few ulp for x
// outside [0.5, 2], a small absolute error inside).  logf on the host.
XC_HD float fast_log(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y * 0.6931471805599453f;
#else
  return logf(x);
#endif
}

// Base-2 forms of the approximate exp and log, for expressions whose factors
// log2(e) and ln 2 fold into constants (ex2.approx / lg2.approx,
// flush-to-zero); exp2f / log2f on the host.
XC_HD float fast_exp2(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#else
  return exp2f(x);
#endif
}
XC_HD float fast_log2(float x) {
#if defined(__CUDA_ARCH__)
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
#else
  return log2f(x);
#endif
}
// The reciprocal that fast_div multiplies by; 1 / x on the host.
XC_HD float fast_rcp(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}

constexpr float LOG2E = 1.4426950408889634f;
constexpr float LN2 = 0.6931471805599453f;
constexpr float LG2_P00 = 16.609640474436812f;  // log2(P00)
constexpr float LG2_ES0 = 9.255500733148386f;   // log2(611.2)

// getthe of the accelerated solvers' source selection: the same formula with
// the approximate log, exp and divides (powf as exp of the log), a relative
// error near 1e-6 of theta-e.  The host build computes exactly what getthe
// does except for powf, evaluated as exp(b log a).
XC_HD float getthe_fast(float p, float t, float td, float q) {
  float tlcl;
  if ((td - t) >= -0.1f) {
    tlcl = t;
  } else {
    tlcl = 56.0f + fast_div(1.0f, fast_div(1.0f, td - 56.0f) + 0.00125f * fast_log(fast_div(t, td)));
  }
#if defined(__CUDA_ARCH__)
  // the two factors (P00/p)^a exp(b) as one power of two, 2^(a log2(P00/p) + b log2(e))
  return t * fast_exp2(fmaf(0.2854f * (1.0f - 0.28f * q), fast_log2(fast_div(100000.0f, p)),
                            (fast_div(3376.0f, tlcl) - 2.54f) * q * (1.0f + 0.81f * q) * LOG2E));
#else
  return t * fast_exp(0.2854f * (1.0f - 0.28f * q) * fast_log(fast_div(100000.0f, p))) *
         fast_exp((fast_div(3376.0f, tlcl) - 2.54f) * q * (1.0f + 0.81f * q));
#endif
}

// What the accelerated saturation mixing ratio computes on its way, kept for
// the slope of the moist-adiabat map: es, 1 / (T - b) and 1 / (p - es).
struct QsatParts {
  float es, rtb, rpe;
};

// getqvs (ICE false: a = 17.67, b = 29.65) / getqvi (ICE true: a =
// 21.8745584, b = 7.66) of the accelerated solvers: es = 611.2 exp(a (T -
// 273.15) / (T - b)), qsat = QEPS es / (p - es), with the approximate
// reciprocals and exp.  On the device the exponent is taken to base 2, with
// a log2(e) folded into one constant and log2(611.2) added by the same
// multiply-add.  The host build computes exactly what getqvs / getqvi do
// (and the two reciprocals beside them).
template <bool ICE>
XC_HD float qsat_fast(float p, float t, QsatParts &q) {
  constexpr float A = ICE ? 21.8745584f : 17.67f;
  constexpr float B = ICE ? 7.66f : 29.65f;
#if defined(__CUDA_ARCH__)
  q.rtb = fast_rcp(t - B);
  q.es = fast_exp2(fmaf((t - 273.15f) * (A * LOG2E), q.rtb, LG2_ES0));
  q.rpe = fast_rcp(p - q.es);
  return QEPS * q.es * q.rpe;
#else
  q.es = 611.2f * expf(A * (t - 273.15f) / (t - B));
  q.rtb = 1.0f / (t - B);
  q.rpe = 1.0f / (p - q.es);
  return QEPS * q.es / (p - q.es);
#endif
}
XC_HD float getqvs_fast(float p, float t) {
  QsatParts q;
  return qsat_fast<false>(p, t, q);
}

// Fortran MIN/MAX as gfortran lowers them for the reference build: the
// second operand is returned when the comparison fails (NaN included).
template <typename R>
XC_HD R fmin_f(R a, R b) { return a < b ? a : b; }
template <typename R>
XC_HD R fmax_f(R a, R b) { return a > b ? a : b; }

// ---- double precision (the FP64 retry of the CAPE lift) -------------------
// getqvs / getqvi / getthe in double precision with double literals: the
// same formulas (CAPE_CODE_model_lev.f90:570-620) evaluated as the FP64
// oracle evaluates them.
XC_HD double getqvs(double p, double t) {
  const double es = 611.2 * exp(17.67 * (t - 273.15) / (t - 29.65));
  return (287.04 / 461.5) * es / (p - es);
}
XC_HD double getqvi(double p, double t) {
  const double es = 611.2 * exp(21.8745584 * (t - 273.15) / (t - 7.66));
  return (287.04 / 461.5) * es / (p - es);
}
XC_HD double getthe(double p, double t, double td, double q) {
  double tlcl;
  if ((td - t) >= -0.1) {
    tlcl = t;
  } else {
    tlcl = 56.0 + 1.0 / (1.0 / (td - 56.0) + 0.00125 * log(t / td));
  }
  return t * pow(100000.0 / p, 0.2854 * (1.0 - 0.28 * q)) *
         exp(((3376.0 / tlcl) - 2.54) * q * (1.0 + 0.81 * q));
}

// exp, log and pow of the column routines in their precision: CUDA's (or
// libm's) single-precision functions for float, double ones for double.
XC_HD float xexp(float x) { return expf(x); }
XC_HD double xexp(double x) { return exp(x); }
XC_HD float xlog(float x) { return logf(x); }
XC_HD double xlog(double x) { return log(x); }
XC_HD float xpow(float a, float b) { return powf(a, b); }
XC_HD double xpow(double a, double b) { return pow(a, b); }

// ---- input loads ------------------------------------------------------------
template <typename T>
XC_HD T ld(const T *ptr) {
#if defined(__CUDA_ARCH__)
  return __ldg(ptr);
#else
  return *ptr;
#endif
}
template <typename T>
XC_HD float ldf(const T *ptr) {
  return (float)ld(ptr);
}
template <typename T>
XC_HD double ldd(const T *ptr) {
  return (double)ld(ptr);
}

// Masked argmin of ps - p over the levels, 1-based (src/xcape/core.py:286-289):
// entries with ps - p < 0 are masked (filled with +inf), np.argmin then
// returns the first NaN if there is one, else the first minimum; a column
// with every entry masked gives index 0.  The difference is taken in the
// input precision T, as numpy does for same-dtype operands.
template <typename T>
XC_HD int pres_lev_pos_col(const T *p1d, T ps, int nk) {
  T best = ps - ld(p1d);
  int bi = 0;
  if (!(best < (T)0)) {
    if (best != best) return 1;
  } else {
    best = (T)INFINITY;
  }
  for (int k = 1; k < nk; ++k) {
    T d = ps - ld(p1d + k);
    if (d != d) return k + 1;
    if (d < (T)0) d = (T)INFINITY;
    if (d < best) {
      best = d;
      bi = k;
    }
  }
  return bi + 1;
}

}  // namespace xc
