// emul.cu -- host build of the kernels' column routines (test harness).
//
// Compiles cape_column.cuh / srh_column.cuh as ordinary host code (glibc
// expf/logf/powf, -ffp-contract=off) and loops over the columns on the CPU,
// so that the exact code the CUDA kernels run can be compared with the
// oracle without a GPU: the only differences allowed are the ones the column
// routines document (none changes a result for finite inputs).
#include "../../xcape_gb300/csrc/cape_column.cuh"
#include "../../xcape_gb300/csrc/srh_column.cuh"

using namespace xc;

template <typename T, int GRID, int SOLVER, bool DIAG>
static void cape_loop_d(const CapeArgs &a, long long *counters) {
  const bool ice = a.adiabat >= 3, pseudo = (a.adiabat == 1 || a.adiabat == 3);
  long long s = 0, it = 0;
  for (long long i = 0; i < a.n2; ++i) {
    int nsub = 0, niter = 0;
    const float *w = a.guess_w;
    if (ice && pseudo) cape_column_run<T, GRID, true, true, SOLVER, DIAG>(a, i, nsub, niter, w);
    else if (ice) cape_column_run<T, GRID, true, false, SOLVER, DIAG>(a, i, nsub, niter, w);
    else if (pseudo) cape_column_run<T, GRID, false, true, SOLVER, DIAG>(a, i, nsub, niter, w);
    else cape_column_run<T, GRID, false, false, SOLVER, DIAG>(a, i, nsub, niter, w);
    s += nsub;
    it += niter;
  }
  if (counters) {
    counters[0] += s;
    counters[1] += it;
  }
}

template <typename T, int GRID, int SOLVER>
static void cape_loop_s(const CapeArgs &a, long long *counters) {
  if (a.diag) cape_loop_d<T, GRID, SOLVER, true>(a, counters);
  else cape_loop_d<T, GRID, SOLVER, false>(a, counters);
}

template <typename T, int GRID>
static void cape_loop(const CapeArgs &a, long long *counters) {
  switch (a.guess) {
    case 0: cape_loop_s<T, GRID, SOLVE_PLAIN>(a, counters); break;
    case 1: cape_loop_s<T, GRID, SOLVE_LEARNED>(a, counters); break;
    case 2: cape_loop_s<T, GRID, SOLVE_ACCEL>(a, counters); break;
    case 3: cape_loop_s<T, GRID, SOLVE_SECANT>(a, counters); break;
    default: cape_loop_s<T, GRID, SOLVE_LEARNED_ALL>(a, counters); break;
  }
}

// The double-precision plain solver (the FP64 retry's column routine) on
// every column.
template <typename T, int GRID>
static void cape64_loop(const CapeArgs &a) {
  const bool ice = a.adiabat >= 3, pseudo = (a.adiabat == 1 || a.adiabat == 3);
  for (long long i = 0; i < a.n2; ++i) {
    int nsub = 0, niter = 0;
    if (ice && pseudo) cape_column_run<T, GRID, true, true, SOLVE_PLAIN, false, double>(a, i, nsub, niter);
    else if (ice) cape_column_run<T, GRID, true, false, SOLVE_PLAIN, false, double>(a, i, nsub, niter);
    else if (pseudo) cape_column_run<T, GRID, false, true, SOLVE_PLAIN, false, double>(a, i, nsub, niter);
    else cape_column_run<T, GRID, false, false, SOLVE_PLAIN, false, double>(a, i, nsub, niter);
  }
}

extern "C" int emu_cape64(int grid, const void *p, const void *t, const void *td, const void *ps,
                          const void *ts, const void *tds, int dtype, float pinc, int source,
                          float ml_depth, int adiabat, const int *start, int nk, long long n2,
                          float *cape, float *cin, int *mulvl, float *z_out, int *status) {
  CapeArgs a;
  a.grid = grid; a.dtype = dtype; a.p = p; a.t = t; a.td = td; a.ps = ps; a.ts = ts; a.tds = tds;
  a.start = grid == 1 ? nullptr : start; a.pinc = pinc; a.source = source; a.ml_depth = ml_depth;
  a.adiabat = adiabat; a.nk = nk; a.n2 = n2; a.guess = 0; a.perm = nullptr; a.cape = cape;
  a.cin = cin; a.mulvl = mulvl; a.z_out = z_out; a.status = status; a.counters = nullptr;
  a.guess_w = nullptr;
  if (dtype == 0) {
    if (grid == 1) cape64_loop<float, 1>(a);
    else if (grid == 2) cape64_loop<float, 2>(a);
    else cape64_loop<float, 3>(a);
  } else {
    if (grid == 1) cape64_loop<double, 1>(a);
    else if (grid == 2) cape64_loop<double, 2>(a);
    else cape64_loop<double, 3>(a);
  }
  return 0;
}

extern "C" int emu_cape(int grid, const void *p, const void *t, const void *td, const void *ps,
                        const void *ts, const void *tds, int dtype, float pinc, int source,
                        float ml_depth, int adiabat, const int *start, int nk, long long n2,
                        float *cape, float *cin, int *mulvl, float *z_out, int *status,
                        long long *counters, int guess, const float *guess_w, float *diag) {
  CapeArgs a;
  a.diag = diag;
  a.grid = grid; a.dtype = dtype; a.p = p; a.t = t; a.td = td; a.ps = ps; a.ts = ts; a.tds = tds;
  a.start = grid == 1 ? nullptr : start; a.pinc = pinc; a.source = source; a.ml_depth = ml_depth;
  a.adiabat = adiabat; a.nk = nk; a.n2 = n2; a.guess = guess; a.perm = nullptr; a.cape = cape; a.cin = cin;
  a.mulvl = mulvl; a.z_out = z_out; a.status = status; a.counters = nullptr;
  // the column code reads the packed copy the kernels keep in shared memory
  alignas(16) static float packed[GUESS_NPARAM + 3];
  if (guess_w)
    for (int k = 0; k < GUESS_NPARAM; ++k) packed[k] = guess_packed_value(guess_w, k);
  a.guess_w = guess_w ? packed : nullptr;
  if (dtype == 0) {
    if (grid == 1) cape_loop<float, 1>(a, counters);
    else if (grid == 2) cape_loop<float, 2>(a, counters);
    else cape_loop<float, 3>(a, counters);
  } else {
    if (grid == 1) cape_loop<double, 1>(a, counters);
    else if (grid == 2) cape_loop<double, 2>(a, counters);
    else cape_loop<double, 3>(a, counters);
  }
  return 0;
}

extern "C" int emu_srh(int grid, const void *p, const void *t, const void *td, const void *u,
                       const void *v, const void *ps, const void *ts, const void *tds,
                       const void *us, const void *vs, int dtype, const int *start, double depth,
                       double aglh0, int nk, long long n2, double *srh_rm, double *srh_lm,
                       float *rm, float *lm, float *mean6, int precision) {
  SrhArgs a;
  a.grid = grid; a.dtype = dtype; a.p = p; a.t = t; a.td = td; a.u = u; a.v = v; a.ps = ps;
  a.ts = ts; a.tds = tds; a.us = us; a.vs = vs; a.start = grid == 2 ? start : nullptr;
  a.depth = depth; a.aglh0 = aglh0; a.nk = nk; a.n2 = n2; a.srh_rm = srh_rm; a.srh_lm = srh_lm;
  a.rm = rm; a.lm = lm; a.mean6 = mean6; a.precision = precision;
  for (long long i = 0; i < n2; ++i) {
    if (precision == 1) {
      if (dtype == 0) {
        if (grid == 1) srh_column_run<float, 1, true>(a, i);
        else srh_column_run<float, 2, true>(a, i);
      } else {
        if (grid == 1) srh_column_run<double, 1, true>(a, i);
        else srh_column_run<double, 2, true>(a, i);
      }
    } else if (dtype == 0) {
      if (grid == 1) srh_column_run<float, 1>(a, i);
      else srh_column_run<float, 2>(a, i);
    } else {
      if (grid == 1) srh_column_run<double, 1>(a, i);
      else srh_column_run<double, 2>(a, i);
    }
  }
  return 0;
}

extern "C" void emu_pres_lev_pos(const void *p1d, const void *ps, int dtype, int nk, long long n2,
                                 int *start) {
  for (long long i = 0; i < n2; ++i)
    start[i] = dtype == 0 ? pres_lev_pos_col<float>((const float *)p1d, ((const float *)ps)[i], nk)
                          : pres_lev_pos_col<double>((const double *)p1d, ((const double *)ps)[i], nk);
}

extern "C" float emu_guess_eval(const float *w, float f0, float f1, float f2) {
  return guess_eval(w, f0, f1, f2);
}

extern "C" float emu_guess_eval_packed(const float *w, float f0, float f1, float f2) {
  alignas(16) float packed[GUESS_NPARAM + 3];
  for (int k = 0; k < GUESS_NPARAM; ++k) packed[k] = guess_packed_value(w, k);
  return guess_eval_packed(packed, f0, f1, f2);
}

// accel_map at x with the analytic slope: returns F(x) and writes out[0] =
// F'(x) = F(x) pi2 d expo / d t2, out[1..4] = t2, qv2, ql2, qi2, out[5..7] =
// d/dt2 of qv2, ql2, qi2, out[8] = the saturation mixing ratio.
extern "C" float emu_accel_map(int ice, float x, float p2, float pi2, float lp, float t1,
                               float th1, float qv1, float ql1, float qi1, float qt, float *out) {
  float t2, qv2, ql2, qi2;
  MapSlope ms = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  const float f = ice ? accel_map<true>(x, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, true, t2, qv2,
                                        ql2, qi2, ms)
                      : accel_map<false>(x, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, true, t2,
                                         qv2, ql2, qi2, ms);
  out[0] = f * pi2 * ms.dex;
  out[1] = t2;
  out[2] = qv2;
  out[3] = ql2;
  out[4] = qi2;
  out[5] = ms.dqv;
  out[6] = ms.dql;
  out[7] = ms.dqi;
  out[8] = ms.qsat;
  return f;
}

extern "C" void emu_guess_pairs(long long n, unsigned long long seed, float *feats,
                                float *targets, int *iters, int *adiabats) {
  for (long long i = 0; i < n; ++i)
    iters[i] = guess_pair(seed, i, feats + 3 * i, targets + i, adiabats ? adiabats + i : nullptr);
}

// Size and field offsets of xc_cape_request, for the ctypes layout check.
#include <cstddef>
#include "../../include/xcape_gb300.h"
extern "C" void emu_request_layout(long long *out) {
  out[0] = (long long)sizeof(xc_cape_request);
  out[1] = offsetof(xc_cape_request, n2);
  out[2] = offsetof(xc_cape_request, ld);
  out[3] = offsetof(xc_cape_request, p);
  out[4] = offsetof(xc_cape_request, pinc);
  out[5] = offsetof(xc_cape_request, adiabat);
  out[6] = offsetof(xc_cape_request, cape);
  out[7] = offsetof(xc_cape_request, status);
}
