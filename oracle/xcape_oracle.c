/*
 * xcape_oracle.c -- CPU restatement of xcape's Fortran column kernels.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA product
 * path is compared against; only tests/, __graft_entry__.smoke() and the CPU
 * legs of bench.py load it.  Nothing in the xcape_gb300 package imports it.
 *
 * It restates, in plain C, the algorithms of the reference Fortran
 * (paths relative to the reference project):
 *
 *   src/xcape/fortran/CAPE_CODE_model_lev.f90     loopcape_ml    :4-91
 *                                                 getcape_ml     :97-564
 *                                                 getqvs/getqvi  :570-598
 *                                                 getthe         :604-620
 *   src/xcape/fortran/CAPE_CODE_pressure_lev.f90  loopcape_pl    :4-84
 *                                                 loopcape_pl1d  :88-169
 *                                                 getcape_pl     :174-642 (== getcape_ml)
 *   src/xcape/fortran/stdheight_2D_model_lev.f90  loop_stdheight_ml :4-34, stdheight_ml :74-160
 *   src/xcape/fortran/stdheight_2D_pressure_lev.f90 loop_stdheight_pl :5-47,
 *                                                 loop_stdheight_pl1d :65-93
 *   src/xcape/fortran/Bunkers_model_lev.f90       bunkers_loop_ml :4-69, bunkers_calc_ml :75-180,
 *                                                 DINTERP2DZ :188-236
 *   src/xcape/fortran/Bunkers_pressure_lev.f90    bunkers_loop_pl :4-78
 *   src/xcape/fortran/SREH_model_lev.f90          loop_sreh_ml :4-55, DCALRELHL_ml :61-118,
 *                                                 INTERP1 :123-129
 *   src/xcape/fortran/SREH_pressure_lev.f90       loop_sreh_pl :4-63
 *
 * The file is compiled twice:
 *   - default:      `real` is float, literals are single precision and the
 *                   math calls are expf/logf/powf -- the reference's own FP32
 *                   arithmetic (default REAL, no promotion flags in setup.py);
 *   - -DOC_F64:     `real` is double everywhere -- the "FP64 run" against
 *                   which the FP32 error of every path is stated.
 * stdheight and SREH are double precision in the reference already and are
 * built once (in the default pass).
 *
 * Array layout follows the f2py interfaces: a Fortran (nk, n2) array is the
 * C array [n2][nk], i.e. the levels of one column are contiguous; (2, n2)
 * outputs are [n2][2].  Indices written k=1..nk below are Fortran indices;
 * the local arrays are allocated with one spare slot so that they can be
 * used 1-based exactly as in the Fortran.
 *
 * Build with -ffp-contract=off so that x86 and Arm give the same bits.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef OC_F64
typedef double real;
#define LIT(x) x
#define SFX(n) n##_f64
#define R_EXP exp
#define R_LOG log
#define R_POW pow
#define R_SQRT sqrt
#else
typedef float real;
#define LIT(x) x##f
#define SFX(n) n##_f32
#define R_EXP expf
#define R_LOG logf
#define R_POW powf
#define R_SQRT sqrtf
#endif

#define OC_EXPORT __attribute__((visibility("default")))

/* Per-column status bits (also used by the CUDA path). */
#define OC_COL_NOCONV 1    /* moist-adiabat iteration exceeded 100 steps */
#define OC_COL_BADSTART 2  /* pressure-level start index out of range    */

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

/* ---------------------------------------------------------------------- */
/* CAPE_CODE_model_lev.f90:570-581 */
static real getqvs(real p, real t) {
  const real eps = LIT(287.04) / LIT(461.5);
  real es = LIT(611.2) * R_EXP(LIT(17.67) * (t - LIT(273.15)) / (t - LIT(29.65)));
  return eps * es / (p - es);
}

/* CAPE_CODE_model_lev.f90:587-598 */
static real getqvi(real p, real t) {
  const real eps = LIT(287.04) / LIT(461.5);
  real es = LIT(611.2) * R_EXP(LIT(21.8745584) * (t - LIT(273.15)) / (t - LIT(7.66)));
  return eps * es / (p - es);
}

/* Dewpoint (K) of mixing ratio q at pressure p (Pa): getqvs solved for t. */
static real dewpoint_of(real p, real q) {
  const real eps = LIT(287.04) / LIT(461.5);
  const real a = R_LOG(q * p / (eps + q) / LIT(611.2));
  return (LIT(17.67) * LIT(273.15) - LIT(29.65) * a) / (LIT(17.67) - a);
}

/* CAPE_CODE_model_lev.f90:604-620; x**(-1) is 1/x. */
static real getthe(real p, real t, real td, real q) {
  real tlcl;
  if ((td - t) >= -LIT(0.1)) {
    tlcl = t;
  } else {
    tlcl = LIT(56.0) + LIT(1.0) / (LIT(1.0) / (td - LIT(56.0)) + LIT(0.00125) * R_LOG(t / td));
  }
  return t * (R_POW(LIT(100000.0) / p, LIT(0.2854) * (LIT(1.0) - LIT(0.28) * q))) *
         R_EXP(((LIT(3376.0) / tlcl) - LIT(2.54)) * q * (LIT(1.0) + LIT(0.81) * q));
}

/* getcape_ml, CAPE_CODE_model_lev.f90:97-564.
 * p_A/t_A/td_A hold nk_in levels (p_A may be strided: p_stride 0 means the
 * same column for every call is not needed -- the caller passes the slice).
 * Returns the number of sub-steps and iterations through *nsub / *niter. */
static void getcape(const real *p_A, const real *t_A, const real *td_A, real ps_B, real ts_B,
                    real tds_B, real pinc, int source, real ml_depth, int adiabat, int nk_in,
                    real *cape_out, real *cin_out, int *mulvl_out, real *z_out_out,
                    int *nsub_out, int *niter_out, int *status_out, float *bmin_out,
                    real *diag_out) {
  /* CAPE_CODE_model_lev.f90:188-211 */
  const real g = LIT(9.81);
  const real p00 = LIT(100000.0);
  const real cp = LIT(1005.7);
  const real rd = LIT(287.04);
  const real rv = LIT(461.5);
  const real xlv = LIT(2501000.0);
  const real xls = LIT(2836017.0);
  const real t0 = LIT(273.15);
  const real cpv = LIT(1875.0);
  const real cpl = LIT(4190.0);
  const real cpi = LIT(2118.636);
  const real lv1 = xlv + (cpl - cpv) * t0;
  const real lv2 = cpl - cpv;
  const real ls1 = xls + (cpi - cpv) * t0;
  const real ls2 = cpi - cpv;
  const real rp00 = LIT(1.0) / p00;
  const real reps = rv / rd;
  const real rddcp = rd / cp;
  const real cpdg = cp / g;
  const real rddcp_term = rd / cp; /* the rd/cp inside th2's exponent */
  const real converge = LIT(0.0002);

  const int nk = nk_in + 1; /* :219 */
  real *buf = (real *)malloc(sizeof(real) * 9 * (size_t)(nk + 2));
  real *p = buf, *t = p + nk + 2, *td = t + nk + 2, *pi = td + nk + 2, *q = pi + nk + 2;
  real *z = q + nk + 2, *th = z + nk + 2, *thv = th + nk + 2, *pin = thv + nk + 2;
  int k, kmax = 1, n, nloop, i;
  int mulvl;
  real z_out, cape, cin;
  real maxthe, the, parea, narea;
  real th1, p1, t1, qv1, ql1, qi1, b1, qt, dp, dz, frac;
  real th2, p2, t2, qv2, ql2, qi2, b2, pi2, thv2;
  real thlast, fliq, fice, tbar, qvbar, qlbar, qibar, lhv, lhs, rm, cpm;
  double avgth = 0.0, avgqv = 0.0; /* real*8, :183 */
  int doit, ice, not_converged;
  int nsub = 0, niter = 0, status = 0;
  double bmin = INFINITY; /* smallest |buoyancy| met by the ascent (test statistic) */
  /* Diagnostics the reference computes and discards (the crossing pressure
   * ps of :511 and :526, the parcel's theta-e): LFC and EL pressure (hPa)
   * and height (m), source height and theta-e.  LFC: the lowest point of the
   * first layer with positive area -- the neg->pos crossing, or the layer's
   * base when the parcel is already buoyant there.  EL: the highest pos->neg
   * crossing, or the last level reached when the parcel is still buoyant
   * there.  All -999999 when the parcel never has positive area, when the
   * ascent does not run, or when the iteration gives up. */
  const real dmiss = LIT(-999999.);
  real d_plfc = dmiss, d_zlfc = dmiss, d_pel = dmiss, d_zel = dmiss, d_zsrc = dmiss,
       d_the = dmiss;
  int have_lfc = 0, ascended = 0;
  if (diag_out)
    for (int d = 0; d < 6; ++d) diag_out[d] = dmiss;

  /* :220-225 -- surface first, then the 3-D levels; then :232-240 */
  for (k = 1; k <= nk; ++k) {
    real pi_k, ti_k, tdi_k;
    if (k == 1) {
      pi_k = ps_B; ti_k = ts_B; tdi_k = tds_B;
    } else {
      pi_k = p_A[k - 2]; ti_k = t_A[k - 2]; tdi_k = td_A[k - 2];
    }
    pin[k] = pi_k;
    p[k] = LIT(100.0) * pi_k;
    t[k] = LIT(273.15) + ti_k;
    td[k] = LIT(273.15) + tdi_k;
    pi[k] = R_POW(p[k] * rp00, rddcp);
    q[k] = getqvs(p[k], td[k]);
    th[k] = t[k] / pi[k];
    thv[k] = th[k] * (LIT(1.0) + reps * q[k]) / (LIT(1.0) + q[k]);
  }
  (void)pin;

  /* :244-248 */
  z[1] = LIT(0.0);
  for (k = 2; k <= nk; ++k) {
    dz = -cpdg * LIT(0.5) * (thv[k] + thv[k - 1]) * (pi[k] - pi[k - 1]);
    z[k] = z[k - 1] + dz;
  }

  /* :252-253 */
  mulvl = -999999;
  z_out = LIT(-999999.);

  /* :257-352 source selection; invalid sources are rejected by the caller */
  if (source == 1) {
    kmax = 1;
  } else if (source == 2) {
    if (p[1] < LIT(50000.0)) {
      kmax = 1;
    } else {
      maxthe = LIT(0.0);
      for (k = 1; k <= nk; ++k) {
        if (p[k] >= LIT(50000.0)) {
          the = getthe(p[k], t[k], td[k], q[k]);
          if (the > maxthe) {
            mulvl = k;
            maxthe = the;
            kmax = k;
          }
        }
      }
    }
  } else { /* source == 3 */
    if ((z[2] - z[1]) > ml_depth) {
      avgth = th[1];
      avgqv = q[1];
      kmax = 1;
    } else if (z[nk] < ml_depth) {
      avgth = th[nk];
      avgqv = q[nk];
      kmax = nk;
    } else {
      avgth = 0.0;
      avgqv = 0.0;
      k = 2;
      while (k <= nk && z[k] <= ml_depth) {
        avgth = avgth + (double)(LIT(0.5) * (z[k] - z[k - 1]) * (th[k] + th[k - 1]));
        avgqv = avgqv + (double)(LIT(0.5) * (z[k] - z[k - 1]) * (q[k] + q[k - 1]));
        k = k + 1;
      }
      if (k <= nk) {
        th2 = th[k - 1] + (th[k] - th[k - 1]) * (ml_depth - z[k - 1]) / (z[k] - z[k - 1]);
        qv2 = q[k - 1] + (q[k] - q[k - 1]) * (ml_depth - z[k - 1]) / (z[k] - z[k - 1]);
      } else {
        /* z(nk) == ml_depth exactly: the Fortran reads one slot past the
         * column, multiplied by (ml_depth - z(k-1)) == 0. */
        th2 = th[k - 1];
        qv2 = q[k - 1];
      }
      avgth = avgth + (double)(LIT(0.5) * (ml_depth - z[k - 1]) * (th2 + th[k - 1]));
      avgqv = avgqv + (double)(LIT(0.5) * (ml_depth - z[k - 1]) * (qv2 + q[k - 1]));
      avgth = avgth / (double)ml_depth;
      avgqv = avgqv / (double)ml_depth;
      kmax = 1;
    }
  }

  /* :355-393 parcel at its initial location */
  narea = LIT(0.0);
  if (source == 1 || source == 2) {
    k = kmax;
    th2 = th[kmax];
    pi2 = pi[kmax];
    p2 = p[kmax];
    t2 = t[kmax];
    thv2 = thv[kmax];
    qv2 = q[kmax];
    b2 = LIT(0.0);
  } else {
    k = kmax;
    th2 = (real)avgth;
    qv2 = (real)avgqv;
    thv2 = th2 * (LIT(1.0) + reps * qv2) / (LIT(1.0) + qv2);
    pi2 = pi[kmax];
    p2 = p[kmax];
    t2 = th2 * pi2;
    b2 = g * (thv2 - thv[kmax]) / thv[kmax];
    bmin = fabs((double)b2);
  }
  (void)thv2;
  if (diag_out) {
    d_zsrc = z[kmax];
    d_the = (source == 3) ? getthe(p2, t2, dewpoint_of(p2, qv2), qv2)
                          : getthe(p[kmax], t[kmax], td[kmax], q[kmax]);
  }
  ql2 = LIT(0.0);
  qi2 = LIT(0.0);
  qt = qv2;
  cape = LIT(0.0);
  cin = LIT(0.0);
  doit = 1;
  ice = !(adiabat == 1 || adiabat == 2);

  /* :403-559 ascent */
  while (doit && (k < nk)) {
    k = k + 1;
    b1 = b2;
    dp = p[k - 1] - p[k];
    if (dp < pinc) {
      nloop = 1;
    } else {
      nloop = 1 + (int)(dp / pinc);
      dp = dp / (real)nloop;
    }
    for (n = 1; n <= nloop; ++n) {
      p1 = p2;
      t1 = t2;
      th1 = th2;
      qv1 = qv2;
      ql1 = ql2;
      qi1 = qi2;
      p2 = p2 - dp;
      pi2 = R_POW(p2 * rp00, rddcp);
      thlast = th1;
      i = 0;
      not_converged = 1;
      ++nsub;
      while (not_converged) {
        i = i + 1;
        ++niter;
        t2 = thlast * pi2;
        if (ice) {
          fliq = (t2 - LIT(233.15)) / (LIT(273.15) - LIT(233.15));
          fliq = fliq < LIT(1.0) ? fliq : LIT(1.0);
          fliq = fliq > LIT(0.0) ? fliq : LIT(0.0);
          fice = LIT(1.0) - fliq;
        } else {
          fliq = LIT(1.0);
          fice = LIT(0.0);
        }
        {
          real qsat = fliq * getqvs(p2, t2) + fice * getqvi(p2, t2);
          qv2 = qt < qsat ? qt : qsat;
        }
        qi2 = fice * (qt - qv2);
        qi2 = qi2 > LIT(0.0) ? qi2 : LIT(0.0);
        ql2 = qt - qv2 - qi2;
        ql2 = ql2 > LIT(0.0) ? ql2 : LIT(0.0);

        tbar = LIT(0.5) * (t1 + t2);
        qvbar = LIT(0.5) * (qv1 + qv2);
        qlbar = LIT(0.5) * (ql1 + ql2);
        qibar = LIT(0.5) * (qi1 + qi2);

        lhv = lv1 - lv2 * tbar;
        lhs = ls1 - ls2 * tbar;

        rm = rd + rv * qvbar;
        cpm = cp + cpv * qvbar + cpl * qlbar + cpi * qibar;
        th2 = th1 * R_EXP(lhv * (ql2 - ql1) / (cpm * tbar) + lhs * (qi2 - qi1) / (cpm * tbar) +
                          (rm / cpm - rddcp_term) * R_LOG(p2 / p1));
        if (i > 100) { /* :465-474 */
          cape = LIT(0.0);
          cin = LIT(0.0);
          status |= OC_COL_NOCONV;
          goto done;
        }
        if (fabs((double)(th2 - thlast)) > (double)converge) {
          thlast = thlast + LIT(0.3) * (th2 - thlast);
        } else {
          not_converged = 0;
        }
      }
      if (adiabat == 1 || adiabat == 3) { /* :487-491 pseudoadiabat */
        qt = qv2;
        ql2 = LIT(0.0);
        qi2 = LIT(0.0);
      }
    }

    /* :501-503 */
    thv2 = th2 * (LIT(1.0) + reps * qv2) / (LIT(1.0) + qv2 + ql2 + qi2);
    b2 = g * (thv2 - thv[k]) / thv[k];
    if (fabs((double)b2) < bmin) bmin = fabs((double)b2);
    dz = -cpdg * LIT(0.5) * (thv[k] + thv[k - 1]) * (pi[k] - pi[k - 1]);

    if (diag_out) {
      ascended = 1;
      if ((b2 >= LIT(0.0)) && (b1 < LIT(0.0))) {
        const real w = (LIT(0.0) - b1) / (b2 - b1);
        if (!have_lfc) {
          d_plfc = (p[k - 1] + (p[k] - p[k - 1]) * w) / LIT(100.0);
          d_zlfc = z[k - 1] + dz * w;
          have_lfc = 1;
        }
      } else if ((b2 < LIT(0.0)) && (b1 > LIT(0.0))) {
        const real w = (LIT(0.0) - b1) / (b2 - b1);
        if (!have_lfc) {
          d_plfc = p[k - 1] / LIT(100.0);
          d_zlfc = z[k - 1];
          have_lfc = 1;
        }
        d_pel = (p[k - 1] + (p[k] - p[k - 1]) * w) / LIT(100.0);
        d_zel = z[k - 1] + dz * w;
      } else if (b2 >= LIT(0.0)) {
        if (!have_lfc) {
          d_plfc = p[k - 1] / LIT(100.0);
          d_zlfc = z[k - 1];
          have_lfc = 1;
        }
      }
    }

    /* :509-547 */
    if ((b2 >= LIT(0.0)) && (b1 < LIT(0.0))) {
      frac = b2 / (b2 - b1);
      parea = LIT(0.5) * b2 * dz * frac;
      narea = narea - LIT(0.5) * b1 * dz * (LIT(1.0) - frac);
      cin = cin + narea;
      narea = LIT(0.0);
    } else if ((b2 < LIT(0.0)) && (b1 > LIT(0.0))) {
      frac = b1 / (b1 - b2);
      parea = LIT(0.5) * b1 * dz * frac;
      narea = -LIT(0.5) * b2 * dz * (LIT(1.0) - frac);
    } else if (b2 < LIT(0.0)) {
      parea = LIT(0.0);
      narea = narea - LIT(0.5) * dz * (b1 + b2);
    } else {
      parea = LIT(0.5) * dz * (b1 + b2);
      narea = LIT(0.0);
    }
    cape = cape + (LIT(0.0) > parea ? LIT(0.0) : parea);

    /* :554-558 */
    if ((p[k] <= LIT(10000.0)) && (b2 < LIT(0.0))) doit = 0;
    z_out = z[k];
  }

  if (diag_out && have_lfc && b2 >= LIT(0.0)) {
    d_pel = p[k] / LIT(100.0);
    d_zel = z[k];
  }
  if (diag_out) {
    if (ascended) {
      diag_out[0] = have_lfc ? d_plfc : dmiss;
      diag_out[1] = have_lfc ? d_zlfc : dmiss;
      diag_out[2] = have_lfc ? d_pel : dmiss;
      diag_out[3] = have_lfc ? d_zel : dmiss;
      diag_out[4] = d_zsrc;
      diag_out[5] = d_the;
    }
  }

done:
  *cape_out = cape;
  *cin_out = cin;
  *mulvl_out = mulvl;
  *z_out_out = z_out;
  if (nsub_out) *nsub_out = nsub;
  if (niter_out) *niter_out = niter;
  if (status_out) *status_out = status;
  if (bmin_out) *bmin_out = (float)bmin;
  free(buf);
}

/* loopcape_ml, CAPE_CODE_model_lev.f90:76-89: the ts > 0 gate. */
static void loopcape_ml_common(const real *p3d, const real *t3d, const real *td3d,
                               const real *ps, const real *ts, const real *tds, real pinc,
                               int source, real ml_depth, int adiabat, int nk, int n2, real *cape,
                               real *cin, int *mulvl, real *z_out, int *nsub, int *niter,
                               int *status, float *bmin, real *diag, int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(dynamic, 64)
  for (i = 0; i < n2; ++i) {
    if (bmin) bmin[i] = INFINITY;
    if (diag)
      for (int d = 0; d < 6; ++d) diag[6 * i + d] = LIT(-999999.);
    if (ts[i] > LIT(0.0)) {
      getcape(p3d + (size_t)i * nk, t3d + (size_t)i * nk, td3d + (size_t)i * nk, ps[i], ts[i],
              tds[i], pinc, source, ml_depth, adiabat, nk, &cape[i], &cin[i], &mulvl[i],
              &z_out[i], nsub ? &nsub[i] : 0, niter ? &niter[i] : 0, status ? &status[i] : 0,
              bmin ? &bmin[i] : 0, diag ? diag + 6 * i : 0);
    } else {
      cape[i] = LIT(0.0);
      cin[i] = LIT(0.0);
      z_out[i] = LIT(0.0);
      mulvl[i] = 0;
      if (nsub) nsub[i] = 0;
      if (niter) niter[i] = 0;
      if (status) status[i] = 0;
    }
  }
}

OC_EXPORT void SFX(oc_loopcape_ml)(const real *p3d, const real *t3d, const real *td3d,
                                   const real *ps, const real *ts, const real *tds, real pinc,
                                   int source, real ml_depth, int adiabat, int nk, int n2,
                                   real *cape, real *cin, int *mulvl, real *z_out, int *nsub,
                                   int *niter, int *status, float *bmin, int nthreads) {
  loopcape_ml_common(p3d, t3d, td3d, ps, ts, tds, pinc, source, ml_depth, adiabat, nk, n2, cape,
                     cin, mulvl, z_out, nsub, niter, status, bmin, 0, nthreads);
}

/* loopcape_ml with the diagnostics of getcape: diag [n2][6] = LFC pressure
 * (hPa), LFC height (m), EL pressure, EL height, source height, source
 * theta-e (K); -999999 where undefined. */
OC_EXPORT void SFX(oc_loopcape_diag_ml)(const real *p3d, const real *t3d, const real *td3d,
                                        const real *ps, const real *ts, const real *tds,
                                        real pinc, int source, real ml_depth, int adiabat, int nk,
                                        int n2, real *cape, real *cin, int *mulvl, real *z_out,
                                        int *status, real *diag, int nthreads) {
  loopcape_ml_common(p3d, t3d, td3d, ps, ts, tds, pinc, source, ml_depth, adiabat, nk, n2, cape,
                     cin, mulvl, z_out, 0, 0, status, 0, diag, nthreads);
}

/* loopcape_pl1d (CAPE_CODE_pressure_lev.f90:151-167) when p_stride == 0 and
 * loopcape_pl (:66-82) when p_stride == nk: column i uses levels
 * start(i)..nk of its profile. */
static void loopcape_pl_common(const real *p3d, long p_stride, const real *t3d, const real *td3d,
                               const real *ps, const real *ts, const real *tds, real pinc,
                               int source, real ml_depth, int adiabat, const int *start, int nk,
                               int n2, real *cape, real *cin, int *mulvl, real *z_out, int *nsub,
                               int *niter, int *status, float *bmin, real *diag, int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(dynamic, 64)
  for (i = 0; i < n2; ++i) {
    int st = start[i];
    if (bmin) bmin[i] = INFINITY;
    if (diag)
      for (int d = 0; d < 6; ++d) diag[6 * i + d] = LIT(-999999.);
    if (ts[i] > LIT(0.0) && st >= 1 && st <= nk) {
      int nk_pl_in = nk - st + 1;
      getcape(p3d + (size_t)i * p_stride + (st - 1), t3d + (size_t)i * nk + (st - 1),
              td3d + (size_t)i * nk + (st - 1), ps[i], ts[i], tds[i], pinc, source, ml_depth,
              adiabat, nk_pl_in, &cape[i], &cin[i], &mulvl[i], &z_out[i], nsub ? &nsub[i] : 0,
              niter ? &niter[i] : 0, status ? &status[i] : 0, bmin ? &bmin[i] : 0,
              diag ? diag + 6 * i : 0);
    } else {
      cape[i] = LIT(0.0);
      cin[i] = LIT(0.0);
      z_out[i] = LIT(0.0);
      mulvl[i] = 0;
      if (nsub) nsub[i] = 0;
      if (niter) niter[i] = 0;
      if (status) status[i] = (ts[i] > LIT(0.0)) ? OC_COL_BADSTART : 0;
    }
  }
}

OC_EXPORT void SFX(oc_loopcape_pl1d)(const real *t3d, const real *td3d, const real *p1d,
                                     const real *ps, const real *ts, const real *tds, real pinc,
                                     int source, real ml_depth, int adiabat, const int *start,
                                     int nk, int n2, real *cape, real *cin, int *mulvl,
                                     real *z_out, int *nsub, int *niter, int *status,
                                     float *bmin, int nthreads) {
  loopcape_pl_common(p1d, 0, t3d, td3d, ps, ts, tds, pinc, source, ml_depth, adiabat, start, nk,
                     n2, cape, cin, mulvl, z_out, nsub, niter, status, bmin, 0, nthreads);
}

/* loopcape_pl1d with the diagnostics (see oc_loopcape_diag_ml). */
OC_EXPORT void SFX(oc_loopcape_diag_pl1d)(const real *t3d, const real *td3d, const real *p1d,
                                          const real *ps, const real *ts, const real *tds,
                                          real pinc, int source, real ml_depth, int adiabat,
                                          const int *start, int nk, int n2, real *cape,
                                          real *cin, int *mulvl, real *z_out, int *status,
                                          real *diag, int nthreads) {
  loopcape_pl_common(p1d, 0, t3d, td3d, ps, ts, tds, pinc, source, ml_depth, adiabat, start, nk,
                     n2, cape, cin, mulvl, z_out, 0, 0, status, 0, diag, nthreads);
}

OC_EXPORT void SFX(oc_loopcape_pl)(const real *p3d, const real *t3d, const real *td3d,
                                   const real *ps, const real *ts, const real *tds, real pinc,
                                   int source, real ml_depth, int adiabat, const int *start,
                                   int nk, int n2, real *cape, real *cin, int *mulvl, real *z_out,
                                   int *nsub, int *niter, int *status, float *bmin,
                                   int nthreads) {
  loopcape_pl_common(p3d, nk, t3d, td3d, ps, ts, tds, pinc, source, ml_depth, adiabat, start, nk,
                     n2, cape, cin, mulvl, z_out, nsub, niter, status, bmin, 0, nthreads);
}

/* ---------------------------------------------------------------------- */
/* DINTERP2DZ for one column (N2 = 1), Bunkers_model_lev.f90:188-236. */
static real dinterp2dz(const real *v3d, const real *z, real loc, int nz) {
  real height = loc;
  real vmsg = LIT(-999999.);
  int ip = 0, im = 1, kp, interp = 0;
  real v2d = vmsg;
  if (z[0] > z[nz - 1]) {
    ip = 1;
    im = 0;
  }
  kp = nz;
  while (!interp && kp >= 2) {
    /* Fortran Z(KP-IM) is z[kp-im-1] */
    if ((z[kp - im - 1] <= height) && (z[kp - ip - 1] > height)) {
      real w2 = (height - z[kp - im - 1]) / (z[kp - ip - 1] - z[kp - im - 1]);
      real w1 = (real)(1.0 - (double)w2); /* W1 = 1.D0 - W2 */
      v2d = w1 * v3d[kp - im - 1] + w2 * v3d[kp - ip - 1];
      interp = 1;
    }
    kp = kp - 1;
  }
  return v2d;
}

/* bunkers_calc_ml, Bunkers_model_lev.f90:75-180, on the assembled column
 * (surface first).  Mean6kmwind starts at zero (f2py zero-fills intent(out));
 * ushr_u/vshr_u/ushr_d/vshr_d are read before being set in the Fortran and
 * are taken as zero here. */
static void bunkers_calc(const real *u, const real *v, const real *aglh, int nk, real *rm, real *lm,
                         real *mean) {
  static const float lv[12] = {500.f,  1000.f, 1500.f, 2000.f, 2500.f, 3000.f,
                               3500.f, 4000.f, 4500.f, 5000.f, 5500.f, 6000.f};
  real us6[13], vs6[13];
  real m0 = LIT(0.0), m1 = LIT(0.0);
  real ushr_u = LIT(0.0), vshr_u = LIT(0.0), ushr_d = LIT(0.0), vshr_d = LIT(0.0);
  real ushr, vshr;
  int i;
  for (i = 1; i <= 13; ++i) {
    if (i == 1) {
      us6[0] = u[0];
      vs6[0] = v[0];
    } else {
      us6[i - 1] = dinterp2dz(u, aglh, (real)lv[i - 2], nk);
      vs6[i - 1] = dinterp2dz(v, aglh, (real)lv[i - 2], nk);
    }
  }
  for (i = 0; i < 13; ++i) {
    m0 = m0 + us6[i];
    m1 = m1 + vs6[i];
  }
  m0 = m0 / (real)13;
  m1 = m1 / (real)13;
  for (i = 11; i < 13; ++i) {
    ushr_u = ushr_u + us6[i];
    vshr_u = vshr_u + vs6[i];
  }
  ushr_u = ushr_u / (real)2;
  vshr_u = vshr_u / (real)2;
  for (i = 0; i < 2; ++i) {
    ushr_d = ushr_d + us6[i];
    vshr_d = vshr_d + vs6[i];
  }
  ushr_d = ushr_d / (real)2;
  vshr_d = vshr_d / (real)2;
  ushr = ushr_u - ushr_d;
  vshr = vshr_u - vshr_d;
  /* (x**2 + y**2)**0.5: the square root of a non-negative value */
  {
    real nrm = R_SQRT(ushr * ushr + vshr * vshr);
    rm[0] = m0 + LIT(7.5) * vshr / nrm;
    rm[1] = m1 - LIT(7.5) * ushr / nrm;
    lm[0] = m0 - LIT(7.5) * vshr / nrm;
    lm[1] = m1 + LIT(7.5) * ushr / nrm;
  }
  mean[0] = m0;
  mean[1] = m1;
}

/* bunkers_loop_ml (:58-67) with start == NULL, bunkers_loop_pl
 * (Bunkers_pressure_lev.f90:59-77) otherwise. */
static void bunkers_loop_common(const real *U3d, const real *V3d, const real *AGLH3d,
                                const real *Us, const real *Vs, const real *AGLHs,
                                const int *start, int nk, int n2, real *RM, real *LM, real *Mean,
                                int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n2; ++i) {
    real *ua = (real *)malloc(sizeof(real) * 3 * (size_t)(nk + 1));
    real *va = ua + nk + 1, *ha = va + nk + 1;
    int st = start ? start[i] : 1;
    int nk_all, k;
    if (st < 1) st = 1;
    if (st > nk + 1) st = nk + 1;
    nk_all = nk - st + 2;
    ua[0] = Us[i];
    va[0] = Vs[i];
    ha[0] = AGLHs[i];
    for (k = 1; k < nk_all; ++k) {
      ua[k] = U3d[(size_t)i * nk + st - 2 + k];
      va[k] = V3d[(size_t)i * nk + st - 2 + k];
      ha[k] = AGLH3d[(size_t)i * nk + st - 2 + k];
    }
    bunkers_calc(ua, va, ha, nk_all, &RM[2 * i], &LM[2 * i], &Mean[2 * i]);
    free(ua);
  }
}

OC_EXPORT void SFX(oc_bunkers_loop_ml)(const real *U3d, const real *V3d, const real *AGLH3d,
                                       const real *Us, const real *Vs, const real *AGLHs, int nk,
                                       int n2, real *RM, real *LM, real *Mean, int nthreads) {
  bunkers_loop_common(U3d, V3d, AGLH3d, Us, Vs, AGLHs, 0, nk, n2, RM, LM, Mean, nthreads);
}

OC_EXPORT void SFX(oc_bunkers_loop_pl)(const real *U3d, const real *V3d, const real *AGLH3d,
                                       const real *Us, const real *Vs, const real *AGLHs,
                                       const int *start, int nk, int n2, real *RM, real *LM,
                                       real *Mean, int nthreads) {
  bunkers_loop_common(U3d, V3d, AGLH3d, Us, Vs, AGLHs, start, nk, n2, RM, LM, Mean, nthreads);
}

#ifndef OC_F64
/* ---------------------------------------------------------------------- */
/* stdheight_ml, stdheight_2D_model_lev.f90:74-160.  DOUBLE PRECISION with
 * default-REAL literals: 273.15, 287.04, -9.80665, 0.6219800858985514, 6.112,
 * 53.49 and 5.09 are single-precision constants widened to double. */
static void stdheight(const double *P, const double *T, const double *Td, double Ps, double Ts,
                      double Tds, double Hin, int NK, double *H, double *Hs) {
  const double R = (double)287.04f;
  const double g = (double)-9.80665f;
  const double eps = (double)0.6219800858985514f;
  const double c27315 = (double)273.15f;
  const double c6112 = (double)6.112f, c5349 = (double)53.49f, c509 = (double)5.09f;
  double Tin, Tdin, E, w, Tvs, Tv_prev = 0.0, Tv_k;
  int k, k_all;
  Tin = Ts + c27315;
  Tdin = Tds + c27315;
  E = c6112 * exp((c5349 - (6808.0 / Tdin) - c509 * log(Tdin)));
  w = eps * (E / (Ps - E));
  Tvs = Tin * ((w + eps) / (eps * (1.0 + w)));
  *Hs = Hin;
  for (k_all = 2; k_all <= NK + 1; ++k_all) {
    k = k_all - 1; /* Fortran k, 1-based into P/T/Td/H */
    Tin = T[k - 1] + c27315;
    Tdin = Td[k - 1] + c27315;
    E = c6112 * exp((c5349 - (6808.0 / Tdin) - c509 * log(Tdin)));
    w = eps * (E / (P[k - 1] - E));
    Tv_k = Tin * ((w + eps) / (eps * (1.0 + w)));
    if (k_all == 2) {
      H[k - 1] = *Hs + ((R * ((Tv_k + Tvs) / 2.0) / g)) * (log(P[k - 1] / Ps));
    } else {
      H[k - 1] = H[k - 2] + ((R * ((Tv_k + Tv_prev) / 2.0) / g)) * (log(P[k - 1] / P[k - 2]));
    }
    Tv_prev = Tv_k;
  }
}

/* loop_stdheight_ml, :29-32 */
OC_EXPORT void oc_loop_stdheight_ml(const double *P, const double *T, const double *Td,
                                    const double *Ps, const double *Ts, const double *Tds,
                                    const double *Hin, int NK, int NX, double *H, double *Hs,
                                    int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < NX; ++i)
    stdheight(P + (size_t)i * NK, T + (size_t)i * NK, Td + (size_t)i * NK, Ps[i], Ts[i], Tds[i],
              Hin[i], NK, H + (size_t)i * NK, &Hs[i]);
}

/* loop_stdheight_pl1d (stdheight_2D_pressure_lev.f90:79-91) with
 * p_stride == 0, loop_stdheight_pl (:33-45) with p_stride == NK.  Levels
 * below start are set to -999999. */
static void stdheight_pl_common(const double *P, long p_stride, const double *T, const double *Td,
                                const double *Ps, const double *Ts, const double *Tds,
                                const double *Hin, const int *start, int NK, int NX, double *H,
                                double *Hs, int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < NX; ++i) {
    int st = start[i], k;
    if (st < 1) st = 1;
    if (st > NK + 1) st = NK + 1;
    for (k = 1; k < st; ++k) H[(size_t)i * NK + k - 1] = -999999.0;
    stdheight(P + (size_t)i * p_stride + st - 1, T + (size_t)i * NK + st - 1,
              Td + (size_t)i * NK + st - 1, Ps[i], Ts[i], Tds[i], Hin[i], NK - st + 1,
              H + (size_t)i * NK + st - 1, &Hs[i]);
  }
}

OC_EXPORT void oc_loop_stdheight_pl1d(const double *T, const double *Td, const double *P1d,
                                      const double *Ps, const double *Ts, const double *Tds,
                                      const double *Hin, const int *start, int NK, int NX,
                                      double *H, double *Hs, int nthreads) {
  stdheight_pl_common(P1d, 0, T, Td, Ps, Ts, Tds, Hin, start, NK, NX, H, Hs, nthreads);
}

OC_EXPORT void oc_loop_stdheight_pl(const double *P, const double *T, const double *Td,
                                    const double *Ps, const double *Ts, const double *Tds,
                                    const double *Hin, const int *start, int NK, int NX,
                                    double *H, double *Hs, int nthreads) {
  stdheight_pl_common(P, NK, T, Td, Ps, Ts, Tds, Hin, start, NK, NX, H, Hs, nthreads);
}

/* ---------------------------------------------------------------------- */
/* INTERP1, SREH_model_lev.f90:123-129.  X1 is passed by reference and is
 * lowered by 0.01 when X3 == X1; the caller sees the change. */
static double interp1(double y1, double y3, double *x1, double x2, double x3) {
  if (x3 == *x1) *x1 = *x1 - (double)0.01f;
  return y1 + ((y3 - y1) * ((x2 - *x1) / (x3 - *x1)));
}

/* DCALRELHL_ml, SREH_model_lev.f90:61-118 (aglh is the caller's copy). */
static void dcalrelhl(const double *u, const double *v, double *aglh, double cu_rm, double cv_rm,
                      double cu_lm, double cv_lm, double top, int nk, double *sreh_rm,
                      double *sreh_lm, double *utop, double *vtop) {
  int k, ktop = 0;
  double sum, x;
  memcpy(utop, u, sizeof(double) * nk);
  memcpy(vtop, v, sizeof(double) * nk);
  for (k = 2; k <= nk; ++k) {
    if ((aglh[k - 1] > top) && (ktop == 0)) {
      ktop = k;
      utop[ktop - 1] = interp1(u[ktop - 1], u[ktop - 2], &aglh[ktop - 1], top, aglh[ktop - 2]);
      vtop[ktop - 1] = interp1(v[ktop - 1], v[ktop - 2], &aglh[ktop - 1], top, aglh[ktop - 2]);
    }
  }
  sum = 0.0;
  for (k = 2; k <= ktop; ++k) {
    x = ((utop[k - 1] - cu_rm) * (vtop[k - 1] - vtop[k - 2])) -
        ((vtop[k - 1] - cv_rm) * (utop[k - 1] - utop[k - 2]));
    sum = sum + x;
  }
  *sreh_rm = -sum;
  sum = 0.0;
  for (k = 2; k <= ktop; ++k) {
    x = ((utop[k - 1] - cu_lm) * (vtop[k - 1] - vtop[k - 2])) -
        ((vtop[k - 1] - cv_lm) * (utop[k - 1] - utop[k - 2]));
    sum = sum + x;
  }
  *sreh_lm = -sum;
}

/* loop_sreh_ml (:42-53) with start == NULL, loop_sreh_pl
 * (SREH_pressure_lev.f90:43-60) otherwise. */
static void sreh_loop_common(const double *u, const double *v, const double *aglh,
                             const double *us, const double *vs, const double *aglhs,
                             const double *cu_rm, const double *cv_rm, const double *cu_lm,
                             const double *cv_lm, double top, const int *start, int nk, int n2,
                             double *sreh_rm, double *sreh_lm, int nthreads) {
  set_threads(nthreads);
  long i;
#pragma omp parallel for schedule(static)
  for (i = 0; i < n2; ++i) {
    double *ua = (double *)malloc(sizeof(double) * 5 * (size_t)(nk + 1));
    double *va = ua + nk + 1, *ha = va + nk + 1, *ut = ha + nk + 1, *vt = ut + nk + 1;
    int st = start ? start[i] : 1, nk_all, k;
    if (st < 1) st = 1;
    if (st > nk + 1) st = nk + 1;
    nk_all = nk - st + 2;
    ua[0] = us[i];
    va[0] = vs[i];
    ha[0] = aglhs[i];
    for (k = 1; k < nk_all; ++k) {
      ua[k] = u[(size_t)i * nk + st - 2 + k];
      va[k] = v[(size_t)i * nk + st - 2 + k];
      ha[k] = aglh[(size_t)i * nk + st - 2 + k];
    }
    dcalrelhl(ua, va, ha, cu_rm[i], cv_rm[i], cu_lm[i], cv_lm[i], top, nk_all, &sreh_rm[i],
              &sreh_lm[i], ut, vt);
    free(ua);
  }
}

OC_EXPORT void oc_loop_sreh_ml(const double *u, const double *v, const double *aglh,
                               const double *us, const double *vs, const double *aglhs,
                               const double *cu_rm, const double *cv_rm, const double *cu_lm,
                               const double *cv_lm, double top, int nk, int n2, double *sreh_rm,
                               double *sreh_lm, int nthreads) {
  sreh_loop_common(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top, 0, nk, n2,
                   sreh_rm, sreh_lm, nthreads);
}

OC_EXPORT void oc_loop_sreh_pl(const double *u, const double *v, const double *aglh,
                               const double *us, const double *vs, const double *aglhs,
                               const double *cu_rm, const double *cv_rm, const double *cu_lm,
                               const double *cv_lm, double top, const int *start, int nk, int n2,
                               double *sreh_rm, double *sreh_lm, int nthreads) {
  sreh_loop_common(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top, start, nk, n2,
                   sreh_rm, sreh_lm, nthreads);
}

OC_EXPORT int oc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
#endif /* !OC_F64 */
