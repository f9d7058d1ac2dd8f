// cape_column.cuh -- getcape on one column, compiled for the device (the
// CAPE kernels) and for the host (the CPU emulation harness of the tests).
//
// The column is never materialised: every pass walks the levels upward and
// recomputes the environment (p, T, Td -> pi, q, theta, theta_v, z) from the
// input arrays, so the per-column state is a handful of registers.
//
// The arithmetic follows getcape_ml (src/xcape/fortran/CAPE_CODE_model_lev.f90
// :97-564; getcape_pl in CAPE_CODE_pressure_lev.f90:174-642 is the same
// routine) operation for operation, in FP32 with the ML accumulators in FP64
// (:183).  Two loop-invariant hoists keep the results unchanged:
//   * log(p2/p1) is evaluated once per sub-step instead of once per
//     iteration (p1, p2 do not change inside the iteration, :460-462);
//   * in the liquid-only adiabats the ice term lhs*(qi2-qi1)/(cpm*tbar) is
//     identically zero (qi1 = qi2 = 0) and is not evaluated, nor is getqvi
//     whose product with fice = 0 it would be.
//
// The routines are templated on their real type R.  R = float is the
// kernels' arithmetic above.  R = double runs the same plain solver in
// double precision for the FP64 retry of columns whose FP32 iteration gave
// up (cape_retry64_kernel): literals are then the double values of the
// decimal constants, the named physical constants the FP32 program's,
// widened.
#pragma once
#include "guess_mlp.cuh"
#include "xc_common.cuh"
#include "xc_kernels.h"

// A decimal literal in the routine's precision: the single-precision
// literal (x)f for float, the double literal x for double.
#define XC_LIT(R, x) (sizeof(R) == sizeof(float) ? (R)(x##f) : (R)(x))

namespace xc {

XC_HD float xabs(float x) { return fabsf(x); }
XC_HD double xabs(double x) { return fabs(x); }

// Environment of one level (:232-240).
template <typename R = float>
struct EnvT {
  R p, t, td, pi, q, th, thv;
};
using Env = EnvT<float>;

// FAST (the accelerated solvers, float only): pi as 2^(RDDCP log2(p/P00)),
// q from getqvs_fast and the two quotients from approximate divides.
template <bool FAST = false, typename R = float>
XC_HD EnvT<R> make_env(R pin, R tin, R tdin) {
  EnvT<R> e;
  e.p = XC_LIT(R, 100.0) * pin;
  e.t = XC_LIT(R, 273.15) + tin;
  e.td = XC_LIT(R, 273.15) + tdin;
  if constexpr (FAST) {
    static_assert(sizeof(R) == sizeof(float), "the accelerated environment is FP32");
    e.pi = fast_exp2(RDDCP * fast_log2(e.p * RP00));
    e.q = getqvs_fast(e.p, e.td);
    e.th = fast_div(e.t, e.pi);
    e.thv = fast_div(e.th * (1.0f + REPS * e.q), 1.0f + e.q);
  } else {
    e.pi = xpow(e.p * (R)RP00, (R)RDDCP);
    e.q = getqvs(e.p, e.td);
    e.th = e.t / e.pi;
    e.thv = e.th * (XC_LIT(R, 1.0) + (R)REPS * e.q) / (XC_LIT(R, 1.0) + e.q);
  }
  return e;
}

// Reader of one assembled column: level 1 is the surface, level j >= 2 is
// the 1-based input level start + j - 2, i.e. 0-based index start - 3 + j.
// The array pointers are those of all columns (the kernel's arguments) and
// one 64-bit offset locates the column, so that a column costs the ascent
// one register pair instead of three pointers.
template <typename T, int GRID, typename R = float>
struct ColumnReader {
  const T *p;   // GRID 1/3: p of all columns; GRID 2: the shared p1d
  const T *t;   // t of all columns
  const T *td;  // td of all columns
  R ps, ts, tds;
  long long cbase;  // column offset + start - 3: t, td (and GRID 1/3 p) of level j at cbase + j
  int base;         // start - 3: the GRID 2 p of level j at base + j

  XC_HD void set(const T *p_all, const T *t_all, const T *td_all, long long col_off, int start) {
    p = p_all;
    t = t_all;
    td = td_all;
    cbase = col_off + start - 3;
    base = start - 3;
  }
  XC_HD const T *p_at(int j) const { return GRID == 2 ? p + (base + j) : p + (cbase + j); }

  XC_HD void level(int j, R &pin, R &tin, R &tdin) const {
    if (j == 1) {
      pin = ps;
      tin = ts;
      tdin = tds;
    } else {
      pin = (R)ld(p_at(j));
      tin = (R)ld(t + (cbase + j));
      tdin = (R)ld(td + (cbase + j));
    }
  }
  template <bool FAST = false>
  XC_HD EnvT<R> env(int j) const {
    R a, b, c;
    level(j, a, b, c);
    return make_env<FAST, R>(a, b, c);
  }
  // level j >= 2 (above the surface): loops over those levels then need no
  // surface values, which frees their registers
  template <bool FAST = false>
  XC_HD EnvT<R> env_above(int j) const {
    return make_env<FAST, R>((R)ld(p_at(j)), (R)ld(t + (cbase + j)), (R)ld(td + (cbase + j)));
  }
};

struct CapeResult {
  float cape, cin, z_out;
  int mulvl, status;
  int nsub, niter;
};

// Moist-adiabat solvers of a sub-step.
//   SOLVE_PLAIN: the reference's damped fixed point, thlast = th1, step
//                0.3 * (th2 - thlast) (:431-480).
//   SOLVE_ACCEL: same map F, same stopping test |F(x) - x| <= 2e-4 and the
//                same result th2 = F(x), but the first guess extrapolates
//                the previous sub-step's increment (scaled by the ratio of
//                the pressure steps), the first step is a Newton step on
//                g(x) = F(x) - x with F' differentiated analytically at the
//                first evaluation, and from the second evaluation on x
//                moves by a secant step on g.  The fixed
//                0.3 damping contracts by |1 - 0.3 (1 - F')|, about 0.8 for
//                the F' ~ -5 of warm saturated sub-steps, and in FP32 it can
//                lock into a two-value cycle one ulp wide whose step stays
//                above 2e-4 (the reference then gives up after 100
//                iterations); the secant step lands on the fixed point.
//   SOLVE_LEARNED: SOLVE_ACCEL, except on the first sub-step that starts
//                saturated, where the extrapolation has only the partial
//                increment of the sub-step that crossed saturation: there
//                the first guess is th1 plus the guess network's increment
//                (guess_mlp.cuh), entered as the extrapolation history when
//                the parcel saturates.  The network is evaluated once per column,
//                before the ascent, at the parcel's lifting condensation
//                level (lcl_features), where the threads of a warp evaluate
//                it together (warp_guess_eval, cape_learned.cuh; per thread
//                through parcel_lcl_slope in the diagnostics kernel); inside
//                the sub-step loop the threads that reach saturation at
//                different sub-steps would evaluate it one after another.
//   SOLVE_LEARNED_ALL: the network's guess on every sub-step that starts
//                saturated, th1 on the others; secant steps.
//   SOLVE_SECANT: first guess th1 (the reference's), secant steps -- the
//                method without the network, against which
//                SOLVE_LEARNED_ALL shows the network's iteration savings.
// Every mode falls back to its guess without the network when the network's
// output is out of range.
constexpr int SOLVE_PLAIN = 0;
constexpr int SOLVE_ACCEL = 1;
constexpr int SOLVE_LEARNED = 2;
constexpr int SOLVE_SECANT = 3;
constexpr int SOLVE_LEARNED_ALL = 4;
// SOLVE_LEARNED_WARP: SOLVE_ACCEL's Newton and secant steps, with the guess
// network's increment as the first guess of every sub-step that starts
// saturated (the extrapolated guess on the others); the warp evaluates the
// network for its 32 lanes in lockstep at every sub-step, on the tensor cores
// (ascend_col_warp, cape_learned.cuh), and hands each lane its increment in
// SolverState::net_dth.
constexpr int SOLVE_LEARNED_WARP = 5;

struct SolverState {
  // (SOLVE_ACCEL, SOLVE_LEARNED) (th2 - th1) / dp of the previous sub-step;
  // 0 before the first, so that the first guess is th1
  float rate = 0.0f;
  // (SOLVE_ACCEL, SOLVE_LEARNED*) fast_rcp of the current level's sub-step
  // dp, taken once per level for the rate
  float rdp = 0.0f;
  bool saturated = false;   // (SOLVE_LEARNED_ALL) condensate at the end of the last sub-step
  // (SOLVE_LEARNED) the network's output at the parcel's LCL until the
  // parcel first saturates, NaN once used or when there is none
  float lcl_y = NAN;
  float lnp = 0.0f;         // ln of the parcel pressure (accelerated modes)
  const float *guess_w = nullptr;  // packed guess network (guess_packed_value), SOLVE_LEARNED*
  float net_dth = NAN;      // (SOLVE_LEARNED_WARP) this sub-step's network increment, or NaN
};

// The guess network's output y at the lifting condensation level of a parcel
// (p, t, td in Pa and K, mixing ratio q): Bolton's (1980) LCL temperature
// from the temperature and dewpoint, the LCL pressure along the dry
// adiabat, the features (p_lcl, theta-e, q).  Returns false when the
// output is out of the network's range.
// The inputs only steer the first guess, so they use the approximate log,
// exp and divides.
XC_HD void lcl_features(float p, float t, float td, float q, float &f0, float &f1, float &f2) {
  const float tlcl =
      56.0f + fast_div(1.0f, fast_div(1.0f, td - 56.0f) + fast_log(fast_div(t, td)) * (1.0f / 800.0f));
  const float plcl = td < t ? p * fast_exp((1.0f / RDDCP) * fast_log(fast_div(tlcl, t))) : p;
  guess_features(plcl, getthe_fast(p, t, td, q), q, f0, f1, f2);
}

XC_HD bool parcel_lcl_slope(const float *w, float p, float t, float td, float q, float &y) {
  float f0, f1, f2;
  lcl_features(p, t, td, q, f0, f1, f2);
  y = guess_eval_packed(w, f0, f1, f2);
  return y >= GUESS_Y_MIN && y <= GUESS_Y_MAX;
}

// Dewpoint (K) of mixing ratio q at pressure p (Pa): getqvs solved for T.
XC_HD float dewpoint_of(float p, float q) {
  const float a = logf(q * p / (QEPS + q) / 611.2f);
  return (17.67f * 273.15f - 29.65f * a) / (17.67f - a);
}

// theta increment of a sub-step from p1 to p2 that starts saturated at
// (t1, qv1) with total water qt, from the guess network; returns false when
// the network's output is out of its range.
XC_HD bool network_increment(const float *w, float p1, float p2, float t1, float qv1, float qt,
                             float lp, float &dth) {
  float f0, f1, f2;
  guess_features(p2, getthe(p1, t1, t1, qv1), qt, f0, f1, f2);
  const float y = guess_eval_packed(w, f0, f1, f2);
  if (!(y >= GUESS_Y_MIN && y <= GUESS_Y_MAX)) return false;
  dth = -GUESS_SLOPE_SCALE * y * lp;
  return true;
}

// d qsat / dT of qsat = QEPS es / (p - es), es = 611.2 exp(a (T - 273.15) / (T - b))
// (getqvs: a = 17.67, b = 29.65; getqvi: a = 21.8745584, b = 7.66), from the
// parts qsat_fast already has: qsat p / (p - es) * k / (T - b)^2 with
// k = a (273.15 - b).
XC_HD float dqsat_dt(float qsat, float p, const QsatParts &q, float k) {
  return qsat * p * q.rpe * (k * q.rtb) * q.rtb;
}

// The map F of a sub-step (:435-463): th2 = F(x) for the guess x, with t2,
// qv2, ql2, qi2 at x.  The parcel starts the sub-step at (t1, th1, qv1, ql1,
// qi1) with total water qt; p2, pi2 = (p2/P00)^(Rd/cp) and lp = ln(p2/p1).
// plain_map is the reference's sequence of operations.
template <bool ICE, typename R>
XC_HD R plain_map(R x, R p2, R pi2, R lp, R t1, R th1, R qv1, R ql1, R qi1, R qt, R &t2, R &qv2,
                  R &ql2, R &qi2) {
  const R zero = XC_LIT(R, 0.0), one = XC_LIT(R, 1.0), half = XC_LIT(R, 0.5);
  t2 = x * pi2;
  R fliq, fice, qsat;
  if (ICE) {
    fliq = fmax_f(fmin_f((t2 - XC_LIT(R, 233.15)) / (XC_LIT(R, 273.15) - XC_LIT(R, 233.15)), one),
                  zero);
    fice = one - fliq;
    qsat = fliq * getqvs(p2, t2) + fice * getqvi(p2, t2);
  } else {
    fliq = one;
    fice = zero;
    qsat = getqvs(p2, t2);
  }
  qv2 = fmin_f(qt, qsat);
  if (ICE) {
    qi2 = fmax_f(fice * (qt - qv2), zero);
  } else {
    qi2 = zero;
  }
  ql2 = fmax_f(qt - qv2 - qi2, zero);
  const R tbar = half * (t1 + t2);
  const R qvbar = half * (qv1 + qv2);
  const R qlbar = half * (ql1 + ql2);
  const R lhv = (R)LV1 - (R)LV2 * tbar;
  const R rm = (R)RD + (R)RV * qvbar;
  R expo;
  if (ICE) {
    const R qibar = half * (qi1 + qi2);
    const R lhs = (R)LS1 - (R)LS2 * tbar;
    const R cpm = (R)CP + (R)CPV * qvbar + (R)CPL * qlbar + (R)CPI * qibar;
    expo = lhv * (ql2 - ql1) / (cpm * tbar) + lhs * (qi2 - qi1) / (cpm * tbar) +
           (rm / cpm - (R)RDDCP) * lp;
  } else {
    const R cpm = (R)CP + (R)CPV * qvbar + (R)CPL * qlbar;
    expo = lhv * (ql2 - ql1) / (cpm * tbar) + (rm / cpm - (R)RDDCP) * lp;
  }
  return th1 * xexp(expo);
}

// What accel_map returns beside th2 when asked for the slope: dex = d expo /
// d t2 at x, and d/dt2 of qv2, ql2 and qi2 there (zero where the parcel is
// unsaturated); qsat is the saturation mixing ratio at x in every call.
struct MapSlope {
  float dex, dqv, dql, dqi, qsat;
};

// The same map for the accelerated solvers: the approximate exp and
// reciprocals of qsat_fast, the exponent over one common denominator (one
// approximate divide), and the clamps as single min/max operations (equal to
// the reference's compare-and-select for the non-NaN bounds used here).  The
// means of the two ends (tbar, qvbar, ...) enter as sums with the factors
// 1/2 folded into the constants: with tsum = t1 + t2,
//   lhv = LV1 - LV2 tbar  -> 4 lhv = 4 LV1 - 2 LV2 tsum   (and lhs alike),
//   rm = RD + RV qvbar    -> 2 rm = 2 RD + RV qvsum,
//   cpm = CP + CPV qvbar + CPL qlbar (+ CPI qibar) -> 2 cpm, likewise,
// so that the exponent's quotient
//   [lhv (ql2 - ql1) + lhs (qi2 - qi1) + rm lp tbar] / (cpm tbar)
// is [4 lhv (ql2 - ql1) + 4 lhs (qi2 - qi1) + 2 rm lp tsum] / (2 cpm tsum).
// With slope set it also returns the map's derivatives at x (MapSlope),
// differentiated through the saturation mixing ratio (dqsat_dt), the
// liquid/ice split and the exponent, for the Newton step of substep and for
// the parcel state at the Newton point.
template <bool ICE>
XC_HD float accel_map(float x, float p2, float pi2, float lp, float t1, float th1, float qv1,
                      float ql1, float qi1, float qt, bool slope, float &t2, float &qv2,
                      float &ql2, float &qi2, MapSlope &ms) {
  t2 = x * pi2;
  float fliq, fice, qsat;
  float dq = 0.0f, dql = 0.0f, dqi = 0.0f;  // d/dt2 of qv2, ql2, qi2 (slope)
  if (ICE) {
    fliq = fmaxf(fminf((t2 - 233.15f) * (1.0f / (273.15f - 233.15f)), 1.0f), 0.0f);
    fice = 1.0f - fliq;
    // both are evaluated: skipping the one of weight 0 outside the
    // 233.15-273.15 K ramp was slower (the lanes of a warp straddle it)
    QsatParts ql, qi;
    const float qvs = qsat_fast<false>(p2, t2, ql), qvi = qsat_fast<true>(p2, t2, qi);
    qsat = fliq * qvs + fice * qvi;
    if (slope && qt > qsat) {
      // saturated: qv2 = qsat, ql2 = fliq (qt - qsat), qi2 = fice (qt - qsat)
      const float dfl = (t2 > 233.15f && t2 < 273.15f) ? 1.0f / (273.15f - 233.15f) : 0.0f;
      dq = dfl * (qvs - qvi) + fliq * dqsat_dt(qvs, p2, ql, 17.67f * (273.15f - 29.65f)) +
           fice * dqsat_dt(qvi, p2, qi, 21.8745584f * (273.15f - 7.66f));
      const float c = dfl * (qt - qsat);
      dql = c - fliq * dq;
      dqi = -c - fice * dq;
    }
  } else {
    fliq = 1.0f;
    fice = 0.0f;
    QsatParts ql;
    qsat = qsat_fast<false>(p2, t2, ql);
    if (slope && qt > qsat) {
      dq = dqsat_dt(qsat, p2, ql, 17.67f * (273.15f - 29.65f));
      dql = -dq;
    }
  }
  qv2 = fmin_f(qt, qsat);  // NaN qsat (a NaN column) stays NaN, as in the reference
  if (ICE) {
    qi2 = fmaxf(fice * (qt - qv2), 0.0f);
  } else {
    qi2 = 0.0f;
  }
  ql2 = fmaxf(qt - qv2 - qi2, 0.0f);
  ms.dqv = dq;
  ms.dql = dql;
  ms.dqi = dqi;
  ms.qsat = qsat;
  const float tsum = t1 + t2;
  const float qvsum = qv1 + qv2;
  const float gl = ql2 - ql1;
  const float lhv4 = 4.0f * LV1 - 2.0f * LV2 * tsum;
  const float rm2 = 2.0f * RD + RV * qvsum;
  float cpm2 = 2.0f * CP + CPV * qvsum + CPL * (ql1 + ql2);
  if (ICE) cpm2 += CPI * (qi1 + qi2);
  float num = lhv4 * gl + rm2 * lp * tsum;
  float lhs4 = 0.0f;
  if (ICE) {
    lhs4 = 4.0f * LS1 - 2.0f * LS2 * tsum;
    num += lhs4 * (qi2 - qi1);
  }
  const float den = cpm2 * tsum;
  const float rden = fast_rcp(den);
  const float r = num * rden;
  if (slope) {
    // d r / d t2 = (num' - r den') / den, tsum' = 1
    float dnum = lhv4 * dql - 2.0f * LV2 * gl + lp * (RV * dq * tsum + rm2);
    float dcpm2 = CPV * dq + CPL * dql;
    if (ICE) {
      dnum += lhs4 * dqi - 2.0f * LS2 * (qi2 - qi1);
      dcpm2 += CPI * dqi;
    }
    ms.dex = (dnum - r * (dcpm2 * tsum + cpm2)) * rden;
  }
  return th1 * fast_exp(r - RDDCP * lp);
}

// The accelerated solvers' first Newton step x0 -> xn ends the sub-step when
// it is below NEWTON_ACCEPT: the map is smooth there, so the fixed point
// lies within F''/2 (xn - x0)^2 of xn -- under 1e-5 K for the map's
// curvature (about 0.15 / K when saturated), far inside the 2e-4 K test --
// and the parcel state at xn follows from the state and its derivatives at
// x0 (MapSlope) to second order, without a second evaluation of the map.
// Such a sub-step returns th2 = xn where the iteration returns the map's
// value at its last guess, a few ulp away; summed over a column's sub-steps
// that moves CAPE by up to 0.5 J/kg against the FP64 reference (0.17 J/kg
// without this step, 15,350 columns of 37 pressure levels, most-unstable),
// for 1.08 instead of 1.91 evaluations of the map per sub-step.
// It does not end the sub-step when the step crosses the liquid/ice ramp's
// corners (ICE) or the saturation point, where the map has a kink; nor when
// the parcel is unsaturated at x0 with its saturation mixing ratio within
// 1% of qt.  Returns whether it took the step, then with th2 = xn and the
// state (t2, qv2, ql2, qi2) at xn.
constexpr float NEWTON_ACCEPT = 0.01f;

template <bool ICE>
XC_HD bool newton_accept(float x0, float xn, float pi2, float qt, const MapSlope &ms, float &th2,
                         float &t2, float &qv2, float &ql2, float &qi2) {
  if (!(fabsf(xn - x0) <= NEWTON_ACCEPT)) return false;
  const float tn = xn * pi2, dt = tn - t2;
  if (ICE && ((t2 > 233.15f) != (tn > 233.15f) || (t2 < 273.15f) != (tn < 273.15f)))
    return false;
  if (ql2 + qi2 > 0.0f) {
    // saturated at x0, and by a margin at xn
    const float qln = ql2 + ms.dql * dt, qin = qi2 + ms.dqi * dt;
    if (!(qln + qin > 1e-3f * (ql2 + qi2))) return false;
    qv2 = qv2 + ms.dqv * dt;
    ql2 = fmaxf(qln, 0.0f);
    qi2 = fmaxf(qin, 0.0f);
  } else if (!(qt < 0.99f * ms.qsat)) {
    return false;  // unsaturated at x0, but close to saturation
  }
  t2 = tn;
  th2 = xn;
  return true;
}

// The step of F(x) - x from x with slope q (secant or Newton), q kept in
// [-50, 0.5] so that a noisy slope cannot throw x far.
XC_HD float root_step(float x, float fx, float q) {
  return x + fast_div(fx - x, 1.0f - fminf(fmaxf(q, -50.0f), 0.5f));
}

// One sub-step of the moist adiabat (:417-498).  Returns false when the
// iteration did not converge within 100 steps (:465-474).
//
// The accelerated modes (SOLVE_ACCEL, SOLVE_LEARNED) take their first step
// from the first guess x0 as a Newton step on F(x) - x, with the slope F'(x0)
// of the map differentiated analytically at the first evaluation (accel_map
// with slope).  Secant steps follow.  The stopping test is the reference's.
template <bool ICE, bool PSEUDO, int SOLVER = SOLVE_PLAIN, typename R = float>
XC_HD bool substep(R dp, R &p2, R &t2, R &th2, R &qv2, R &ql2, R &qi2, R &qt, int &niter,
                   SolverState &ss) {
  static_assert(SOLVER == SOLVE_PLAIN || sizeof(R) == sizeof(float),
                "only the plain solver runs in double precision");
  const R p1 = p2, t1 = t2, th1 = th2, qv1 = qv2, ql1 = ql2, qi1 = qi2;
  p2 = p2 - dp;
  // The accelerated modes take pi2 and ln(p2/p1) from one logarithm of p2
  // (ln p1 is the previous sub-step's), with the approximate log and exp, in
  // place of powf, a divide and logf.  The log's error (3 ulp of ln p2 at
  // most, about 3e-6) enters ln(p2/p1) only through the dry term
  // (R_m/c_pm - R_d/c_p) ln(p2/p1) of the exponent, whose prefactor is below
  // 0.02, and pi2 = exp(R_d/c_p (ln p2 - ln P00)) as a relative error of
  // about 1e-6 in t2, which the next sub-step's map does not carry forward.
  constexpr bool ACCEL_MATH = SOLVER != SOLVE_PLAIN;
  R pi2, lp;
  if constexpr (ACCEL_MATH) {
    const float l2p2 = fast_log2(p2);
    const float lnp2 = l2p2 * LN2;
    lp = lnp2 - ss.lnp;
    pi2 = fast_exp2(fmaf(RDDCP, l2p2, -RDDCP * LG2_P00));
    ss.lnp = lnp2;
  } else {
    pi2 = xpow(p2 * (R)RP00, (R)RDDCP);
    lp = xlog(p2 / p1);
  }
  R thlast = th1;
  R x_prev = XC_LIT(R, 0.0), f_prev = XC_LIT(R, 0.0);
  constexpr bool EXTRAP =
      SOLVER == SOLVE_ACCEL || SOLVER == SOLVE_LEARNED || SOLVER == SOLVE_LEARNED_WARP;
  if constexpr (EXTRAP) {
    // the first evaluation, at the extrapolated guess, also gives the map's
    // slope: a Newton step from it, then secant steps through the last two
    // evaluations (Newton again where x repeated).  The first evaluation is
    // written out apart from the loop of the later ones, which never take
    // the slope: one loop whose first pass took it issued 11% more
    // instructions per launch.
    thlast = th1 + ss.rate * dp;
    if constexpr (SOLVER == SOLVE_LEARNED_WARP) {
      if (ss.net_dth == ss.net_dth) thlast = th1 + ss.net_dth;
    }
    MapSlope ms = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    th2 = accel_map<ICE>(thlast, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, true, t2, qv2, ql2,
                         qi2, ms);
    ++niter;
    if (fabsf(th2 - thlast) > CONVERGE) {
      const float xn = root_step(thlast, th2, th2 * pi2 * ms.dex);
      if (!newton_accept<ICE>(thlast, xn, pi2, qt, ms, th2, t2, qv2, ql2, qi2)) {
        x_prev = thlast;
        f_prev = th2;
        thlast = xn;
        for (int i = 2;; ++i) {
          MapSlope unused;
          th2 = accel_map<ICE>(thlast, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, false, t2, qv2,
                               ql2, qi2, unused);
          ++niter;
          if (i > 100) return false;
          if (!(fabsf(th2 - thlast) > CONVERGE)) break;
          const float q = thlast != x_prev ? fast_div(th2 - f_prev, thlast - x_prev)
                                           : th2 * pi2 * ms.dex;
          x_prev = thlast;
          f_prev = th2;
          thlast = root_step(thlast, th2, q);
        }
      }
    }
    // a sub-step without a pressure drop (a level at the pressure of the
    // one below it, e.g. the surface exactly on a pressure level) has no
    // rate to extrapolate: 0/0 would make every later guess NaN
    if (dp != 0.0f) ss.rate = (th2 - th1) * ss.rdp;
  } else {
    if constexpr (SOLVER == SOLVE_LEARNED_ALL) {
      float dth_net;
      if (ss.saturated && network_increment(ss.guess_w, p1, p2, t1, qv1, qt, lp, dth_net))
        thlast = th1 + dth_net;
    }
    int i = 0;
    while (true) {
      i = i + 1;
      if constexpr (ACCEL_MATH) {
        MapSlope unused;
        th2 = accel_map<ICE>(thlast, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, false, t2, qv2,
                             ql2, qi2, unused);
      } else {
        th2 = plain_map<ICE>(thlast, p2, pi2, lp, t1, th1, qv1, ql1, qi1, qt, t2, qv2, ql2, qi2);
      }
      ++niter;
      if (i > 100) return false;
      if (xabs(th2 - thlast) > XC_LIT(R, 0.0002)) {
        bool secant = false;
        if constexpr (ACCEL_MATH) secant = i >= 2 && thlast != x_prev;
        if (secant) {
          if constexpr (ACCEL_MATH) {
            const float q = fast_div(th2 - f_prev, thlast - x_prev);
            x_prev = thlast;
            f_prev = th2;
            thlast = root_step(thlast, th2, q);  // secant step on F(x) - x
          }
        } else {
          const R step = th2 - thlast;
          x_prev = thlast;
          f_prev = th2;
          thlast = thlast + XC_LIT(R, 0.3) * step;
        }
      } else {
        break;
      }
    }
  }
  if constexpr (SOLVER == SOLVE_LEARNED) {
    if (ss.lcl_y == ss.lcl_y) {  // the network's output not yet taken
      if (ql2 + qi2 > 0.0f && dp != 0.0f) {
        // the parcel has just saturated: the increment extrapolated into the
        // next sub-step is the network's, not this sub-step's partial one
        ss.rate = -GUESS_SLOPE_SCALE * ss.lcl_y * fast_div(lp, dp);
        ss.lcl_y = NAN;
      }
    }
  }
  if constexpr (SOLVER == SOLVE_LEARNED_ALL || SOLVER == SOLVE_LEARNED_WARP)
    ss.saturated = ql2 + qi2 > 0.0f;
  if (PSEUDO) {  // :487-491
    qt = qv2;
    ql2 = XC_LIT(R, 0.0);
    qi2 = XC_LIT(R, 0.0);
  }
  return true;
}

// Liquid fraction of the ice adiabats' condensate at temperature t (K): the
// linear ramp between 233.15 and 273.15 K of the map (:441-444).
XC_HD float liquid_fraction(float t) {
  return fmax_f(fmin_f((t - 233.15f) / (273.15f - 233.15f), 1.0f), 0.0f);
}

// Training pair i of the guess network, over the four adiabats: the adiabat
// (pseudo/reversible x liquid/ice, uniform), a saturated parcel state with p1
// uniform in 100..1050 hPa (less the step) and T1 uniform in -80..40 degC,
// cooled in 2 K steps until its saturation mixing ratio is at most 40 g/kg
// (the warm corner of that box at low pressure holds more water than any
// atmosphere); the reversible adiabats carry 0..10 g/kg of condensate, split
// into liquid and ice by the ramp; a pressure step dp log-uniform in
// 50..2000 Pa; and the plain solver's (the reference's iteration's) solution
// of that sub-step.  Writes the features and the target y of guess_mlp.cuh
// and, when adiabat_out is set, the adiabat code; returns the iteration
// count, negative when the plain iteration gave up.
XC_HD int guess_pair(uint64_t seed, long long i, float *f, float *y, int *adiabat_out = nullptr) {
  const int adiabat = 1 + (int)fminf(3.0f, 4.0f * guess_uniform01(seed, i, 3));
  const bool ice = adiabat >= 3, pseudo = adiabat == 1 || adiabat == 3;
  const float dp = 50.0f * expf(3.6888795f * guess_uniform01(seed, i, 1));  // 50 * 40^u
  const float p1 = 10000.0f + dp + (95000.0f - dp) * guess_uniform01(seed, i, 0);
  float t1 = 193.15f + 120.0f * guess_uniform01(seed, i, 2);
  auto qsat = [&](float t) {
    if (!ice) return getqvs(p1, t);
    const float fl = liquid_fraction(t);
    return fl * getqvs(p1, t) + (1.0f - fl) * getqvi(p1, t);
  };
  float qv1 = qsat(t1);
  for (int k = 0; k < 64 && !(qv1 > 0.0f && qv1 <= 0.04f); ++k) {
    t1 -= 2.0f;
    qv1 = qsat(t1);
  }
  const float cond = pseudo ? 0.0f : 0.01f * guess_uniform01(seed, i, 4);
  const float fl = ice ? liquid_fraction(t1) : 1.0f;
  const float th1 = t1 / powf(p1 * RP00, RDDCP);
  float p2 = p1, t2 = t1, th2 = th1, qv2 = qv1, ql2 = fl * cond, qi2 = (1.0f - fl) * cond;
  float qt = qv1 + cond;
  const float qt1 = qt;
  int niter = 0;
  SolverState ss;
  bool ok;
  switch (adiabat) {
    case 1: ok = substep<false, true, SOLVE_PLAIN>(dp, p2, t2, th2, qv2, ql2, qi2, qt, niter, ss); break;
    case 2: ok = substep<false, false, SOLVE_PLAIN>(dp, p2, t2, th2, qv2, ql2, qi2, qt, niter, ss); break;
    case 3: ok = substep<true, true, SOLVE_PLAIN>(dp, p2, t2, th2, qv2, ql2, qi2, qt, niter, ss); break;
    default: ok = substep<true, false, SOLVE_PLAIN>(dp, p2, t2, th2, qv2, ql2, qi2, qt, niter, ss); break;
  }
  guess_features(p2, getthe(p1, t1, t1, qv1), qt1, f[0], f[1], f[2]);
  *y = (th2 - th1) / (GUESS_SLOPE_SCALE * logf(p1 / p2));
  if (adiabat_out) *adiabat_out = adiabat;
  return ok ? niter : -niter;
}

// Running sum with Kahan compensation (SOLVE_ACCEL) or plain FP32 addition in
// the reference's order (SOLVE_PLAIN).
template <bool COMPENSATED, typename R = float>
struct Acc {
  R s = XC_LIT(R, 0.0), c = XC_LIT(R, 0.0);
  XC_HD void add(R x) {
    if (COMPENSATED) {
      const R y = x - c;
      const R t = s + y;
      c = (t - s) - y;
      s = t;
    } else {
      s = s + x;
    }
  }
};

// getcape on one assembled column of ncl levels (surface included).
// Diagnostics that getcape computes and discards (the crossing pressure ps
// of :511 and :526, the parcel theta-e), written to dg[6] when DIAG:
//   dg[0], dg[1]  LFC pressure (hPa) and height (m): the lowest point of the
//                 first layer with positive area -- the neg->pos crossing, or
//                 the layer's base when the parcel is already buoyant there;
//   dg[2], dg[3]  EL pressure and height: the highest pos->neg crossing, or
//                 the last level reached when the parcel is still buoyant;
//   dg[4], dg[5]  height (m) and theta-e (K, getthe) of the source parcel.
// All -999999 when the parcel never has positive area (LFC/EL), when the
// ascent does not run or when the iteration gives up.
constexpr float DIAG_MISSING = -999999.f;
constexpr int DIAG_N = 6;

// The lifted parcel's source (:252-352): its level kmax, the mixed-layer
// means (FP64 accumulation, :183), the most-unstable level (mulvl,
// -999999 otherwise) and whether the ascent runs at all.
template <typename R = float>
struct SourceSelT {
  int kmax;
  int mulvl;
  R avgth, avgqv;  // the FP64 means, rounded once to R (every use is in R)
  bool ascend;
};
using SourceSel = SourceSelT<float>;

// FAST: the accelerated solvers' theta-e (getthe_fast) for the most
// unstable level and environment (make_env) in the mixed layer.
template <bool FAST, typename T, int GRID, typename R = float>
XC_HD SourceSelT<R> select_source(const ColumnReader<T, GRID, R> &col, int ncl, int source,
                                  R ml_depth) {
  static_assert(!FAST || sizeof(R) == sizeof(float), "the accelerated source selection is FP32");
  SourceSelT<R> sel;
  sel.mulvl = -999999;  // :252-253
  sel.ascend = true;
  int kmax = 1;
  double avgth = 0.0, avgqv = 0.0;

  if (source == 2) {
    // :261-281 -- argmax of theta-e over levels with p >= 500 hPa, strict >.
    const R p1 = XC_LIT(R, 100.0) * col.ps;
    if (!(p1 < XC_LIT(R, 50000.0))) {
      R maxthe = XC_LIT(R, 0.0);
      for (int j = 1; j <= ncl; ++j) {
        R pin, tin, tdin;
        col.level(j, pin, tin, tdin);
        const R p = XC_LIT(R, 100.0) * pin;
        if (p >= XC_LIT(R, 50000.0)) {
          const R t = XC_LIT(R, 273.15) + tin;
          const R td = XC_LIT(R, 273.15) + tdin;
          R q, the;
          if constexpr (FAST) {
            q = getqvs_fast(p, td);
            the = getthe_fast(p, t, td, q);
          } else {
            q = getqvs(p, td);
            the = getthe(p, t, td, q);
          }
          if (the > maxthe) {
            sel.mulvl = j;
            maxthe = the;
            kmax = j;
          }
        }
      }
    }
  } else if (source == 3) {
    // :284-339 -- mixed layer.  One upward pass evaluates the do-while
    // accumulation (:313-322) and the two guards (:287, :295), which need
    // z(2) and z(nk).
    const R half = XC_LIT(R, 0.5);
    EnvT<R> prev = col.template env<FAST>(1);
    const EnvT<R> e1 = prev;
    R zprev = XC_LIT(R, 0.0), z2 = XC_LIT(R, 0.0);
    bool active = true;
    double acc_th = 0.0, acc_qv = 0.0;
    EnvT<R> last = prev;
    for (int j = 2; j <= ncl; ++j) {
      const EnvT<R> e = col.template env_above<FAST>(j);
      const R dz = -(R)CPDG * half * (e.thv + prev.thv) * (e.pi - prev.pi);
      const R z = zprev + dz;
      if (j == 2) z2 = z;
      if (active) {
        if (z <= ml_depth) {
          acc_th = acc_th + (double)(half * (z - zprev) * (e.th + prev.th));
          acc_qv = acc_qv + (double)(half * (z - zprev) * (e.q + prev.q));
        } else {
          const R th2 = prev.th + (e.th - prev.th) * (ml_depth - zprev) / (z - zprev);
          const R qv2 = prev.q + (e.q - prev.q) * (ml_depth - zprev) / (z - zprev);
          acc_th = acc_th + (double)(half * (ml_depth - zprev) * (th2 + prev.th));
          acc_qv = acc_qv + (double)(half * (ml_depth - zprev) * (qv2 + prev.q));
          active = false;
        }
      }
      prev = e;
      zprev = z;
      last = e;
    }
    if (active) {
      // The loop ran past the top (z(nk) == ml_depth): the interpolation
      // term is multiplied by ml_depth - z(nk) == 0, th2 = th(nk).
      acc_th = acc_th + (double)(half * (ml_depth - zprev) * (last.th + last.th));
      acc_qv = acc_qv + (double)(half * (ml_depth - zprev) * (last.q + last.q));
    }
    if ((z2 - XC_LIT(R, 0.0)) > ml_depth) {
      avgth = e1.th;
      avgqv = e1.q;
      kmax = 1;
    } else if (zprev < ml_depth) {
      // Top-most level inside the mixed layer: the ascent starts at the top
      // and never runs (k < nk fails), so cape = cin = 0 and the sentinels
      // stay.
      sel.ascend = false;
    } else {
      avgth = acc_th / (double)ml_depth;
      avgqv = acc_qv / (double)ml_depth;
      kmax = 1;
    }
  }
  sel.kmax = kmax;
  sel.avgth = (R)avgth;
  sel.avgqv = (R)avgqv;
  return sel;
}

// The source parcel's state (p, t, td in Pa and K, mixing ratio q): the
// environment at kmax, or the mixed-layer means at the surface with the
// dewpoint of the mean mixing ratio.
template <bool FAST, typename T, int GRID>
XC_HD void source_parcel(const ColumnReader<T, GRID> &col, const SourceSel &sel, int source,
                         float &p, float &t, float &td, float &q) {
  const Env es = col.template env<FAST>(sel.kmax);
  p = es.p;
  if (source == 3) {
    q = sel.avgqv;
    t = sel.avgth * es.pi;
    td = dewpoint_of(es.p, q);
  } else {
    q = es.q;
    t = es.t;
    td = es.td;
  }
}

// The ascent (:355-559) from a selected source.  SOLVE_LEARNED takes the
// guess network's output at the parcel's LCL from `net_y` when guess_w is
// null (the CAPE kernel evaluates it for a whole warp on the tensor cores),
// and evaluates it here otherwise; a non-finite net_y means none.
template <bool ICE, bool PSEUDO, int SOLVER, bool DIAG, typename T, int GRID, typename R = float>
XC_HD CapeResult ascend_col(const ColumnReader<T, GRID, R> &col, int ncl, float pinc, int source,
                            const SourceSelT<R> &sel, const float *guess_w, float *dg,
                            float net_y) {
  static_assert((SOLVER == SOLVE_PLAIN && !DIAG) || sizeof(R) == sizeof(float),
                "the double-precision ascent is the plain solver's, without diagnostics");
  CapeResult r;
  float d_plfc = DIAG_MISSING, d_zlfc = DIAG_MISSING, d_pel = DIAG_MISSING,
        d_zel = DIAG_MISSING, d_zsrc = DIAG_MISSING, d_the = DIAG_MISSING;
  bool have_lfc = false, ascended = false;
  r.mulvl = sel.mulvl;
  r.z_out = -999999.f;
  r.cape = 0.0f;
  r.cin = 0.0f;
  r.status = 0;
  r.nsub = 0;
  r.niter = 0;
  const int kmax = sel.kmax;
  const R avgth = sel.avgth, avgqv = sel.avgqv;
  const R zero = XC_LIT(R, 0.0), one = XC_LIT(R, 1.0), half = XC_LIT(R, 0.5);

  // Ascent (:355-559).  Levels below kmax only integrate z.
  constexpr bool FAST = SOLVER != SOLVE_PLAIN;
  EnvT<R> prev = col.template env<FAST>(1);
  R z = zero;
  R th2 = zero, p2 = zero, t2 = zero, qv2 = zero, b2 = zero, ql2 = zero, qi2 = zero, qt = zero;
  R narea = zero;
  SolverState ss;
  ss.guess_w = guess_w;
  if constexpr (SOLVER == SOLVE_LEARNED) {
    if (guess_w) {
      // the parcel that init_parcel will start at level kmax
      float p0, t0, td0, q0;
      source_parcel<SOLVER != SOLVE_PLAIN>(col, sel, source, p0, t0, td0, q0);
      float y;
      if (parcel_lcl_slope(guess_w, p0, t0, td0, q0, y)) ss.lcl_y = y;
    } else if (net_y >= GUESS_Y_MIN && net_y <= GUESS_Y_MAX) {
      ss.lcl_y = net_y;
    }
  }
  Acc<SOLVER != SOLVE_PLAIN, R> cape_acc, cin_acc;
  auto init_parcel = [&](const EnvT<R> &e) {
    if (source == 3) {
      th2 = avgth;
      qv2 = avgqv;
      const R thv2 = th2 * (one + (R)REPS * qv2) / (one + qv2);
      p2 = e.p;
      t2 = th2 * e.pi;
      b2 = (R)G * (thv2 - e.thv) / e.thv;
    } else {
      th2 = e.th;
      p2 = e.p;
      t2 = e.t;
      qv2 = e.q;
      b2 = zero;
    }
    ql2 = zero;
    qi2 = zero;
    qt = qv2;
    if constexpr (SOLVER != SOLVE_PLAIN) ss.lnp = fast_log(p2);
  };
  auto source_diag = [&](const EnvT<R> &e) {
    if constexpr (DIAG) {
      d_zsrc = z;
      d_the = source == 3 ? getthe(p2, t2, dewpoint_of(p2, qv2), qv2) : getthe(e.p, e.t, e.td, e.q);
    }
  };
  if (kmax == 1) {
    init_parcel(prev);
    source_diag(prev);
  }
  R p_last = zero;
  const R pinc_r = (R)pinc;

  for (int k = 2; k <= ncl; ++k) {
    const EnvT<R> cur = col.template env_above<FAST>(k);
    const R dz = -(R)CPDG * half * (cur.thv + prev.thv) * (cur.pi - prev.pi);
    const R z_low = z;
    z = z + dz;
    if (k == kmax) {
      init_parcel(cur);
      source_diag(cur);
    } else if (k > kmax) {
      const R b1 = b2;
      R dp = prev.p - cur.p;
      int nloop;
      if (dp < pinc_r) {
        nloop = 1;
      } else {
        const R f = dp / pinc_r;
        if (!(f < (R)MAX_SUBSTEPS)) {
          r.cape = 0.0f;
          r.cin = 0.0f;
          r.status |= COL_TOOMANYSTEPS;
          return r;
        }
        nloop = 1 + (int)f;
        if constexpr (FAST) {
          dp = dp * fast_rcp((float)nloop);
        } else {
          dp = dp / (R)nloop;
        }
      }
      if constexpr (SOLVER != SOLVE_PLAIN) ss.rdp = fast_rcp(dp);
      if (r.nsub + nloop > MAX_SUBSTEPS) {
        r.cape = 0.0f;
        r.cin = 0.0f;
        r.status |= COL_TOOMANYSTEPS;
        return r;
      }
      // two sub-steps per pass of the loop on the device: the launch took 3%
      // less time than with one
#if defined(__CUDA_ARCH__)
#pragma unroll 2
#endif
      for (int n = 1; n <= nloop; ++n) {
        ++r.nsub;
        if (!substep<ICE, PSEUDO, SOLVER>(dp, p2, t2, th2, qv2, ql2, qi2, qt, r.niter, ss)) {
          r.cape = 0.0f;  // :471-473
          r.cin = 0.0f;
          r.status |= COL_NOCONV;
          return r;
        }
      }
      // :501-503 (FAST: approximate divides, which keep the sign of b2)
      R thv2;
      if constexpr (FAST) {
        thv2 = fast_div(th2 * (1.0f + REPS * qv2), 1.0f + qv2 + ql2 + qi2);
        b2 = fast_div(G * (thv2 - cur.thv), cur.thv);
      } else {
        thv2 = th2 * (one + (R)REPS * qv2) / (one + qv2 + ql2 + qi2);
        b2 = (R)G * (thv2 - cur.thv) / cur.thv;
      }
      if constexpr (DIAG) {
        ascended = true;
        p_last = cur.p;
        if ((b2 >= 0.0f) && (b1 < 0.0f)) {
          const float w = (0.0f - b1) / (b2 - b1);
          if (!have_lfc) {
            d_plfc = (prev.p + (cur.p - prev.p) * w) / 100.0f;
            d_zlfc = z_low + dz * w;
            have_lfc = true;
          }
        } else if ((b2 < 0.0f) && (b1 > 0.0f)) {
          const float w = (0.0f - b1) / (b2 - b1);
          if (!have_lfc) {
            d_plfc = prev.p / 100.0f;
            d_zlfc = z_low;
            have_lfc = true;
          }
          d_pel = (prev.p + (cur.p - prev.p) * w) / 100.0f;
          d_zel = z_low + dz * w;
        } else if (b2 >= 0.0f) {
          if (!have_lfc) {
            d_plfc = prev.p / 100.0f;
            d_zlfc = z_low;
            have_lfc = true;
          }
        }
      }
      // :509-547
      R parea;
      if ((b2 >= zero) && (b1 < zero)) {
        const R frac = b2 / (b2 - b1);
        parea = half * b2 * dz * frac;
        narea = narea - half * b1 * dz * (one - frac);
        cin_acc.add(narea);
        narea = zero;
      } else if ((b2 < zero) && (b1 > zero)) {
        const R frac = b1 / (b1 - b2);
        parea = half * b1 * dz * frac;
        narea = -half * b2 * dz * (one - frac);
      } else if (b2 < zero) {
        parea = zero;
        narea = narea - half * dz * (b1 + b2);
      } else {
        parea = half * dz * (b1 + b2);
        narea = zero;
      }
      cape_acc.add(fmax_f(zero, parea));
      r.z_out = (float)z;
      // :554-557
      if ((cur.p <= XC_LIT(R, 10000.0)) && (b2 < zero)) break;
    }
    prev = cur;
  }
  r.cape = (float)cape_acc.s;
  r.cin = (float)cin_acc.s;
  if constexpr (DIAG) {
   if (ascended) {
    if (have_lfc && b2 >= 0.0f) {
      d_pel = p_last / 100.0f;
      d_zel = r.z_out;
    }
    dg[0] = have_lfc ? d_plfc : DIAG_MISSING;
    dg[1] = have_lfc ? d_zlfc : DIAG_MISSING;
    dg[2] = have_lfc ? d_pel : DIAG_MISSING;
    dg[3] = have_lfc ? d_zel : DIAG_MISSING;
    dg[4] = d_zsrc;
    dg[5] = d_the;
   }
  }
  return r;
}

template <bool ICE, bool PSEUDO, int SOLVER, bool DIAG, typename T, int GRID, typename R = float>
XC_HD CapeResult getcape_col(const ColumnReader<T, GRID, R> &col, int ncl, float pinc,
                                  int source, float ml_depth, const float *guess_w = nullptr,
                                  float *dg = nullptr) {
  const SourceSelT<R> sel = select_source<SOLVER != SOLVE_PLAIN>(col, ncl, source, (R)ml_depth);
  if (!sel.ascend) {
    CapeResult r;
    r.mulvl = sel.mulvl;
    r.z_out = -999999.f;
    r.cape = 0.0f;
    r.cin = 0.0f;
    r.status = 0;
    r.nsub = 0;
    r.niter = 0;
    return r;
  }
  return ascend_col<ICE, PSEUDO, SOLVER, DIAG>(col, ncl, pinc, source, sel, guess_w, dg, 0.0f);
}


// One column of loopcape_ml / loopcape_pl1d / loopcape_pl
// (CAPE_CODE_model_lev.f90:76-89, CAPE_CODE_pressure_lev.f90:66-82, 151-167):
// the ts > 0 gate, the start level, getcape, and the outputs of column i.
template <typename T, int GRID, bool ICE, bool PSEUDO, int SOLVER = SOLVE_PLAIN,
          bool DIAG = false, typename R = float>
XC_HD void cape_column_run(const CapeArgs &a, long long i, int &nsub, int &niter,
                           const float *guess_w = nullptr) {
    float dg[DIAG_N];
    if (DIAG)
      for (int d = 0; d < DIAG_N; ++d) dg[d] = DIAG_MISSING;
    const long long stride = a.ld > 0 ? a.ld : a.nk;
    const R ts = (R)ld((const T *)a.ts + i);
    float cape = 0.0f, cin = 0.0f, zo = 0.0f;
    int mulvl = 0, status = 0;
    int start = 1;
    if (GRID != 1) {
      if (a.start) {
        start = ld(a.start + i);
      } else {
        start = pres_lev_pos_col<T>((const T *)a.p, ld((const T *)a.ps + i), a.nk);
      }
    }
    if (ts > XC_LIT(R, 0.0)) {  // CAPE_CODE_model_lev.f90:77
      if (start < 1 || start > a.nk) {
        status = COL_BADSTART;
      } else {
        ColumnReader<T, GRID, R> col;
        col.set((const T *)a.p, (const T *)a.t, (const T *)a.td, i * stride, start);
        col.ps = (R)ld((const T *)a.ps + i);
        col.ts = ts;
        col.tds = (R)ld((const T *)a.tds + i);
        const int ncl = a.nk - start + 2;
        CapeResult r =
            getcape_col<ICE, PSEUDO, SOLVER, DIAG>(col, ncl, a.pinc, a.source, a.ml_depth, guess_w,
                                                   dg);
        cape = r.cape;
        cin = r.cin;
        zo = r.z_out;
        mulvl = r.mulvl;
        status = r.status;
        nsub = r.nsub;
        niter = r.niter;
      }
    }
    a.cape[i] = cape;
    a.cin[i] = cin;
    a.mulvl[i] = mulvl;
    a.z_out[i] = zo;
    if (a.status) a.status[i] = status;
    if (DIAG)
      for (int d = 0; d < DIAG_N; ++d) a.diag[DIAG_N * i + d] = dg[d];
}

}  // namespace xc
