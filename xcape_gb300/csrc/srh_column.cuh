// srh_column.cuh -- storm-relative helicity on one column, compiled for the
// device (srh_kernel.cu) and for the host (the CPU emulation harness).
//
// The reference computes SRH with three f2py calls that each materialise an
// (nlev, ncol) array on the host (src/xcape/core.py:516-542):
//   loop_stdheight_*  (stdheight_2D_model_lev.f90:74-160, FP64)
//   bunkers_loop_*    (Bunkers_model_lev.f90:4-236, FP32)
//   loop_sreh_*       (SREH_model_lev.f90:4-129, FP64)
// srh_column_run does the same work for one column:
//   pass 1 walks the levels upward once, integrating the hypsometric height
//          (FP64, as stdheight_ml), locating the 12 Bunkers target heights
//          (FP32, as DINTERP2DZ on the f2py-rounded heights) and the SREH top
//          level (FP64, as DCALRELHL);
//   pass 2 re-reads u, v up to the SREH top level and forms the two helicity
//          sums in the reference's order.
// DINTERP2DZ scans each column from the top and keeps the first bracket it
// finds; pass 1 scans upward and lets every later bracket overwrite the
// earlier one, which selects the same (highest) bracket.  The scan direction
// rule (Bunkers_model_lev.f90:210-215) depends on the top height, known only
// after pass 1; the rare decreasing-height column is redone with the other
// rule.
#pragma once
#include <math.h>

#include "xc_common.cuh"
#include "xc_kernels.h"

namespace xc {

// stdheight constants: DOUBLE PRECISION variables initialised from
// default-REAL literals (stdheight_2D_model_lev.f90:90-93, 102-106).
constexpr double SH_R = (double)287.04f;
constexpr double SH_G = (double)-9.80665f;
constexpr double SH_EPS = (double)0.6219800858985514f;
constexpr double SH_T0 = (double)273.15f;
constexpr double SH_C6112 = (double)6.112f;
constexpr double SH_C5349 = (double)53.49f;
constexpr double SH_C509 = (double)5.09f;
constexpr float VMSG = -999999.f;

// A product that feeds an addition, rounded on its own as the reference's
// compiled code rounds it: the device build never fuses it into a
// multiply-add, whatever the -fmad setting of the translation unit that
// inlines this file, so every kernel that runs these routines (the SRH
// kernels, the fused CAPE + SRH kernel) gives the same bits.
XC_HD float nc_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
XC_HD double nc_mul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

// Virtual temperature of one level (stdheight_2D_model_lev.f90:102-111,
// 116-131); P in hPa, T/Td in degC.
XC_HD double stdh_tv(double P, double T, double Td) {
  const double Tin = T + SH_T0;
  const double Tdin = Td + SH_T0;
  const double E = nc_mul(SH_C6112, exp((SH_C5349 - (6808.0 / Tdin) - nc_mul(SH_C509, log(Tdin)))));
  const double w = nc_mul(SH_EPS, (E / (P - E)));
  return nc_mul(Tin, ((w + SH_EPS) / (SH_EPS * (1.0 + w))));
}

// Hypsometric step (:147, :155).
XC_HD double stdh_step(double Hprev, double Tv, double Tvprev, double P, double Pprev) {
  return Hprev + nc_mul((SH_R * ((Tv + Tvprev) / 2.0) / SH_G), (log(P / Pprev)));
}

// FP32 forms of the two stdheight formulas, for the FP32 SRH path (the
// height is then accumulated with Kahan compensation, see srh_pass1).  Its
// contract is agreement with FP64 within tolerance, so they use the
// approximate exp, log and divides (exact on the host).
XC_HD float stdh_tv_f(float P, float T, float Td) {
  const float eps = 0.6219800858985514f;
  const float Tin = T + 273.15f;
  const float Tdin = Td + 273.15f;
  const float E =
      nc_mul(6.112f, fast_exp((53.49f - fast_div(6808.0f, Tdin) - nc_mul(5.09f, fast_log(Tdin)))));
  const float w = nc_mul(eps, fast_div(E, P - E));
  return nc_mul(Tin, fast_div(w + eps, eps * (1.0f + w)));
}
XC_HD float stdh_dh_f(float Tv, float Tvprev, float P, float Pprev) {
  return nc_mul(fast_div(287.04f * ((Tv + Tvprev) / 2.0f), -9.80665f), fast_log(fast_div(P, Pprev)));
}

// Real type of the stdheight / SREH stages: double as in the reference, or
// float for the FP32 path.
template <bool F32> struct SrhReal { typedef double type; };
template <> struct SrhReal<true> { typedef float type; };

// Kahan-compensated running sum in R (plain addition for double, where the
// reference's own order is kept).
template <typename R>
struct KSum {
  R s, c;
  XC_HD explicit KSum(R init) : s(init), c(0) {}
  XC_HD void add(R x) {
    if (sizeof(R) == 4) {
      const R y = x - c;
      const R t = s + y;
      c = (t - s) - y;
      s = t;
    } else {
      s = s + x;
    }
  }
};

// DINTERP2DZ (Bunkers_model_lev.f90:188-236) folded into an upward sweep:
// the level pair (KP-1, KP) = (lo, hi) matches target h when
// Z(KP-IM) <= h < Z(KP-IP).  Every match overwrites (highest KP wins).
template <bool DEC>
XC_HD void bunkers_bracket(float zlo, float zhi, float ulo, float uhi, float vlo, float vhi,
                           float *u6, float *v6) {
  // (za, ua) is level KP-IM and (zb, ub) level KP-IP.
  const float za = DEC ? zhi : zlo, zb = DEC ? zlo : zhi;
  const float ua = DEC ? uhi : ulo, ub = DEC ? ulo : uhi;
  const float va = DEC ? vhi : vlo, vb = DEC ? vlo : vhi;
  if (!(za < zb)) return;  // no h with za <= h < zb (NaN included)
  float c = ceilf(za * (1.0f / 500.0f));
  c = fminf(fmaxf(c, 0.0f), 13.0f);
  int i0 = (int)c - 1;
  if (i0 < 0) i0 = 0;
  while (i0 > 0 && 500.0f * (float)i0 >= za) --i0;
  while (i0 < 12 && 500.0f * (float)(i0 + 1) < za) ++i0;
  for (int i = i0; i < 12; ++i) {
    const float h = nc_mul(500.0f, (float)(i + 1));
    if (!(zb > h)) break;
    if (za <= h) {
      const float w2 = (h - za) / (zb - za);
      const float w1 = (float)(1.0 - (double)w2);  // W1 = 1.D0 - W2
      u6[i] = nc_mul(w1, ua) + nc_mul(w2, ub);
      v6[i] = nc_mul(w1, va) + nc_mul(w2, vb);
    }
  }
}

// bunkers_calc_ml tail (:123-177) from the surface point and the 12
// interpolated points.  Mean6kmwind starts at zero (f2py zero-fills
// intent(out)); the shear accumulators, never initialised in the Fortran,
// start at zero.
XC_HD void bunkers_finish(float u1, float v1, const float *u6, const float *v6, float *rm,
                          float *lm, float *mean) {
  float m0 = 0.0f + u1, m1 = 0.0f + v1;
  for (int i = 0; i < 12; ++i) {
    m0 = m0 + u6[i];
    m1 = m1 + v6[i];
  }
  m0 = m0 / 13.0f;
  m1 = m1 / 13.0f;
  const float ushr_u = ((0.0f + u6[10]) + u6[11]) / 2.0f;
  const float vshr_u = ((0.0f + v6[10]) + v6[11]) / 2.0f;
  const float ushr_d = ((0.0f + u1) + u6[0]) / 2.0f;
  const float vshr_d = ((0.0f + v1) + v6[0]) / 2.0f;
  const float ushr = ushr_u - ushr_d;
  const float vshr = vshr_u - vshr_d;
  const float nrm = sqrtf(nc_mul(ushr, ushr) + nc_mul(vshr, vshr));
  rm[0] = m0 + 7.5f * vshr / nrm;
  rm[1] = m1 - 7.5f * ushr / nrm;
  lm[0] = m0 - 7.5f * vshr / nrm;
  lm[1] = m1 + 7.5f * ushr / nrm;
  mean[0] = m0;
  mean[1] = m1;
}

template <typename T>
struct SrhColumn {
  const T *p, *t, *td, *u, *v;  // p: this column (grid 1) or the shared axis (grid 2)
  double ps, ts, tds, us, vs;
  int base;  // start - 3: the 0-based input index of assembled level j is base + j
};

// Level reader of the column path: the input arrays of one column, the
// virtual temperature computed from p, t, td as the level is reached.
template <bool F32, typename T>
struct GlobalLevels {
  typedef typename SrhReal<F32>::type R;
  const SrhColumn<T> *c;
  XC_HD R p(int m) const { return F32 ? (R)ldf(c->p + m) : (R)ldd(c->p + m); }
  XC_HD R tv(int m, R P) const {
    return F32 ? (R)stdh_tv_f((float)P, ldf(c->t + m), ldf(c->td + m))
               : (R)stdh_tv((double)P, ldd(c->t + m), ldd(c->td + m));
  }
  XC_HD R u(int m) const { return F32 ? (R)ldf(c->u + m) : (R)ldd(c->u + m); }
  XC_HD R v(int m) const { return F32 ? (R)ldf(c->v + m) : (R)ldd(c->v + m); }
};

// Surface values and level window of one column.
struct SrhSurface {
  double ps, ts, tds, us, vs;
  int base;  // start - 3: the 0-based input index of assembled level j is base + j
};

struct SrhPass1 {
  int ktop;
  double utop, vtop;  // interpolated winds at `depth` (level ktop)
  float ztop_f;       // f2py-rounded height of the top level (Z(NZ))
};

// Pass 1 (see the file comment) as a sweep that takes levels 2..ncl in
// order, one step per level: the hypsometric height (FP64, or FP32 with
// Kahan compensation when F32), the 12 Bunkers targets (DEC selects the
// scan rule) and the SREH top level.  srh_pass1 feeds it the levels through
// a reader (GlobalLevels).
template <bool DEC, bool F32>
struct SrhSweep {
  typedef typename SrhReal<F32>::type R;
  SrhPass1 r;
  R Pprev, Hprev, Tvprev, udprev, vdprev, rdepth;
  KSum<R> Hsum;
  float zprev, uprev, vprev;

  XC_HD SrhSweep(const SrhSurface &c, double depth, double aglh0) : Hsum((R)aglh0) {
    r.ktop = 0;
    r.utop = 0.0;
    r.vtop = 0.0;
    r.ztop_f = (float)aglh0;
    Pprev = (R)c.ps;
    Hprev = (R)aglh0;
    Tvprev = F32 ? (R)stdh_tv_f((float)c.ps, (float)c.ts, (float)c.tds)
                 : (R)stdh_tv(c.ps, c.ts, c.tds);
    rdepth = (R)depth;
    zprev = (float)aglh0;
    uprev = (float)c.us;
    vprev = (float)c.vs;
    udprev = (R)c.us;
    vdprev = (R)c.vs;
  }
  // level j: pressure P, virtual temperature Tv, winds ud, vd
  XC_HD void step(int j, R P, R Tv, R ud, R vd, float *u6, float *v6) {
    R H;
    if (F32) {
      Hsum.add((R)stdh_dh_f((float)Tv, (float)Tvprev, (float)P, (float)Pprev));
      H = Hsum.s;
    } else {
      H = (R)stdh_step((double)Hprev, (double)Tv, (double)Tvprev, (double)P, (double)Pprev);
    }
    const float zf = (float)H, uf = (float)ud, vf = (float)vd;
    bunkers_bracket<DEC>(zprev, zf, uprev, uf, vprev, vf, u6, v6);
    if (r.ktop == 0 && H > rdepth) {
      // DCALRELHL :85-95 with INTERP1 (SREH_model_lev.f90:123-129), whose
      // X1 argument is aglh(ktop) passed by reference.
      r.ktop = j;
      R x1 = H;
      const R x3 = Hprev;
      if (x3 == x1) x1 = x1 - (R)0.01f;
      r.utop = (double)(ud + nc_mul((udprev - ud), ((rdepth - x1) / (x3 - x1))));
      if (x3 == x1) x1 = x1 - (R)0.01f;
      r.vtop = (double)(vd + nc_mul((vdprev - vd), ((rdepth - x1) / (x3 - x1))));
    }
    Pprev = P;
    Hprev = H;
    Tvprev = Tv;
    zprev = zf;
    uprev = uf;
    vprev = vf;
    udprev = ud;
    vdprev = vd;
  }
  XC_HD SrhPass1 finish() {
    r.ztop_f = zprev;
    return r;
  }
};

// Pass 1 over levels 2..ncl read through `lv`.
template <bool DEC, bool F32, typename LV>
XC_HD SrhPass1 srh_pass1(const LV &lv, const SrhSurface &c, int ncl, double depth, double aglh0,
                         float *u6, float *v6) {
  typedef typename SrhReal<F32>::type R;
  SrhSweep<DEC, F32> sw(c, depth, aglh0);
  for (int j = 2; j <= ncl; ++j) {
    const int m = c.base + j;
    const R P = lv.p(m);
    const R Tv = lv.tv(m, P);
    sw.step(j, P, Tv, lv.u(m), lv.v(m), u6, v6);
  }
  return sw.finish();
}

// Pass 2 (DCALRELHL :100-114) as a sweep over levels 2..ktop in order: the
// helicity sums for the right- and left-moving storm motions.
template <bool F32>
struct SrhSums {
  typedef typename SrhReal<F32>::type R;
  R cu_rm, cv_rm, cu_lm, cv_lm, uprev, vprev;
  KSum<R> s_rm, s_lm;
  XC_HD SrhSums(const float *rm, const float *lm, const SrhSurface &c)
      : cu_rm(rm[0]), cv_rm(rm[1]), cu_lm(lm[0]), cv_lm(lm[1]), uprev((R)c.us),
        vprev((R)c.vs), s_rm((R)0), s_lm((R)0) {}
  XC_HD void step(R uk, R vk) {
    s_rm.add(nc_mul((uk - cu_rm), (vk - vprev)) - nc_mul((vk - cv_rm), (uk - uprev)));
    s_lm.add(nc_mul((uk - cu_lm), (vk - vprev)) - nc_mul((vk - cv_lm), (uk - uprev)));
    uprev = uk;
    vprev = vk;
  }
};

// The Bunkers vectors of column i (when requested) and its helicities.
XC_HD void srh_write(const SrhArgs &a, long long i, const float *rm, const float *lm,
                     const float *mean, double srh_rm, double srh_lm) {
  if (a.rm) {
    a.rm[2 * i] = rm[0];
    a.rm[2 * i + 1] = rm[1];
    a.lm[2 * i] = lm[0];
    a.lm[2 * i + 1] = lm[1];
    a.mean6[2 * i] = mean[0];
    a.mean6[2 * i + 1] = mean[1];
  }
  a.srh_rm[i] = srh_rm;
  a.srh_lm[i] = srh_lm;
}

// Passes 1 and 2 of column i (levels through `lv`), and its outputs.
template <bool F32, typename LV>
XC_HD void srh_column_body(const SrhArgs &a, long long i, const LV &lv, const SrhSurface &c,
                           int ncl) {
  typedef typename SrhReal<F32>::type R;
  float u6[12], v6[12];
  for (int k = 0; k < 12; ++k) {
    u6[k] = VMSG;
    v6[k] = VMSG;
  }
  SrhPass1 r = srh_pass1<false, F32>(lv, c, ncl, a.depth, a.aglh0, u6, v6);
  if ((float)a.aglh0 > r.ztop_f) {
    // Z(1) > Z(NZ): DINTERP2DZ switches to the decreasing-height rule.
    for (int k = 0; k < 12; ++k) {
      u6[k] = VMSG;
      v6[k] = VMSG;
    }
    r = srh_pass1<true, F32>(lv, c, ncl, a.depth, a.aglh0, u6, v6);
  }
  float rm[2], lm[2], mean[2];
  bunkers_finish((float)c.us, (float)c.vs, u6, v6, rm, lm, mean);
  SrhSums<F32> sums(rm, lm, c);
  for (int k = 2; k <= r.ktop; ++k) {
    if (k == r.ktop) sums.step((R)r.utop, (R)r.vtop);
    else sums.step(lv.u(c.base + k), lv.v(c.base + k));
  }
  srh_write(a, i, rm, lm, mean, -(double)sums.s_rm.s, -(double)sums.s_lm.s);
}

// Column i of the fused SRH path (core.py:_calc_srh_numpy :473-542).
// F32 = false follows the reference's precisions (FP64 stdheight and SREH,
// FP32 Bunkers); F32 = true runs the stdheight and SREH stages in FP32 with
// compensated sums.
template <typename T, int GRID, bool F32 = false>
XC_HD void srh_column_run(const SrhArgs &a, long long i) {
  SrhColumn<T> c;
  c.p = GRID == 2 ? (const T *)a.p : (const T *)a.p + i * a.nk;
  c.t = (const T *)a.t + i * a.nk;
  c.td = (const T *)a.td + i * a.nk;
  c.u = (const T *)a.u + i * a.nk;
  c.v = (const T *)a.v + i * a.nk;
  c.ps = ldd((const T *)a.ps + i);
  c.ts = ldd((const T *)a.ts + i);
  c.tds = ldd((const T *)a.tds + i);
  c.us = ldd((const T *)a.us + i);
  c.vs = ldd((const T *)a.vs + i);
  int st = 1;
  if (GRID == 2) {
    st = a.start ? ld(a.start + i) : pres_lev_pos_col<T>((const T *)a.p, ld((const T *)a.ps + i), a.nk);
    st = st < 1 ? 1 : (st > a.nk + 1 ? a.nk + 1 : st);
  }
  c.base = st - 3;
  const int ncl = a.nk - st + 2;
  SrhSurface sf;
  sf.ps = c.ps;
  sf.ts = c.ts;
  sf.tds = c.tds;
  sf.us = c.us;
  sf.vs = c.vs;
  sf.base = c.base;
  GlobalLevels<F32, T> lv;
  lv.c = &c;
  srh_column_body<F32>(a, i, lv, sf, ncl);
}

// ---- stage columns -----------------------------------------------------------

XC_HD int clamp_start(const int *start, long long i, int nk) {
  int st = start ? ld(start + i) : 1;
  return st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
}

// loop_stdheight_ml / _pl1d / _pl (stdheight_2D_model_lev.f90:29-32,
// stdheight_2D_pressure_lev.f90:33-45, 79-91); p_stride 0 = shared p.
XC_HD void stdheight_column_run(const double *P, long long p_stride, const double *T,
                                const double *Td, const double *Ps, const double *Ts,
                                const double *Tds, const double *Hin, const int *start, int NK,
                                long long i, double *H, double *Hs) {
  const int st = clamp_start(start, i, NK);
  double *Hc = H + i * NK;
  for (int k = 1; k < st; ++k) Hc[k - 1] = -999999.0;
  const double *Pc = P + i * p_stride;
  const double *Tc = T + i * NK;
  const double *Tdc = Td + i * NK;
  const double ps = Ps[i];
  double Hprev = Hin[i];
  Hs[i] = Hprev;
  double Tvprev = stdh_tv(ps, Ts[i], Tds[i]);
  double Pprev = ps;
  for (int k = st; k <= NK; ++k) {
    const double Pk = Pc[k - 1];
    const double Tv = stdh_tv(Pk, Tc[k - 1], Tdc[k - 1]);
    const double Hk = stdh_step(Hprev, Tv, Tvprev, Pk, Pprev);
    Hc[k - 1] = Hk;
    Hprev = Hk;
    Tvprev = Tv;
    Pprev = Pk;
  }
}

// DINTERP2DZ exactly as written (a top-down scan) on an assembled column:
// index 1 is the surface (zs, vs), index k >= 2 is Z[k-2].
XC_HD float dinterp2dz_col(const float *V, const float *Z, float vs, float zs, int nz, float loc) {
  int ip = 0, im = 1;
  const float ztop = nz == 1 ? zs : Z[nz - 2];
  if (zs > ztop) {
    ip = 1;
    im = 0;
  }
  for (int kp = nz; kp >= 2; --kp) {
    const int ka = kp - im, kb = kp - ip;
    const float za = ka == 1 ? zs : Z[ka - 2], zb = kb == 1 ? zs : Z[kb - 2];
    if ((za <= loc) && (zb > loc)) {
      const float w2 = (loc - za) / (zb - za);
      const float w1 = (float)(1.0 - (double)w2);
      const float va = ka == 1 ? vs : V[ka - 2], vb = kb == 1 ? vs : V[kb - 2];
      return nc_mul(w1, va) + nc_mul(w2, vb);
    }
  }
  return VMSG;
}

// bunkers_loop_ml / _pl (Bunkers_model_lev.f90:58-67, Bunkers_pressure_lev.f90:59-77).
XC_HD void bunkers_column_run(const float *U, const float *V, const float *Z, const float *Us,
                              const float *Vs, const float *Zs, const int *start, int nk,
                              long long i, float *RM, float *LM, float *Mean) {
  const int st = clamp_start(start, i, nk);
  const int nz = nk - st + 2;
  const float *Uc = U + i * nk + st - 1, *Vc = V + i * nk + st - 1, *Zc = Z + i * nk + st - 1;
  float u6[12], v6[12];
  for (int k = 0; k < 12; ++k) {
    const float h = nc_mul(500.0f, (float)(k + 1));
    u6[k] = dinterp2dz_col(Uc, Zc, Us[i], Zs[i], nz, h);
    v6[k] = dinterp2dz_col(Vc, Zc, Vs[i], Zs[i], nz, h);
  }
  bunkers_finish(Us[i], Vs[i], u6, v6, RM + 2 * i, LM + 2 * i, Mean + 2 * i);
}

// loop_sreh_ml / _pl (SREH_model_lev.f90:42-53, SREH_pressure_lev.f90:43-60)
// with DCALRELHL (:61-118) as written.
XC_HD void sreh_column_run(const double *u, const double *v, const double *aglh,
                           const double *us, const double *vs, const double *aglhs,
                           const double *cu_rm, const double *cv_rm, const double *cu_lm,
                           const double *cv_lm, double top, const int *start, int nk,
                           long long i, double *sreh_rm, double *sreh_lm) {
  const int st = clamp_start(start, i, nk);
  const int nka = nk - st + 2;
  const double *uc = u + i * nk + st - 1, *vc = v + i * nk + st - 1, *hc = aglh + i * nk + st - 1;
  int ktop = 0;
  double ut = 0.0, vt = 0.0;
  for (int k = 2; k <= nka; ++k) {
    const double hk = hc[k - 2];
    if (hk > top) {
      ktop = k;
      double x1 = hk;
      const double x3 = k == 2 ? aglhs[i] : hc[k - 3];
      const double uk = uc[k - 2], vk = vc[k - 2];
      const double up = k == 2 ? us[i] : uc[k - 3], vp = k == 2 ? vs[i] : vc[k - 3];
      if (x3 == x1) x1 = x1 - (double)0.01f;
      ut = uk + nc_mul((up - uk), ((top - x1) / (x3 - x1)));
      if (x3 == x1) x1 = x1 - (double)0.01f;
      vt = vk + nc_mul((vp - vk), ((top - x1) / (x3 - x1)));
      break;
    }
  }
  double s1 = 0.0, s2 = 0.0;
  double up = us[i], vp = vs[i];
  for (int k = 2; k <= ktop; ++k) {
    const double uk = k == ktop ? ut : uc[k - 2], vk = k == ktop ? vt : vc[k - 2];
    s1 = s1 + (nc_mul((uk - cu_rm[i]), (vk - vp)) - nc_mul((vk - cv_rm[i]), (uk - up)));
    s2 = s2 + (nc_mul((uk - cu_lm[i]), (vk - vp)) - nc_mul((vk - cv_lm[i]), (uk - up)));
    up = uk;
    vp = vk;
  }
  sreh_rm[i] = -s1;
  sreh_lm[i] = -s2;
}

}  // namespace xc
