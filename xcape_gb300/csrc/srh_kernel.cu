// srh_kernel.cu -- storm-relative helicity for sm_103a.
//
// The reference computes SRH with three f2py calls that each materialise an
// (nlev, ncol) array on the host (src/xcape/core.py:516-542):
//   loop_stdheight_*  (stdheight_2D_model_lev.f90:74-160, FP64)
//   bunkers_loop_*    (Bunkers_model_lev.f90:4-236, FP32)
//   loop_sreh_*       (SREH_model_lev.f90:4-129, FP64)
// srh_fused_kernel does the same work in one thread per column:
//   pass 1 walks the levels upward once, integrating the hypsometric height
//          (FP64, as stdheight_ml), locating the 12 Bunkers target heights
//          (FP32, as DINTERP2DZ on the f2py-rounded heights) and the SREH top
//          level (FP64, as DCALRELHL);
//   pass 2 re-reads u, v up to the SREH top level and forms the two helicity
//          sums in the reference's order.
// DINTERP2DZ scans each column from the top and keeps the first bracket it
// finds; pass 1 scans upward and lets every later bracket overwrite the
// earlier one, which selects the same (highest) bracket.  The scan direction
// rule (:212-215) depends on the top height, known only after pass 1; the
// rare decreasing-height column is redone with the other rule.
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

// Virtual temperature of one level (stdheight_2D_model_lev.f90:102-111,
// 116-131); P in hPa, T/Td in degC.
__device__ __forceinline__ double stdh_tv(double P, double T, double Td) {
  const double Tin = T + SH_T0;
  const double Tdin = Td + SH_T0;
  const double E = SH_C6112 * exp((SH_C5349 - (6808.0 / Tdin) - SH_C509 * log(Tdin)));
  const double w = SH_EPS * (E / (P - E));
  return Tin * ((w + SH_EPS) / (SH_EPS * (1.0 + w)));
}

// Hypsometric step (:147, :155).
__device__ __forceinline__ double stdh_step(double Hprev, double Tv, double Tvprev, double P,
                                            double Pprev) {
  return Hprev + ((SH_R * ((Tv + Tvprev) / 2.0) / SH_G)) * (log(P / Pprev));
}

// DINTERP2DZ (Bunkers_model_lev.f90:188-236) folded into an upward sweep:
// the level pair (KP-1, KP) = (lo, hi) matches target h when
// Z(KP-IM) <= h < Z(KP-IP).  Every match overwrites (highest KP wins).
template <bool DEC>
__device__ __forceinline__ void bunkers_bracket(float zlo, float zhi, float ulo, float uhi,
                                                float vlo, float vhi, float *u6, float *v6) {
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
    const float h = 500.0f * (float)(i + 1);
    if (!(zb > h)) break;
    if (za <= h) {
      const float w2 = (h - za) / (zb - za);
      const float w1 = (float)(1.0 - (double)w2);  // W1 = 1.D0 - W2
      u6[i] = w1 * ua + w2 * ub;
      v6[i] = w1 * va + w2 * vb;
    }
  }
}

// bunkers_calc_ml tail (:123-177) from the 12 interpolated points and the
// surface point.  Mean6kmwind starts at zero (f2py zero-fills intent(out));
// the shear accumulators, never initialised in the Fortran, start at zero.
__device__ __forceinline__ void bunkers_finish(float u1, float v1, const float *u6,
                                               const float *v6, float *rm, float *lm,
                                               float *mean) {
  float m0 = 0.0f + u1, m1 = 0.0f + v1;
#pragma unroll
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
  const float nrm = sqrtf(ushr * ushr + vshr * vshr);
  rm[0] = m0 + 7.5f * vshr / nrm;
  rm[1] = m1 - 7.5f * ushr / nrm;
  lm[0] = m0 - 7.5f * vshr / nrm;
  lm[1] = m1 + 7.5f * ushr / nrm;
  mean[0] = m0;
  mean[1] = m1;
}

template <typename T, int GRID>
struct SrhColumn {
  const T *p, *t, *td, *u, *v;  // p: this column (GRID 1) or shared (GRID 2)
  double ps, ts, tds, us, vs;
  int base;  // start - 2: input index of assembled level j is base + j
};

struct SrhPass1 {
  int ktop;
  double utop, vtop;  // interpolated winds at `depth` (level ktop)
  float ztop_f;       // f2py-rounded height of the top level (Z(NZ))
};

// Pass 1 over levels 2..ncl (see file comment).
template <bool DEC, typename T, int GRID>
__device__ SrhPass1 srh_pass1(const SrhColumn<T, GRID> &c, int ncl, double depth, double aglh0,
                              float *u6, float *v6) {
  SrhPass1 r;
  r.ktop = 0;
  r.utop = 0.0;
  r.vtop = 0.0;
  double Pprev = c.ps;
  double Hprev = aglh0;
  double Tvprev = stdh_tv(c.ps, c.ts, c.tds);
  float zprev = (float)aglh0, uprev = (float)c.us, vprev = (float)c.vs;
  double udprev = c.us, vdprev = c.vs;
  for (int j = 2; j <= ncl; ++j) {
    const int m = c.base + j;
    const double P = ldd(c.p + m);
    const double Tv = stdh_tv(P, ldd(c.t + m), ldd(c.td + m));
    const double H = stdh_step(Hprev, Tv, Tvprev, P, Pprev);
    const double ud = ldd(c.u + m), vd = ldd(c.v + m);
    const float zf = (float)H, uf = (float)ud, vf = (float)vd;
    bunkers_bracket<DEC>(zprev, zf, uprev, uf, vprev, vf, u6, v6);
    if (r.ktop == 0 && H > depth) {
      // DCALRELHL :85-95 with INTERP1 (SREH_model_lev.f90:123-129), whose
      // X1 argument is aglh(ktop) by reference.
      r.ktop = j;
      double x1 = H;
      const double x3 = Hprev;
      if (x3 == x1) x1 = x1 - (double)0.01f;
      r.utop = ud + ((udprev - ud) * ((depth - x1) / (x3 - x1)));
      if (x3 == x1) x1 = x1 - (double)0.01f;
      r.vtop = vd + ((vdprev - vd) * ((depth - x1) / (x3 - x1)));
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
  r.ztop_f = zprev;
  return r;
}

template <typename T, int GRID>
__global__ void __launch_bounds__(128) srh_fused_kernel(SrhArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.n2) return;
  SrhColumn<T, GRID> c;
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
    st = a.start ? __ldg(a.start + i)
                 : pres_lev_pos_col<T>((const T *)a.p, __ldg((const T *)a.ps + i), a.nk);
    st = st < 1 ? 1 : (st > a.nk + 1 ? a.nk + 1 : st);
  }
  c.base = st - 2;
  const int ncl = a.nk - st + 2;

  float u6[12], v6[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    u6[k] = -999999.f;
    v6[k] = -999999.f;
  }
  SrhPass1 r = srh_pass1<false>(c, ncl, a.depth, a.aglh0, u6, v6);
  if ((float)a.aglh0 > r.ztop_f) {
    // Z(1) > Z(NZ): DINTERP2DZ switches to the decreasing-height rule.
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      u6[k] = -999999.f;
      v6[k] = -999999.f;
    }
    r = srh_pass1<true>(c, ncl, a.depth, a.aglh0, u6, v6);
  }
  float rm[2], lm[2], mean[2];
  bunkers_finish((float)c.us, (float)c.vs, u6, v6, rm, lm, mean);
  if (a.rm) {
    a.rm[2 * i] = rm[0];
    a.rm[2 * i + 1] = rm[1];
    a.lm[2 * i] = lm[0];
    a.lm[2 * i + 1] = lm[1];
    a.mean6[2 * i] = mean[0];
    a.mean6[2 * i + 1] = mean[1];
  }
  // Pass 2: DCALRELHL :100-114.
  const double cu_rm = rm[0], cv_rm = rm[1], cu_lm = lm[0], cv_lm = lm[1];
  double s_rm = 0.0, s_lm = 0.0;
  double uprev = c.us, vprev = c.vs;
  for (int k = 2; k <= r.ktop; ++k) {
    double uk, vk;
    if (k == r.ktop) {
      uk = r.utop;
      vk = r.vtop;
    } else {
      uk = ldd(c.u + c.base + k);
      vk = ldd(c.v + c.base + k);
    }
    s_rm = s_rm + (((uk - cu_rm) * (vk - vprev)) - ((vk - cv_rm) * (uk - uprev)));
    s_lm = s_lm + (((uk - cu_lm) * (vk - vprev)) - ((vk - cv_lm) * (uk - uprev)));
    uprev = uk;
    vprev = vk;
  }
  a.srh_rm[i] = -s_rm;
  a.srh_lm[i] = -s_lm;
}

cudaError_t launch_srh(const SrhArgs &a, cudaStream_t s) {
  const int threads = 128;
  const unsigned blocks = (unsigned)((a.n2 + threads - 1) / threads);
  if (blocks == 0) return cudaSuccess;
  if (a.dtype == 0) {
    if (a.grid == 1)
      srh_fused_kernel<float, 1><<<blocks, threads, 0, s>>>(a);
    else
      srh_fused_kernel<float, 2><<<blocks, threads, 0, s>>>(a);
  } else {
    if (a.grid == 1)
      srh_fused_kernel<double, 1><<<blocks, threads, 0, s>>>(a);
    else
      srh_fused_kernel<double, 2><<<blocks, threads, 0, s>>>(a);
  }
  return cudaGetLastError();
}

// ---- stage kernels ----------------------------------------------------------

// loop_stdheight_ml / _pl1d / _pl (start == NULL -> 1; p_stride 0 -> shared p).
__global__ void stdheight_kernel(const double *P, long long p_stride, const double *T,
                                 const double *Td, const double *Ps, const double *Ts,
                                 const double *Tds, const double *Hin, const int *start, int NK,
                                 long long NX, double *H, double *Hs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NX) return;
  int st = start ? start[i] : 1;
  st = st < 1 ? 1 : (st > NK + 1 ? NK + 1 : st);
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

// bunkers_loop_ml / _pl on given heights: DINTERP2DZ exactly as written,
// a top-down scan per target.
__device__ float dinterp2dz_col(const float *V, const float *Z, float vs, float zs, int nz,
                                float loc) {
  // Assembled column: index 1 is the surface (zs, vs), index k >= 2 is Z[k-2].
  auto zat = [&](int k) { return k == 1 ? zs : Z[k - 2]; };
  auto vat = [&](int k) { return k == 1 ? vs : V[k - 2]; };
  int ip = 0, im = 1;
  if (zat(1) > zat(nz)) {
    ip = 1;
    im = 0;
  }
  for (int kp = nz; kp >= 2; --kp) {
    const float za = zat(kp - im), zb = zat(kp - ip);
    if ((za <= loc) && (zb > loc)) {
      const float w2 = (loc - za) / (zb - za);
      const float w1 = (float)(1.0 - (double)w2);
      return w1 * vat(kp - im) + w2 * vat(kp - ip);
    }
  }
  return -999999.f;
}

__global__ void bunkers_kernel(const float *U, const float *V, const float *Z, const float *Us,
                               const float *Vs, const float *Zs, const int *start, int nk,
                               long long n2, float *RM, float *LM, float *Mean) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  int st = start ? start[i] : 1;
  st = st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
  const int nz = nk - st + 2;
  const float *Uc = U + i * nk + st - 1, *Vc = V + i * nk + st - 1, *Zc = Z + i * nk + st - 1;
  float u6[12], v6[12];
  for (int k = 0; k < 12; ++k) {
    const float h = 500.0f * (float)(k + 1);
    u6[k] = dinterp2dz_col(Uc, Zc, Us[i], Zs[i], nz, h);
    v6[k] = dinterp2dz_col(Vc, Zc, Vs[i], Zs[i], nz, h);
  }
  bunkers_finish(Us[i], Vs[i], u6, v6, RM + 2 * i, LM + 2 * i, Mean + 2 * i);
}

// loop_sreh_ml / _pl: DCALRELHL as written.
__global__ void sreh_kernel(const double *u, const double *v, const double *aglh,
                            const double *us, const double *vs, const double *aglhs,
                            const double *cu_rm, const double *cv_rm, const double *cu_lm,
                            const double *cv_lm, double top, const int *start, int nk,
                            long long n2, double *sreh_rm, double *sreh_lm) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n2) return;
  int st = start ? start[i] : 1;
  st = st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
  const int nka = nk - st + 2;
  const double *uc = u + i * nk + st - 1, *vc = v + i * nk + st - 1, *hc = aglh + i * nk + st - 1;
  auto uat = [&](int k) { return k == 1 ? us[i] : uc[k - 2]; };
  auto vat = [&](int k) { return k == 1 ? vs[i] : vc[k - 2]; };
  auto hat = [&](int k) { return k == 1 ? aglhs[i] : hc[k - 2]; };
  int ktop = 0;
  double ut = 0.0, vt = 0.0;
  for (int k = 2; k <= nka; ++k) {
    if (hat(k) > top) {
      ktop = k;
      double x1 = hat(k);
      const double x3 = hat(k - 1);
      if (x3 == x1) x1 = x1 - (double)0.01f;
      ut = uat(k) + ((uat(k - 1) - uat(k)) * ((top - x1) / (x3 - x1)));
      if (x3 == x1) x1 = x1 - (double)0.01f;
      vt = vat(k) + ((vat(k - 1) - vat(k)) * ((top - x1) / (x3 - x1)));
      break;
    }
  }
  double s1 = 0.0, s2 = 0.0;
  for (int k = 2; k <= ktop; ++k) {
    const double uk = k == ktop ? ut : uat(k), vk = k == ktop ? vt : vat(k);
    const double up = uat(k - 1), vp = vat(k - 1);
    s1 = s1 + (((uk - cu_rm[i]) * (vk - vp)) - ((vk - cv_rm[i]) * (uk - up)));
    s2 = s2 + (((uk - cu_lm[i]) * (vk - vp)) - ((vk - cv_lm[i]) * (uk - up)));
  }
  sreh_rm[i] = -s1;
  sreh_lm[i] = -s2;
}

cudaError_t launch_stdheight(const double *P, long long p_stride, const double *T,
                             const double *Td, const double *Ps, const double *Ts,
                             const double *Tds, const double *Hin, const int *start, int NK,
                             long long NX, double *H, double *Hs, cudaStream_t s) {
  const unsigned blocks = (unsigned)((NX + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  stdheight_kernel<<<blocks, 128, 0, s>>>(P, p_stride, T, Td, Ps, Ts, Tds, Hin, start, NK, NX,
                                          H, Hs);
  return cudaGetLastError();
}

cudaError_t launch_bunkers(const float *U, const float *V, const float *Z, const float *Us,
                           const float *Vs, const float *Zs, const int *start, int nk,
                           long long n2, float *RM, float *LM, float *Mean, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n2 + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  bunkers_kernel<<<blocks, 128, 0, s>>>(U, V, Z, Us, Vs, Zs, start, nk, n2, RM, LM, Mean);
  return cudaGetLastError();
}

cudaError_t launch_sreh(const double *u, const double *v, const double *aglh, const double *us,
                        const double *vs, const double *aglhs, const double *cu_rm,
                        const double *cv_rm, const double *cu_lm, const double *cv_lm,
                        double top, const int *start, int nk, long long n2, double *sreh_rm,
                        double *sreh_lm, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n2 + 127) / 128);
  if (blocks == 0) return cudaSuccess;
  sreh_kernel<<<blocks, 128, 0, s>>>(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top,
                                     start, nk, n2, sreh_rm, sreh_lm);
  return cudaGetLastError();
}

}  // namespace xc
