// cape_learned.cuh -- the learned solver's column routine for sm_103a
// kernels: the guess network evaluated per warp on the tensor cores, then
// the ascent (cape_learned_kernel in cape_kernel.cu, the fused CAPE + SRH
// kernel in cape_srh.cu).  Device code only.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

#include "cape_column.cuh"
#include "xc_kernels.h"

namespace xc {

// A block of LEARNED_THREADS threads runs each column in three phases:
// (1) every lane selects its parcel's source and forms the network's inputs
// at the parcel's LCL; (2) the warp, converged (__syncwarp), evaluates the
// network for its 32 columns at once -- the 64x64 hidden layer as
// 2 x 8 x 4 mma.sync.m16n8k16 (BF16 operands, FP32 accumulation, as in
// training); (3) every lane runs the ascent with that output (ascend_col).
// No lane leaves before phase 2: lanes without a column (past n2, ts <= 0,
// bad start, no ascent) take part with zero inputs and discard the result.
// Shared memory per block: the network's 9.7 KB image and a 32-byte handoff
// record per thread.
struct WarpNetSmem {
  float4 l1[GUESS_H];                               // {W1[k][0..2], b1[k]}
  float b2[GUESS_H], w3[GUESS_H], b3;
  alignas(16) uint32_t w2[GUESS_H * GUESS_H / 2];   // W2 as bf16 pairs, swizzled rows
};

// 32-bit word w (a bf16 pair) of 64-wide row r, XOR-swizzled so that the
// fragment loads of 8 consecutive rows hit 8 different bank groups.
__device__ __forceinline__ int swz(int r, int w) { return r * 32 + (w ^ ((r & 7) << 2)); }

__device__ __forceinline__ uint32_t bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ inline void load_warp_net(WarpNetSmem &s, const float *w) {
  for (int k = threadIdx.x; k < GUESS_H; k += blockDim.x) {
    s.l1[k] = make_float4(w[GUESS_OFF_W1 + 3 * k], w[GUESS_OFF_W1 + 3 * k + 1],
                          w[GUESS_OFF_W1 + 3 * k + 2], w[GUESS_OFF_B1 + k]);
    s.b2[k] = w[GUESS_OFF_B2 + k];
    s.w3[k] = w[GUESS_OFF_W3 + k];
  }
  if (threadIdx.x == 0) s.b3 = w[GUESS_OFF_B3];
  for (int e = threadIdx.x; e < GUESS_H * GUESS_H / 2; e += blockDim.x) {
    const int n = e / (GUESS_H / 2), wd = e % (GUESS_H / 2);
    s.w2[swz(n, wd)] = bf16x2(w[GUESS_OFF_W2 + n * GUESS_H + 2 * wd],
                              w[GUESS_OFF_W2 + n * GUESS_H + 2 * wd + 1]);
  }
}

constexpr int LEARNED_THREADS = 128;  // the learned kernel's block size

static_assert(sizeof(WarpNetSmem) % 16 == 0, "WarpNetSmem is copied in 16-byte words");

// The network's image (built by build_warp_net) into a block's shared
// memory, by the LEARNED_THREADS threads.
__device__ __forceinline__ void copy_warp_net(WarpNetSmem &dst, const WarpNetSmem *img) {
  constexpr int N16 = sizeof(WarpNetSmem) / 16;
  const uint4 *src = reinterpret_cast<const uint4 *>(img);
  uint4 *d = reinterpret_cast<uint4 *>(&dst);
#pragma unroll
  for (int k = 0; k < (N16 + LEARNED_THREADS - 1) / LEARNED_THREADS; ++k) {
    const int e = k * LEARNED_THREADS + (int)threadIdx.x;
    if (e < N16) d[e] = src[e];
  }
}

// Element (row with inputs f, column k) of the first layer, relu'd.
__device__ __forceinline__ float l1_unit(const WarpNetSmem &s, const float (&f)[3], int k) {
  const float4 l = s.l1[k];
  const float h = l.w + l.x * f[0] + l.y * f[1] + l.z * f[2];
  return h > 0.0f ? h : 0.0f;
}

// The network's output for the calling lane's inputs; all 32 lanes of the
// warp must call it together.  Rows of the hidden-layer product are the
// warp's lanes; each lane builds the A fragments it holds (rows gid,
// gid + 8, 16 + gid, 24 + gid of the 32 x 64 activation matrix, fetched as
// inputs by shuffle) in registers, so no activation tile goes through
// shared memory.
__device__ inline float warp_guess_eval(const WarpNetSmem &s, float f0, float f1, float f2) {
  const int lane = threadIdx.x & 31;
  const int gid = lane >> 2, tig = lane & 3;
  float yp[4];  // rows gid, gid + 8, 16 + gid, 24 + gid
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    // the A fragments of rows mt*16 + gid and mt*16 + gid + 8, k = 0..63
    uint32_t a[4][4];  // [k step][fragment register]
    float lo[3], hi[3];
    const int rlo = mt * 16 + gid, rhi = rlo + 8;
    lo[0] = __shfl_sync(0xffffffffu, f0, rlo);
    lo[1] = __shfl_sync(0xffffffffu, f1, rlo);
    lo[2] = __shfl_sync(0xffffffffu, f2, rlo);
    hi[0] = __shfl_sync(0xffffffffu, f0, rhi);
    hi[1] = __shfl_sync(0xffffffffu, f1, rhi);
    hi[2] = __shfl_sync(0xffffffffu, f2, rhi);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int c = ks * 16 + tig * 2;
      a[ks][0] = bf16x2(l1_unit(s, lo, c), l1_unit(s, lo, c + 1));
      a[ks][1] = bf16x2(l1_unit(s, hi, c), l1_unit(s, hi, c + 1));
      a[ks][2] = bf16x2(l1_unit(s, lo, c + 8), l1_unit(s, lo, c + 9));
      a[ks][3] = bf16x2(l1_unit(s, hi, c + 8), l1_unit(s, hi, c + 9));
    }
    float ylo = 0.0f, yhi = 0.0f;
    for (int nt = 0; nt < GUESS_H / 8; ++nt) {
      float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      const int n = nt * 8 + gid;
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const int wd = ks * 8 + tig;
        mma16816(acc, a[ks], s.w2[swz(n, wd)], s.w2[swz(n, wd + 4)]);
      }
      const int c = nt * 8 + tig * 2;
      const float z0 = acc[0] + s.b2[c], z1 = acc[1] + s.b2[c + 1];
      const float z2 = acc[2] + s.b2[c], z3 = acc[3] + s.b2[c + 1];
      ylo += s.w3[c] * (z0 > 0.0f ? z0 : 0.0f) + s.w3[c + 1] * (z1 > 0.0f ? z1 : 0.0f);
      yhi += s.w3[c] * (z2 > 0.0f ? z2 : 0.0f) + s.w3[c + 1] * (z3 > 0.0f ? z3 : 0.0f);
    }
    yp[2 * mt] = ylo;
    yp[2 * mt + 1] = yhi;
  }
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    yp[j] += __shfl_xor_sync(0xffffffffu, yp[j], 1);
    yp[j] += __shfl_xor_sync(0xffffffffu, yp[j], 2);
  }
  // row `lane` is held (whole) by the lanes of quad (lane & 7), in yp[j]
  const int src = (lane & 7) * 4, j = ((lane >> 4) << 1) | ((lane >> 3) & 1);
  const float v0 = __shfl_sync(0xffffffffu, yp[0], src);
  const float v1 = __shfl_sync(0xffffffffu, yp[1], src);
  const float v2 = __shfl_sync(0xffffffffu, yp[2], src);
  const float v3 = __shfl_sync(0xffffffffu, yp[3], src);
  return (j == 0 ? v0 : j == 1 ? v1 : j == 2 ? v2 : v3) + s.b3;
}

// What phases 1 and 2 hand to phase 3, per thread, through shared memory:
// nothing of the source selection or the network stays live in registers
// across the network's evaluation or the ascent.
struct LearnedPrep {
  int start, kmax, mulvl, status;  // status: COL_* bits, or PREP_RUN when the ascent runs
  float avgth, avgqv, y, pad;
};
constexpr int PREP_RUN = 1 << 30;

// Column perm[t] (t when unordered) of the learned solver, for thread t of
// a LEARNED_THREADS-thread block whose shared memory holds the network
// (net, copied by copy_warp_net) and the handoff records (prep); every
// thread of the block calls it, also past n2.  Writes the CAPE outputs and
// the thread's work counts.
// Phases 1 and 2 for column i of thread t (all 32 lanes of the warp call
// it; inactive lanes, past n2, take part with zero inputs): the column's
// start, gate and source (cape_column_run, getcape_col), then the network
// for the warp's 32 columns at the parcel's LCL.
template <typename T, int GRID>
__device__ __forceinline__ LearnedPrep learned_prepare(const CapeArgs &a, const WarpNetSmem &net,
                                                       long long i, bool active) {
  const long long stride = a.ld > 0 ? a.ld : a.nk;
  int start = 1, status = 0;
  SourceSel sel;
  sel.kmax = 1;
  sel.mulvl = 0;
  sel.avgth = sel.avgqv = 0.0f;
  sel.ascend = false;
  float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f;
  if (active) {
    const float ts = ldf((const T *)a.ts + i);
    if (GRID != 1)
      start = a.start ? __ldg(a.start + i)
                      : pres_lev_pos_col<T>((const T *)a.p, __ldg((const T *)a.ps + i), a.nk);
    if (ts > 0.0f) {  // CAPE_CODE_model_lev.f90:77
      if (start < 1 || start > a.nk) {
        status = COL_BADSTART;
      } else {
        ColumnReader<T, GRID> col;
        col.set((const T *)a.p, (const T *)a.t, (const T *)a.td, i * stride, start);
        col.ps = ldf((const T *)a.ps + i);
        col.ts = ts;
        col.tds = ldf((const T *)a.tds + i);
        sel = select_source<true>(col, a.nk - start + 2, a.source, a.ml_depth);
        if (sel.ascend) {
          float p0, t0, td0, q0;
          source_parcel<true>(col, sel, a.source, p0, t0, td0, q0);
          lcl_features(p0, t0, td0, q0, f0, f1, f2);
          status = PREP_RUN;
        }
      }
    }
  }
  __syncwarp();
  LearnedPrep q;
  q.y = warp_guess_eval(net, f0, f1, f2);
  q.start = start;
  q.kmax = sel.kmax;
  q.mulvl = sel.mulvl;
  q.status = status;
  q.avgth = sel.avgth;
  q.avgqv = sel.avgqv;
  q.pad = 0.0f;
  return q;
}

// Phase 3 for column i from its record q: the ascent and the outputs.
template <typename T, int GRID, bool ICE, bool PSEUDO>
__device__ __forceinline__ void learned_ascend(const CapeArgs &a, const LearnedPrep &q,
                                               long long i, bool active, int &nsub, int &niter) {
  const long long stride = a.ld > 0 ? a.ld : a.nk;
  float cape = 0.0f, cin = 0.0f, zo = 0.0f;
  int mulvl = 0, status = q.status & ~PREP_RUN;
  nsub = 0;
  niter = 0;
  if (active && status == 0 && ldf((const T *)a.ts + i) > 0.0f) {
    SourceSel sel;
    sel.kmax = q.kmax;
    sel.mulvl = q.mulvl;
    sel.avgth = q.avgth;
    sel.avgqv = q.avgqv;
    sel.ascend = true;
    CapeResult r;
    if (q.status & PREP_RUN) {
      ColumnReader<T, GRID> col;
      col.set((const T *)a.p, (const T *)a.t, (const T *)a.td, i * stride, q.start);
      col.ps = ldf((const T *)a.ps + i);
      col.ts = ldf((const T *)a.ts + i);
      col.tds = ldf((const T *)a.tds + i);
      r = ascend_col<ICE, PSEUDO, SOLVE_LEARNED, false>(col, a.nk - q.start + 2, a.pinc, a.source,
                                                        sel, nullptr, nullptr, q.y);
    } else {
      r.mulvl = sel.mulvl;
      r.z_out = -999999.f;
      r.cape = 0.0f;
      r.cin = 0.0f;
      r.status = 0;
      r.nsub = 0;
      r.niter = 0;
    }
    cape = r.cape;
    cin = r.cin;
    zo = r.z_out;
    mulvl = r.mulvl;
    status = r.status;
    nsub = r.nsub;
    niter = r.niter;
  }
  if (active) {
    a.cape[i] = cape;
    a.cin[i] = cin;
    a.mulvl[i] = mulvl;
    a.z_out[i] = zo;
    if (a.status) a.status[i] = status;
  }
}

// Column perm[t] (t when unordered) of the learned solver in one kernel, for
// thread t of a LEARNED_THREADS-thread block whose shared memory holds the
// network (net, copied by copy_warp_net) and the handoff records (prep);
// every thread of the block calls it, also past n2.  The record goes
// through shared memory so that nothing of phases 1-2 stays live in
// registers across the ascent.
template <typename T, int GRID, bool ICE, bool PSEUDO>
__device__ __forceinline__ void learned_column(const CapeArgs &a, const WarpNetSmem &net,
                                               LearnedPrep *prep, long long t, int &nsub,
                                               int &niter) {
  const bool active = t < a.n2;
  const long long i = active ? (a.perm ? (long long)__ldg(a.perm + t) : t) : 0;
  prep[threadIdx.x] = learned_prepare<T, GRID>(a, net, i, active);
  __syncwarp();
  const LearnedPrep q = prep[threadIdx.x];
  learned_ascend<T, GRID, ICE, PSEUDO>(a, q, i, active, nsub, niter);
}

}  // namespace xc

namespace xc {

// The ascent (:355-559) of SOLVE_LEARNED_WARP, in warp lockstep: every lane
// walks its own column, but one sub-step at a time for the whole warp, so
// that before each sub-step the warp evaluates the guess network for the 32
// lanes' states at once on the tensor cores (warp_guess_eval).  A lane
// between levels finishes the level it has sub-stepped through (buoyancy,
// areas) and prepares the next one (advance) before the next evaluation;
// lanes that are done, or whose parcel does not start the sub-step
// saturated, take part in the evaluation with zero inputs and discard the
// output.  The map, the stopping test and the result are those of every
// accelerated solver; only the first guess of a saturated sub-step comes
// from the network: theta1 + 50 K y ln(p1/p2), with y the network's output
// at (p2, theta-e of the saturated parcel, total water).
// All 32 lanes of the warp must call it; `live` is false for lanes without
// an ascent (past n2, ts <= 0, bad start, no ascent from the source).
template <bool ICE, bool PSEUDO, typename T, int GRID>
__device__ CapeResult ascend_col_warp(const ColumnReader<T, GRID> &col, int ncl, float pinc,
                                      int source, const SourceSel &sel, const WarpNetSmem &net,
                                      bool live) {
  CapeResult r;
  r.mulvl = sel.mulvl;
  r.z_out = -999999.f;
  r.cape = 0.0f;
  r.cin = 0.0f;
  r.status = 0;
  r.nsub = 0;
  r.niter = 0;
  const int kmax = sel.kmax;
  const float avgth = sel.avgth, avgqv = sel.avgqv;
  Env prev, cur;
  prev.p = prev.t = prev.td = prev.pi = prev.q = prev.th = prev.thv = 0.0f;
  cur = prev;
  float z = 0.0f, dz = 0.0f, dp = 0.0f, b1 = 0.0f;
  float th2 = 0.f, p2 = 0.f, t2 = 0.f, qv2 = 0.f, b2 = 0.f, ql2 = 0.f, qi2 = 0.f, qt = 0.f;
  float narea = 0.0f;
  SolverState ss;
  Acc<true> cape_acc, cin_acc;
  int k = 1, n = 0, nloop = 0;
  bool done = !live, aborted = false;
  auto init_parcel = [&](const Env &e) {
    if (source == 3) {
      th2 = avgth;
      qv2 = avgqv;
      const float thv2 = th2 * (1.0f + REPS * qv2) / (1.0f + qv2);
      p2 = e.p;
      t2 = th2 * e.pi;
      b2 = G * (thv2 - e.thv) / e.thv;
    } else {
      th2 = e.th;
      p2 = e.p;
      t2 = e.t;
      qv2 = e.q;
      b2 = 0.0f;
    }
    ql2 = 0.0f;
    qi2 = 0.0f;
    qt = qv2;
    ss.lnp = fast_log(p2);
  };
  // Finishes the level whose sub-steps are done and walks up to the next
  // level that needs sub-steps (or to the end of the ascent).
  auto advance = [&]() {
    while (!done) {
      if (n < nloop) return;
      if (nloop > 0) {
        // :501-557, as ascend_col
        const float thv2 = fast_div(th2 * (1.0f + REPS * qv2), 1.0f + qv2 + ql2 + qi2);
        b2 = fast_div(G * (thv2 - cur.thv), cur.thv);
        float parea;
        if ((b2 >= 0.0f) && (b1 < 0.0f)) {
          const float frac = b2 / (b2 - b1);
          parea = 0.5f * b2 * dz * frac;
          narea = narea - 0.5f * b1 * dz * (1.0f - frac);
          cin_acc.add(narea);
          narea = 0.0f;
        } else if ((b2 < 0.0f) && (b1 > 0.0f)) {
          const float frac = b1 / (b1 - b2);
          parea = 0.5f * b1 * dz * frac;
          narea = -0.5f * b2 * dz * (1.0f - frac);
        } else if (b2 < 0.0f) {
          parea = 0.0f;
          narea = narea - 0.5f * dz * (b1 + b2);
        } else {
          parea = 0.5f * dz * (b1 + b2);
          narea = 0.0f;
        }
        cape_acc.add(fmax_f(0.0f, parea));
        r.z_out = z;
        nloop = 0;
        if ((cur.p <= 10000.0f) && (b2 < 0.0f)) {
          done = true;
          return;
        }
        prev = cur;
      }
      if (++k > ncl) {
        done = true;
        return;
      }
      cur = col.template env_above<true>(k);
      dz = -CPDG * 0.5f * (cur.thv + prev.thv) * (cur.pi - prev.pi);
      z = z + dz;
      if (k <= kmax) {
        if (k == kmax) init_parcel(cur);
        prev = cur;
        continue;
      }
      b1 = b2;
      dp = prev.p - cur.p;
      if (dp < pinc) {
        nloop = 1;
      } else {
        const float f = dp / pinc;
        if (!(f < (float)MAX_SUBSTEPS)) {
          r.status |= COL_TOOMANYSTEPS;
          done = aborted = true;
          return;
        }
        nloop = 1 + (int)f;
        dp = dp / (float)nloop;
      }
      ss.rdp = fast_rcp(dp);
      if (r.nsub + nloop > MAX_SUBSTEPS) {
        r.status |= COL_TOOMANYSTEPS;
        done = aborted = true;
        return;
      }
      n = 0;
    }
  };
  if (live) {
    prev = col.template env<true>(1);
    if (kmax == 1) init_parcel(prev);
  }
  advance();
  while (__any_sync(0xffffffffu, !done)) {
    float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, lpn = 0.0f;
    const bool use_net = !done && ss.saturated;
    if (use_net) {
      const float pn = p2 - dp;
      lpn = fast_log(pn) - ss.lnp;
      guess_features(pn, getthe_fast(p2, t2, t2, qv2), qt, f0, f1, f2);
    }
    __syncwarp();
    const float y = warp_guess_eval(net, f0, f1, f2);
    if (!done) {
      ss.net_dth = (use_net && y >= GUESS_Y_MIN && y <= GUESS_Y_MAX) ? -GUESS_SLOPE_SCALE * y * lpn
                                                                    : NAN;
      ++r.nsub;
      ++n;
      if (!substep<ICE, PSEUDO, SOLVE_LEARNED_WARP>(dp, p2, t2, th2, qv2, ql2, qi2, qt, r.niter,
                                                    ss)) {
        r.status |= COL_NOCONV;  // :471-473
        done = aborted = true;
      } else {
        advance();
      }
    }
  }
  if (!aborted) {
    r.cape = cape_acc.s;
    r.cin = cin_acc.s;
  }
  return r;
}

// Column perm[t] (t when unordered) of SOLVE_LEARNED_WARP for thread t of a
// LEARNED_THREADS-thread block whose shared memory holds the network; every
// thread of the block calls it, also past n2.
template <typename T, int GRID, bool ICE, bool PSEUDO>
__device__ __forceinline__ void learned_warp_column(const CapeArgs &a, const WarpNetSmem &net,
                                                    long long t, int &nsub, int &niter) {
  const bool active = t < a.n2;
  const long long i = active ? (a.perm ? (long long)__ldg(a.perm + t) : t) : 0;
  const long long stride = a.ld > 0 ? a.ld : a.nk;
  int start = 1, status = 0;
  SourceSel sel;
  sel.kmax = 1;
  sel.mulvl = 0;
  sel.avgth = sel.avgqv = 0.0f;
  sel.ascend = false;
  ColumnReader<T, GRID> col;
  col.set((const T *)a.p, (const T *)a.t, (const T *)a.td, 0, 3);
  col.ps = col.ts = col.tds = 0.0f;
  bool gate = false, live = false;
  if (active) {
    const float ts = ldf((const T *)a.ts + i);
    if (GRID != 1)
      start = a.start ? __ldg(a.start + i)
                      : pres_lev_pos_col<T>((const T *)a.p, __ldg((const T *)a.ps + i), a.nk);
    gate = ts > 0.0f;  // CAPE_CODE_model_lev.f90:77
    if (gate) {
      if (start < 1 || start > a.nk) {
        status = COL_BADSTART;
      } else {
        col.set((const T *)a.p, (const T *)a.t, (const T *)a.td, i * stride, start);
        col.ps = ldf((const T *)a.ps + i);
        col.ts = ts;
        col.tds = ldf((const T *)a.tds + i);
        sel = select_source<true>(col, a.nk - start + 2, a.source, a.ml_depth);
        live = sel.ascend;
      }
    }
  }
  CapeResult r = ascend_col_warp<ICE, PSEUDO, T, GRID>(col, a.nk - start + 2, a.pinc, a.source,
                                                       sel, net, live);
  nsub = r.nsub;
  niter = r.niter;
  if (active) {
    const bool ran = gate && status == 0;
    a.cape[i] = ran ? r.cape : 0.0f;
    a.cin[i] = ran ? r.cin : 0.0f;
    a.mulvl[i] = ran ? r.mulvl : 0;
    a.z_out[i] = ran ? r.z_out : 0.0f;
    if (a.status) a.status[i] = ran ? r.status : status;
  }
}

}  // namespace xc
