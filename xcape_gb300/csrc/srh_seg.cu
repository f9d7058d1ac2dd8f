// srh_seg.cu -- the FP32 storm-relative helicity kernel for float inputs
// (calc_srh with precision='fp32'): stdheight -> Bunkers -> SREH of one
// column per segment of SEG = 8 lanes, four columns per warp.
//
// A segment sweeps its column in rounds of SEG * RUN levels, lane l taking the
// RUN consecutive levels j0 = 2 + round * SEG * RUN + l * RUN .. j0 + RUN - 1 of
// the assembled column (level 1 is the surface).  Each lane reads its run of
// every input row (a run's sectors stay in L1 between its levels), so the
// per-column dependent chain is RUN levels long, and the lanes talk once per
// round:
//   * per lane, straight-line: the virtual temperature of each level and the
//     hypsometric increment from the level below (the level below the run's
//     first comes from the lane below by shuffle, or from the previous
//     round);
//   * the heights: each lane's running sum on top of the segment's exclusive
//     scan of the lanes' totals and of the previous round's last height;
//   * per lane: a level whose layer [z(j-1), z(j)) holds Bunkers targets
//     interpolates the winds there (DINTERP2DZ, Bunkers_model_lev.f90:
//     188-236) into the column's target slots in shared memory; the first
//     level above `depth` interpolates the winds at `depth` (INTERP1,
//     SREH_model_lev.f90:123-129); every level up to it adds its term of the
//     storm-motion free part of the helicity sums,
//       A = sum_k (u_k dv_k - v_k du_k) = sum_k (u_(k-1) v_k - u_k v_(k-1)).
// The helicity for storm motion (c_u, c_v) then is
//   sum_k (u_k - c_u) dv_k - (v_k - c_v) du_k = A - c_u (v_top - v_s) + c_v (u_top - u_s)
// since dv and du telescope.  This needs heights that increase with level:
// each target then falls in exactly one layer, the highest bracket that
// DINTERP2DZ keeps.  A column whose heights do not increase (pressures that
// do not decrease, a non-finite input), or that has fewer levels above the
// ground than one run, is redone by its segment's first lane with the
// one-thread FP32 column routine (srh_column_run), which follows the
// reference's scan rules for any column.
//
// The arithmetic is FP32 with approximate transcendentals; the contract is
// the FP32 path's, agreement with the FP64 reference within tolerance:
//   E  = 6.112 exp(53.49 - 6808/Td - 5.09 ln Td)   (Td in K, E in hPa)
//   Tv = T (w + eps) / (eps (1 + w)),  w = eps E / (P - E)
//      = T P / (P - (1 - eps) E)
// (stdheight_2D_model_lev.f90:116-131), one reciprocal instead of three
// divides, and log2 E = K0 - K1/Td - 5.09 log2 Td; the hypsometric step
// (:147, :155) between level b (below) and level a
//   dz = (R/|g|) (Tv_a + Tv_b)/2 ln(P_b / P_a) = (C Tv_a + C Tv_b) log2(P_b / P_a),
// with C = (R/|g|) ln(2) / 2 folded into the virtual temperature.  The
// transcendentals are the PTX approximations with subnormals flushed to zero:
// their operands (temperatures in K, pressures in hPa and their ratios) are
// far from the subnormal range for any physical column.
//
// Every lane loads and computes unconditionally: it reads a window of RUN
// levels inside its column's row (its run, or the row's last RUN levels for
// a run that reaches past the column top), at fixed offsets from one
// pointer per array, and a bit mask of the window's slots that hold its own
// levels keeps the others out of the sums; segments past the last column
// read the last column.  The window needs nk >= RUN.
#include "srh_column.cuh"
#include "tc05.cuh"
#include "xc_kernels.h"

namespace xc {
namespace {

constexpr int SEG = 8;
constexpr int SEG_THREADS = 128;

__device__ __forceinline__ float rcp_a(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float lg2_a(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2_a(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

constexpr float SEG_K0 = 79.78140228f;  // log2(6.112) + 53.49 log2(e)
constexpr float SEG_K1 = (float)(6808.0 * 1.4426950408889634);  // 6808 log2(e)
constexpr float SEG_K2 = 5.09f;
constexpr float SEG_OME = (float)(1.0 - (double)0.6219800858985514f);  // 1 - eps
constexpr float SEG_C = (float)((double)287.04f / (double)9.80665f * 0.5 * 0.6931471805599453);

// C Tv of a level: P in hPa, T and Td in degC.
__device__ __forceinline__ float seg_ctv(float P, float T, float Td) {
  const float tdk = Td + 273.15f;
  const float l2e = fmaf(-SEG_K2, lg2_a(tdk), fmaf(-SEG_K1, rcp_a(tdk), SEG_K0));
  const float den = fmaf(-SEG_OME, ex2_a(l2e), P);
  return fmaf(SEG_C, T, SEG_C * 273.15f) * P * rcp_a(den);
}

// Number of the Bunkers targets 500, 1000, ..., 6000 m lying below z (0 for
// NaN).  It is monotone in z, so with heights increasing the targets of the
// layer [z_lo, z_hi) are those numbered seg_below(z_lo) .. seg_below(z_hi) - 1
// and every target falls in exactly one layer; a target within rounding of a
// layer boundary may fall in the layer on the other side, where its
// interpolation weight is 0 or 1 within rounding.
__device__ __forceinline__ int seg_below(float z) {
  const int k = __float2int_ru(z * (1.0f / 500.0f));
  return min(max(k, 1), 13) - 1;
}

// Bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on the mbarrier's transaction
// count (cp.async.bulk, non-tensor).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n"
      :: "r"(tc05::smem_u32(dst)), "l"(src), "r"(bytes), "r"(tc05::smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n"
               :: "r"(tc05::smem_u32(bar)), "r"(bytes) : "memory");
}

}  // namespace

// The column's outputs from its segment's partial sums: A over the lanes,
// the winds at depth from the crossing lane, the Bunkers storm motions
// (bunkers_calc_ml, Bunkers_model_lev.f90:123-177: the 0-6 km mean wind of
// the surface and the 12 targets, and the shear from the 0-500 m mean to the
// 5.5-6 km mean) from the target slots, one output written per lane.  A
// column with irregular heights is redone by the segment's first lane with
// the column routine.  Every lane of the warp calls it.
template <int GRID>
__device__ __forceinline__ void seg_finish(const SrhArgs &a, long long i, bool active, bool mono,
                                           int ktop, float A, float utop, float vtop, float us,
                                           float vs, const float *su6, const float *sv6) {
  constexpr unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int sl = lane & (SEG - 1);
  const unsigned seg_mask = 0xffu << (lane & ~(SEG - 1));
  float ut = utop, vt = vtop;
#pragma unroll
  for (int d = SEG / 2; d > 0; d >>= 1) {
    A += __shfl_xor_sync(FULL, A, d, SEG);
    ut += __shfl_xor_sync(FULL, ut, d, SEG);
    vt += __shfl_xor_sync(FULL, vt, d, SEG);
  }
  const bool all_mono = (__ballot_sync(FULL, !mono) & seg_mask) == 0;
  __syncwarp();
  float su = su6[sl] + (sl < 4 ? su6[sl + 8] : 0.0f);
  float sv = sv6[sl] + (sl < 4 ? sv6[sl + 8] : 0.0f);
#pragma unroll
  for (int d = SEG / 2; d > 0; d >>= 1) {
    su += __shfl_xor_sync(FULL, su, d, SEG);
    sv += __shfl_xor_sync(FULL, sv, d, SEG);
  }
  if (!active) return;
  if (!all_mono) {
    if (sl == 0) srh_column_run<float, GRID, true>(a, i);  // the reference's scan rules
    return;
  }
  const float m0 = (us + su) * (1.0f / 13.0f), m1 = (vs + sv) * (1.0f / 13.0f);
  const float ushr = 0.5f * (su6[10] + su6[11]) - 0.5f * (us + su6[0]);
  const float vshr = 0.5f * (sv6[10] + sv6[11]) - 0.5f * (vs + sv6[0]);
  const float f = 7.5f * rsqrtf(fmaf(ushr, ushr, vshr * vshr));
  const float rm0 = fmaf(f, vshr, m0), rm1 = fmaf(-f, ushr, m1);
  const float lm0 = fmaf(-f, vshr, m0), lm1 = fmaf(f, ushr, m1);
  if (sl < 2) {
    double h = -0.0;
    if (ktop > 0) {
      const float cu = sl == 0 ? rm0 : lm0, cv = sl == 0 ? rm1 : lm1;
      h = -(double)fmaf(cv, ut - us, fmaf(-cu, vt - vs, A));
    }
    (sl == 0 ? a.srh_rm : a.srh_lm)[i] = h;
  } else if (a.rm) {
    float *dst = sl < 4 ? a.rm : (sl < 6 ? a.lm : a.mean6);
    const float val = sl == 2 ? rm0 : sl == 3 ? rm1 : sl == 4 ? lm0 : sl == 5 ? lm1
                    : sl == 6 ? m0 : m1;
    dst[2 * i + (sl & 1)] = val;
  }
}

// STAGED: the block's 16 rows of p (sigma grids), t, td, u and v are first
// copied into shared memory by bulk copies (one per array: the rows are one
// contiguous range), and the lanes read their windows from there; the
// blocks must be full and the arrays 16-byte aligned.  A block whose copies
// do not arrive within the wait's limit lets its first lane of each segment
// run the column routine instead (results unchanged).
template <int GRID, int RUN, bool STAGED>
__global__ void __launch_bounds__(SEG_THREADS, 8) srh_seg_kernel(SrhArgs a) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int COLS = SEG_THREADS / SEG;  // columns per block
  constexpr int ROUND = SEG * RUN;
  constexpr int NARR = GRID == 1 ? 5 : 4;  // staged arrays: t, td, u, v (, p)
  __shared__ float slot_u[COLS][12], slot_v[COLS][12];
  extern __shared__ __align__(128) float stage[];  // [NARR][COLS * nk] when STAGED
  __shared__ uint64_t stage_bar;
  const int lane = threadIdx.x & 31;
  const int sl = lane & (SEG - 1);
  const unsigned seg_mask = 0xffu << (lane & ~(SEG - 1));
  // the column within the block: segment 4w + j of warp w takes column
  // 4w + j, or with seg_colmap 4j + w (the staged rows of columns four
  // apart can start in other shared-memory banks)
  const int seg = threadIdx.x / SEG;
  const int cb = STAGED && a.seg_colmap ? ((seg & 3) << 2) | (seg >> 2) : seg;
  const long long i = (long long)blockIdx.x * COLS + cb;
  const bool active = i < a.n2;
  const long long ic = active ? i : a.n2 - 1;  // the column whose inputs this segment reads
  const int nk = a.nk;
  const float *gp = (const float *)a.p, *gt = (const float *)a.t, *gtd = (const float *)a.td;
  const float *gu = (const float *)a.u, *gv = (const float *)a.v;
  const float ps = __ldg((const float *)a.ps + ic), ts = __ldg((const float *)a.ts + ic);
  const float tds = __ldg((const float *)a.tds + ic);
  const float us = __ldg((const float *)a.us + ic), vs = __ldg((const float *)a.vs + ic);
  int st = 1;
  if (GRID == 2) {
    st = a.start ? __ldg(a.start + ic) : pres_lev_pos_col<float>(gp, ps, nk);
    st = st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
  }
  const int ncl = nk - st + 2;  // assembled levels: 1 (surface) .. ncl
  long long row = ic * nk;
  const int base = st - 3;  // 0-based input index of assembled level j: base + j
  if (STAGED) {
    const long long g0 = (long long)blockIdx.x * COLS * nk;
    const uint32_t bytes = (uint32_t)(COLS * nk * sizeof(float));
    if (threadIdx.x == 0) tc05::mbar_init(&stage_bar, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      mbar_expect_tx(&stage_bar, NARR * bytes);
      const float *src[5] = {gt, gtd, gu, gv, gp};
#pragma unroll
      for (int k = 0; k < NARR; ++k)
        bulk_g2s(stage + k * COLS * nk, src[k] + g0, bytes, &stage_bar);
    }
    const bool arrived = __syncthreads_and(tc05::mbar_wait(&stage_bar, 0, 1u << 22));
    if (!arrived) {
      if (sl == 0 && active) srh_column_run<float, GRID, true>(a, i);
      if (threadIdx.x == 0) tc05::mbar_wait(&stage_bar, 0, 1u << 22);  // the copies in flight
      return;
    }
    // the lanes read their windows from the block's rows in shared memory
    gt = stage;
    gtd = stage + COLS * nk;
    gu = stage + 2 * COLS * nk;
    gv = stage + 3 * COLS * nk;
    if (GRID == 1) gp = stage + 4 * COLS * nk;
    row = (long long)cb * nk;
  }
  for (int k = sl; k < 24; k += SEG) {
    if (k < 12) slot_u[cb][k] = VMSG;
    else slot_v[cb][k - 12] = VMSG;
  }
  __syncwarp();
  const float depth = (float)a.depth;
  // the level below the round's first level: the surface to begin with
  float Pc = ps, Cc = seg_ctv(ps, ts, tds), uc = us, vc = vs, Hc = (float)a.aglh0;
  // a column with fewer levels above the ground than one run would read
  // levels below the ground into its first window: the column routine
  // takes it, as it takes columns whose heights do not increase
  bool mono = ncl - 1 >= RUN;
  int ktop = 0;
  float utop = 0.0f, vtop = 0.0f, A = 0.0f;
  const int nrounds = active ? (ncl - 1 + ROUND - 1) / ROUND : 0;
  const int wrounds = __reduce_max_sync(FULL, nrounds);
  for (int r = 0; r < wrounds; ++r) {
    // this lane's levels: mb .. mb + RUN - 1 (0-based input indices), read
    // through a window of RUN levels inside the row -- the run itself, or for
    // a run that reaches past the column top the last RUN levels of the row,
    // whose first `lo` slots are levels of the lane below
    const int mb = base + 2 + r * ROUND + sl * RUN;
    const int ws = min(mb, nk - RUN);
    const int lo = r < nrounds ? min(mb - ws, RUN) : RUN;
    const unsigned valid = (0xffu << lo) & ((1u << RUN) - 1);  // slots holding this lane's levels
    const float *wp = GRID == 2 ? gp + ws : gp + row + ws;
    const float *wt = gt + row + ws, *wtd = gtd + row + ws;
    const float *wu = gu + row + ws, *wv = gv + row + ws;
    float u[RUN], v[RUN], z[RUN];
    float Pf = 0.0f, Cf = 0.0f, Pl = 0.0f, Cl = 0.0f;  // first and last slot's P and C Tv
    float s = 0.0f;  // running sum of the increments of slots 1 .. RUN-1
#pragma unroll
    for (int c = 0; c < RUN; ++c) {
      const float P = STAGED && GRID == 1 ? wp[c] : __ldg(wp + c);
      u[c] = STAGED ? wu[c] : __ldg(wu + c);
      v[c] = STAGED ? wv[c] : __ldg(wv + c);
      const float ct = seg_ctv(P, STAGED ? wt[c] : __ldg(wt + c), STAGED ? wtd[c] : __ldg(wtd + c));
      if (c == 0) {
        Pf = P;
        Cf = ct;
        z[0] = 0.0f;
      } else {
        const float dz = (ct + Cl) * lg2_a(Pl * rcp_a(P));
        const bool ok = (valid >> c) & 1u;
        mono = mono && (!ok || dz > 0.0f);
        s += ok ? dz : 0.0f;
        z[c] = s;
      }
      Pl = P;
      Cl = ct;
    }
    // the level below slot 0: the lane below's last slot, or the carry
    float Pm = __shfl_up_sync(FULL, Pl, 1, SEG), Cm = __shfl_up_sync(FULL, Cl, 1, SEG);
    float um = __shfl_up_sync(FULL, u[RUN - 1], 1, SEG);
    float vm = __shfl_up_sync(FULL, v[RUN - 1], 1, SEG);
    if (sl == 0) {
      Pm = Pc;
      Cm = Cc;
      um = uc;
      vm = vc;
    }
    float dz0 = (Cf + Cm) * lg2_a(Pm * rcp_a(Pf));
    mono = mono && (lo != 0 || dz0 > 0.0f);
    dz0 = lo == 0 ? dz0 : 0.0f;
    // heights: the exclusive scan of the lanes' run totals; slots below the
    // lane's first level keep the height of the level below it
    const float tot = dz0 + s;
    float x = tot;
#pragma unroll
    for (int d = 1; d < SEG; d <<= 1) {
      const float y = __shfl_up_sync(FULL, x, d, SEG);
      if (sl >= d) x += y;
    }
    float ex = __shfl_up_sync(FULL, x, 1, SEG);
    if (sl == 0) ex = 0.0f;
    const float below = Hc + ex;  // height of the level below the lane's first level
    const float b0 = below + dz0;
    z[0] = b0;
#pragma unroll
    for (int c = 1; c < RUN; ++c) z[c] = b0 + z[c];
    // Bunkers targets of each layer (empty for the slots below the lane's
    // first level), and the slots at or below depth
    int ka = seg_below(below);
    int nle = 0;
    float za = below, ua = um, va = vm;
#pragma unroll
    for (int c = 0; c < RUN; ++c) {
      const float zb = z[c];
      const int kb = seg_below(zb);
      for (int k = ka; k < kb; ++k) {
        const float w = (500.0f * (float)(k + 1) - za) * rcp_a(zb - za);
        slot_u[cb][k] = fmaf(w, u[c] - ua, ua);
        slot_v[cb][k] = fmaf(w, v[c] - va, va);
      }
      nle += zb <= depth ? 1 : 0;
      ka = kb;
      za = zb;
      ua = u[c];
      va = v[c];
    }
    // the lane holding the first level above depth (the lowest such lane in
    // the first round that has one) and, in it, that level's slot; with
    // increasing heights it follows the slots at or below depth, and the
    // slots below the lane's first level count as such when the level
    // below it does
    const bool crosses = valid != 0 && z[RUN - 1] > depth;
    const unsigned cm = __ballot_sync(FULL, ktop == 0 && crosses) & seg_mask;
    const int fl = cm ? (__ffs(cm) - 1) & (SEG - 1) : SEG;
    const int t = min(max(nle, lo), RUN - 1);
    const int hi = (ktop != 0 || sl > fl) ? 0 : (sl < fl ? RUN : t);
    const unsigned incl = valid & ((1u << hi) - 1);  // slots whose helicity terms this lane adds
    const bool top = ktop == 0 && sl == fl;
    float zl = below, zh = 0.0f;
    ua = um;
    va = vm;
#pragma unroll
    for (int c = 0; c < RUN; ++c) {
      if ((incl >> c) & 1u) A = fmaf(ua, v[c], fmaf(-u[c], va, A));
      if (c == t - 1) zl = z[c];
      if (c == t) zh = z[c];
      ua = u[c];
      va = v[c];
    }
    if (top) {
      // INTERP1 with X1 = aglh(ktop), X3 = aglh(ktop-1): X3 < X1 for
      // increasing heights, so its X3 == X1 adjustment never applies here.
      // The winds of the two levels are read again (from L1).
      const float uh = wu[t], vh = wv[t];
      const float ul = t > 0 ? wu[t - 1] : um, vl = t > 0 ? wv[t - 1] : vm;
      const float w = (depth - zh) * rcp_a(zl - zh);
      utop = fmaf(ul - uh, w, uh);
      vtop = fmaf(vl - vh, w, vh);
      A = fmaf(ul, vtop, fmaf(-utop, vl, A));
    }
    if (cm) ktop = 1;  // found (its index itself is not needed)
    // the round's last level, for the next round's first lane
    Pc = __shfl_sync(FULL, Pl, SEG - 1, SEG);
    Cc = __shfl_sync(FULL, Cl, SEG - 1, SEG);
    uc = __shfl_sync(FULL, u[RUN - 1], SEG - 1, SEG);
    vc = __shfl_sync(FULL, v[RUN - 1], SEG - 1, SEG);
    Hc = __shfl_sync(FULL, z[RUN - 1], SEG - 1, SEG);
  }
  seg_finish<GRID>(a, i, active, mono, ktop, A, utop, vtop, us, vs, slot_u[cb], slot_v[cb]);
}

namespace {

constexpr long long SEG_COLS = SEG_THREADS / SEG;  // columns per block
constexpr size_t SEG_STAGE_MAX = 46 * 1024;        // staged rows per block, bytes

// The staged kernel's shared memory for nk levels (0: it does not fit).
size_t seg_stage_bytes(int grid, int nk) {
  const size_t b = (size_t)(grid == 1 ? 5 : 4) * SEG_COLS * nk * sizeof(float);
  return b <= SEG_STAGE_MAX ? b : 0;
}

bool aligned16(const void *p) { return ((uintptr_t)p & 15) == 0; }

// Which columns share a warp in the staged kernel: the assignment whose
// first round of shared-memory reads (a column starting at its first level)
// has the fewer bank conflicts, counted as the sum over the warps' loads of
// the largest number of lanes on one bank.  With 50 levels, columns four
// apart start 200 floats apart, 8 banks, and the 32 lanes of a load fall in
// 32 banks.
int seg_colmap_for(int nk, int run) {
  int cost[2] = {0, 0};
  for (int map = 0; map < 2; ++map)
    for (int w = 0; w < 4; ++w)
      for (int c = 0; c < run; ++c) {
        int cnt[32] = {0}, mx = 0;
        for (int lane = 0; lane < 32; ++lane) {
          const int seg = 4 * w + lane / SEG, sl = lane % SEG;
          const int cb = map ? ((seg & 3) << 2) | (seg >> 2) : seg;
          const int ws = sl * run < nk - run ? sl * run : nk - run;
          const int k = ++cnt[(cb * nk + ws + c) & 31];
          mx = k > mx ? k : mx;
        }
        cost[map] += mx;
      }
  return cost[1] < cost[0] ? 1 : 0;
}

template <int GRID, int RUN>
cudaError_t launch_seg(const SrhArgs &a0, cudaStream_t s) {
  SrhArgs a = a0;
  a.seg_colmap = seg_colmap_for(a.nk, RUN);
  const size_t stage = seg_stage_bytes(GRID, a.nk);
  const bool staged = stage > 0 && aligned16(a.t) && aligned16(a.td) && aligned16(a.u) &&
                      aligned16(a.v) && (GRID == 2 || aligned16(a.p));
  const long long full = staged ? a.n2 / SEG_COLS : 0;  // blocks the staged kernel takes
  if (full > 0) {
    srh_seg_kernel<GRID, RUN, true><<<(unsigned)full, SEG_THREADS, stage, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  const long long c0 = full * SEG_COLS;  // the remaining columns: the direct kernel
  if (c0 >= a.n2) return cudaSuccess;
  SrhArgs t = a;
  if (c0 > 0) {
    const size_t nk = (size_t)a.nk;
    t.n2 = a.n2 - c0;
    if (GRID == 1) t.p = (const float *)a.p + c0 * nk;
    t.t = (const float *)a.t + c0 * nk;
    t.td = (const float *)a.td + c0 * nk;
    t.u = (const float *)a.u + c0 * nk;
    t.v = (const float *)a.v + c0 * nk;
    t.ps = (const float *)a.ps + c0;
    t.ts = (const float *)a.ts + c0;
    t.tds = (const float *)a.tds + c0;
    t.us = (const float *)a.us + c0;
    t.vs = (const float *)a.vs + c0;
    if (a.start) t.start = a.start + c0;
    t.srh_rm = a.srh_rm + c0;
    t.srh_lm = a.srh_lm + c0;
    if (a.rm) {
      t.rm = a.rm + 2 * c0;
      t.lm = a.lm + 2 * c0;
      t.mean6 = a.mean6 + 2 * c0;
    }
  }
  const unsigned blocks = (unsigned)((t.n2 + SEG_COLS - 1) / SEG_COLS);
  srh_seg_kernel<GRID, RUN, false><<<blocks, SEG_THREADS, 0, s>>>(t);
  return cudaGetLastError();
}

template <int GRID>
cudaError_t launch_seg_g(const SrhArgs &a, int run, cudaStream_t s) {
  switch (run) {
    case 5: return launch_seg<GRID, 5>(a, s);
    case 6: return launch_seg<GRID, 6>(a, s);
    case 7: return launch_seg<GRID, 7>(a, s);
    default: return launch_seg<GRID, 8>(a, s);
  }
}

}  // namespace

// The run length for columns of nk input levels: the fewest level slots
// rounds * RUN over RUN = 5..min(8, nk), the longer run on a tie (fewer
// rounds); 0 (the column kernel serves) below 5 levels.  50 levels take one
// round of 8 x 7, 37 one of 8 x 5, 137 three of 8 x 6.
int srh_seg_run(int levels) {
  if (levels < 5) return 0;
  int best = 5, best_slots = 1 << 30;
  for (int run = levels < 8 ? levels : 8; run >= 5; --run) {
    const int rounds = (levels + SEG * run - 1) / (SEG * run);
    if (rounds * run < best_slots) {
      best = run;
      best_slots = rounds * run;
    }
  }
  return best;
}

cudaError_t launch_srh_seg(const SrhArgs &a, cudaStream_t s) {
  const int run = srh_seg_run(a.nk);
  if (run == 0) return cudaErrorInvalidValue;  // the caller checks srh_seg_run first
  if (a.n2 <= 0) return cudaSuccess;
  return a.grid == 1 ? launch_seg_g<1>(a, run, s) : launch_seg_g<2>(a, run, s);
}

}  // namespace xc
