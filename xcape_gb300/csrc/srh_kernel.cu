// srh_kernel.cu -- storm-relative helicity kernels for sm_103a: one thread per
// column running the column routines of srh_column.cuh (the fused
// stdheight -> Bunkers -> SREH path and the three stage loops on their own).
#include <stdint.h>

#include "srh_column.cuh"
#include "xc_kernels.h"

namespace xc {

template <typename T, int GRID, bool F32>
__global__ void __launch_bounds__(128) srh_fused_kernel(SrhArgs a) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.n2) srh_column_run<T, GRID, F32>(a, i);
}

__global__ void stdheight_kernel(const double *P, long long p_stride, const double *T,
                                 const double *Td, const double *Ps, const double *Ts,
                                 const double *Tds, const double *Hin, const int *start, int NK,
                                 long long NX, double *H, double *Hs) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < NX) stdheight_column_run(P, p_stride, T, Td, Ps, Ts, Tds, Hin, start, NK, i, H, Hs);
}

__global__ void bunkers_kernel(const float *U, const float *V, const float *Z, const float *Us,
                               const float *Vs, const float *Zs, const int *start, int nk,
                               long long n2, float *RM, float *LM, float *Mean) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2) bunkers_column_run(U, V, Z, Us, Vs, Zs, start, nk, i, RM, LM, Mean);
}

__global__ void sreh_kernel(const double *u, const double *v, const double *aglh,
                            const double *us, const double *vs, const double *aglhs,
                            const double *cu_rm, const double *cv_rm, const double *cu_lm,
                            const double *cv_lm, double top, const int *start, int nk,
                            long long n2, double *sreh_rm, double *sreh_lm) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n2)
    sreh_column_run(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top, start, nk, i,
                    sreh_rm, sreh_lm);
}

// FP32 path for float inputs with the column tile staged in shared memory.
// One warp per block takes 32 consecutive columns, whose rows (nk levels
// each) are one contiguous range of every input array.  The warp first walks
// that range together -- every load a full, coalesced line, 16 bytes per lane
// where the arrays are 16-byte aligned -- computing the virtual temperature
// of each (column, level) element as it goes, and stores the rows of p
// (sigma grids), Tv, u and v in shared memory with an odd row stride S
// (lanes then read the same level of their own rows in distinct banks).
// Each lane then runs passes 1 and 2 of its column from those rows
// (srh_column_body, the code of the FP32 column path).  Without staging,
// each lane walks its own 200-byte row through the cache, a warp's level
// load touches 32 lines, and the lines leave L1 before their next levels are
// read: the kernel fetched 5.4x its algorithmic bytes.
constexpr int SRH_TILE = 32;

__host__ __device__ inline int srh_tile_stride(int nk) { return nk | 1; }

inline size_t srh_tile_smem(int grid, int nk) {
  const size_t S = (size_t)srh_tile_stride(nk);
  return sizeof(float) * (grid == 1 ? 4 * SRH_TILE * S : 3 * SRH_TILE * S + (size_t)nk);
}
constexpr size_t SRH_TILE_SMEM_MAX = 200 * 1024;

template <int GRID>
__device__ __forceinline__ void srh_stage(float *TV, float *U, float *V, float *P, int S, int nk,
                                          int e, float p, float t, float td, float u, float v) {
  const int c = e / nk, m = e - c * nk;
  if (GRID == 1) P[c * S + m] = p;
  else p = P[m];
  TV[c * S + m] = stdh_tv_f(p, t, td);
  U[c * S + m] = u;
  V[c * S + m] = v;
}

template <int GRID>
__global__ void __launch_bounds__(SRH_TILE) srh_tile_kernel(SrhArgs a) {
  extern __shared__ __align__(16) float sm[];
  const int nk = a.nk, S = srh_tile_stride(nk);
  float *TV = sm, *U = TV + SRH_TILE * S, *V = U + SRH_TILE * S, *P = V + SRH_TILE * S;
  const long long i0 = (long long)blockIdx.x * SRH_TILE;
  const int lane = threadIdx.x;
  const int ncols = (int)min((long long)SRH_TILE, a.n2 - i0);
  const long long e0 = i0 * nk;
  const int ne = ncols * nk;
  const float *gp = (const float *)a.p, *gt = (const float *)a.t, *gtd = (const float *)a.td;
  const float *gu = (const float *)a.u, *gv = (const float *)a.v;
  if (GRID == 2) {
    for (int m = lane; m < nk; m += 32) P[m] = __ldg(gp + m);
    __syncwarp();
  } else {
    gp += e0;
  }
  gt += e0;
  gtd += e0;
  gu += e0;
  gv += e0;
  const bool vec = ((((uintptr_t)gt | (uintptr_t)gtd | (uintptr_t)gu | (uintptr_t)gv |
                      (GRID == 1 ? (uintptr_t)gp : 0)) & 15) == 0);
  int done = 0;
  if (vec) {
    const int nq = ne >> 2;
#pragma unroll 2
    for (int q = lane; q < nq; q += 32) {
      const float4 t4 = __ldg(reinterpret_cast<const float4 *>(gt) + q);
      const float4 d4 = __ldg(reinterpret_cast<const float4 *>(gtd) + q);
      const float4 u4 = __ldg(reinterpret_cast<const float4 *>(gu) + q);
      const float4 v4 = __ldg(reinterpret_cast<const float4 *>(gv) + q);
      float4 p4 = make_float4(0.f, 0.f, 0.f, 0.f);
      if (GRID == 1) p4 = __ldg(reinterpret_cast<const float4 *>(gp) + q);
      const int e = 4 * q;
      srh_stage<GRID>(TV, U, V, P, S, nk, e, p4.x, t4.x, d4.x, u4.x, v4.x);
      srh_stage<GRID>(TV, U, V, P, S, nk, e + 1, p4.y, t4.y, d4.y, u4.y, v4.y);
      srh_stage<GRID>(TV, U, V, P, S, nk, e + 2, p4.z, t4.z, d4.z, u4.z, v4.z);
      srh_stage<GRID>(TV, U, V, P, S, nk, e + 3, p4.w, t4.w, d4.w, u4.w, v4.w);
    }
    done = nq << 2;
  }
  for (int e = done + lane; e < ne; e += 32)
    srh_stage<GRID>(TV, U, V, P, S, nk, e, GRID == 1 ? __ldg(gp + e) : 0.0f, __ldg(gt + e),
                    __ldg(gtd + e), __ldg(gu + e), __ldg(gv + e));
  __syncwarp();
  if (lane >= ncols) return;
  const long long i = i0 + lane;
  SrhSurface sf;
  sf.ps = ldd((const float *)a.ps + i);
  sf.ts = ldd((const float *)a.ts + i);
  sf.tds = ldd((const float *)a.tds + i);
  sf.us = ldd((const float *)a.us + i);
  sf.vs = ldd((const float *)a.vs + i);
  int st = 1;
  if (GRID == 2) {
    st = a.start ? __ldg(a.start + i)
                 : pres_lev_pos_col<float>((const float *)a.p, __ldg((const float *)a.ps + i), nk);
    st = st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
  }
  sf.base = st - 3;
  SharedLevels lv;
  lv.P = GRID == 1 ? P + lane * S : P;
  lv.TV = TV + lane * S;
  lv.U = U + lane * S;
  lv.V = V + lane * S;
  srh_column_body<true>(a, i, lv, sf, nk - st + 2);
}

// FP32 path for float inputs, level-parallel: a segment of SRH_SEG lanes
// sweeps one column in rounds of SRH_SEG * SRH_RUN levels, lane l taking the
// run of SRH_RUN consecutive levels j = j0 + SRH_RUN l .. of the round.
// Each lane reads its run of every input row (the warp's loads cover four
// columns' rows, and the run's sectors stay in L1 between its levels: no
// shared-memory staging), so a column's dependent chain is SRH_RUN levels
// long instead of ncl, and the lanes talk only once per round:
//   * phase 1, per lane: the virtual temperature of each level of the run
//     and its hypsometric increment (the level below the run's first comes
//     from the lane below by shuffle, or from the previous round);
//   * the heights: each lane's running sum of its increments on top of the
//     segment's exclusive scan of the lanes' totals and of the previous
//     round's last height;
//   * phase 2, per lane: a level whose layer [H(j-1), H(j)) holds a Bunkers
//     target height interpolates the winds there (DINTERP2DZ's weights) into
//     the column's target slots in shared memory; the first level above
//     `depth` (the lowest lane's first such level, in the first round that
//     has one) interpolates the winds at `depth` (INTERP1); every level up
//     to it adds its term of the helicity sums' storm-motion free part
//     A = sum(u_k dv_k - v_k du_k).
// The sums over k = 2..ktop of (u_k - c_u) dv_k - (v_k - c_v) du_k then
// follow for both storm motions: A - c_u (v_top - v_s) + c_v (u_top - u_s),
// since dv and du telescope.  This needs heights that increase with level:
// each target then falls in exactly one layer, the highest bracket
// DINTERP2DZ keeps.  A column whose heights do not increase (a non-finite
// input, pressures that are not decreasing) is redone by its segment's
// first lane with the one-thread column routine of the FP32 path
// (srh_column_run), which follows the reference's scan rules for any
// column.  Its contract is the FP32 path's: agreement with the FP64
// reference within tolerance.
constexpr int SRH_SEG = 8;
constexpr int SRH_RUN = 8;
constexpr int SRH_SEG_THREADS = 128;

template <int GRID>
__global__ void __launch_bounds__(SRH_SEG_THREADS) srh_seg_kernel(SrhArgs a) {
  constexpr unsigned FULL = 0xffffffffu;
  constexpr int COLS = SRH_SEG_THREADS / SRH_SEG;  // columns per block
  __shared__ float slot_u[COLS][12], slot_v[COLS][12];
  const int lane = threadIdx.x & 31;
  const int sl = lane & (SRH_SEG - 1);
  const unsigned seg_mask = 0xffu << (lane & ~(SRH_SEG - 1));
  const int cb = threadIdx.x / SRH_SEG;  // column within the block
  const long long i = (long long)blockIdx.x * COLS + cb;
  const bool active = i < a.n2;
  const int nk = a.nk;
  const float *gp = (const float *)a.p, *gt = (const float *)a.t, *gtd = (const float *)a.td;
  const float *gu = (const float *)a.u, *gv = (const float *)a.v;
  // the column's surface and level window
  float ps = 1000.0f, ts = 0.0f, tds = 0.0f, us = 0.0f, vs = 0.0f;
  int st = 1, ncl = 1;
  long long row = 0;
  if (active) {
    ps = __ldg((const float *)a.ps + i);
    ts = __ldg((const float *)a.ts + i);
    tds = __ldg((const float *)a.tds + i);
    us = __ldg((const float *)a.us + i);
    vs = __ldg((const float *)a.vs + i);
    if (GRID == 2) {
      st = a.start ? __ldg(a.start + i) : pres_lev_pos_col<float>(gp, ps, nk);
      st = st < 1 ? 1 : (st > nk + 1 ? nk + 1 : st);
    }
    ncl = nk - st + 2;
    row = i * nk;
  }
  const int base = st - 3;  // 0-based input index of assembled level j: base + j
  for (int k = sl; k < 24; k += SRH_SEG) {
    if (k < 12) slot_u[cb][k] = VMSG;
    else slot_v[cb][k - 12] = VMSG;
  }
  __syncwarp();
  const float depth = (float)a.depth, aglh0 = (float)a.aglh0;
  // the level below the round's first level: the surface to begin with
  float Pc = ps, Tvc = stdh_tv_f(ps, ts, tds), uc = us, vc = vs, Hc = aglh0;
  bool mono = true;
  int ktop = 0;
  float utop = 0.0f, vtop = 0.0f, A = 0.0f;
  constexpr int ROUND = SRH_SEG * SRH_RUN;
  const int nrounds = active ? (ncl - 1 + ROUND - 1) / ROUND : 0;
  const int wrounds = __reduce_max_sync(FULL, nrounds);
  for (int r = 0; r < wrounds; ++r) {
    const int j0 = 2 + r * ROUND + sl * SRH_RUN;  // this lane's first level
    float P[SRH_RUN], Tv[SRH_RUN], u[SRH_RUN], v[SRH_RUN], h[SRH_RUN];
    int nv = r < nrounds ? ncl - j0 + 1 : 0;  // valid levels of the run
    nv = nv < 0 ? 0 : (nv > SRH_RUN ? SRH_RUN : nv);
#pragma unroll
    for (int c = 0; c < SRH_RUN; ++c) {
      P[c] = 1.0f;
      Tv[c] = 0.0f;
      u[c] = 0.0f;
      v[c] = 0.0f;
      if (c < nv) {
        const int m = base + j0 + c;
        P[c] = __ldg(GRID == 2 ? gp + m : gp + row + m);
        const float T = __ldg(gt + row + m), Td = __ldg(gtd + row + m);
        u[c] = __ldg(gu + row + m);
        v[c] = __ldg(gv + row + m);
        Tv[c] = stdh_tv_f(P[c], T, Td);
      }
    }
    // the level below the run: the lane below's last level, or the carry
    const float Pl = P[SRH_RUN - 1], Tvl = Tv[SRH_RUN - 1], ul = u[SRH_RUN - 1], vl = v[SRH_RUN - 1];
    float Pm = __shfl_up_sync(FULL, Pl, 1, SRH_SEG), Tvm = __shfl_up_sync(FULL, Tvl, 1, SRH_SEG);
    float um = __shfl_up_sync(FULL, ul, 1, SRH_SEG), vm = __shfl_up_sync(FULL, vl, 1, SRH_SEG);
    if (sl == 0) {
      Pm = Pc;
      Tvm = Tvc;
      um = uc;
      vm = vc;
    }
    // increments and the run's running sum
    float run = 0.0f;
#pragma unroll
    for (int c = 0; c < SRH_RUN; ++c) {
      float dh = 0.0f;
      if (c < nv) {
        dh = stdh_dh_f(Tv[c], c == 0 ? Tvm : Tv[c - 1], P[c], c == 0 ? Pm : P[c - 1]);
        mono = mono && dh > 0.0f;
      }
      run += dh;
      h[c] = run;
    }
    // heights: the exclusive scan of the lanes' run totals
    float x = run;
#pragma unroll
    for (int d = 1; d < SRH_SEG; d <<= 1) {
      const float y = __shfl_up_sync(FULL, x, d, SRH_SEG);
      if (sl >= d) x += y;
    }
    const float below = Hc + (x - run);  // height of the level below the run
    // phase 2: Bunkers targets, the SREH top and the helicity terms
    float hp = below, up = um, vp = vm;
    int first = SRH_RUN;  // this lane's first level above depth
#pragma unroll
    for (int c = 0; c < SRH_RUN; ++c) {
      const float H = below + h[c];
      h[c] = H;
      if (c < nv) {
        if (mono && hp <= 6000.0f)  // no target above 6 km
          bunkers_bracket<false>(hp, H, up, u[c], vp, v[c], slot_u[cb], slot_v[cb]);
        if (first == SRH_RUN && H > depth) first = c;
      }
      hp = H;
      up = u[c];
      vp = v[c];
    }
    const unsigned cm = __ballot_sync(FULL, ktop == 0 && first < SRH_RUN) & seg_mask;
    const int fl = cm ? (__ffs(cm) - 1) & (SRH_SEG - 1) : SRH_SEG;  // the crossing lane
    if (ktop == 0 && sl <= fl) {
      const int upto = sl < fl ? nv : first;  // levels whose terms this lane adds
      hp = below;
      up = um;
      vp = vm;
#pragma unroll
      for (int c = 0; c < SRH_RUN; ++c) {
        if (c < upto) A += nc_mul(u[c], v[c] - vp) - nc_mul(v[c], u[c] - up);
        if (sl == fl && c == first) {
          // INTERP1 (SREH_model_lev.f90:123-129): X1 = aglh(ktop), X3 = aglh(ktop-1)
          float x1 = h[c];
          const float x3 = hp;
          if (x3 == x1) x1 = x1 - 0.01f;
          utop = u[c] + nc_mul((up - u[c]), ((depth - x1) / (x3 - x1)));
          if (x3 == x1) x1 = x1 - 0.01f;
          vtop = v[c] + nc_mul((vp - v[c]), ((depth - x1) / (x3 - x1)));
          A += nc_mul(utop, vtop - vp) - nc_mul(vtop, utop - up);
        }
        hp = h[c];
        up = u[c];
        vp = v[c];
      }
    }
    if (ktop == 0 && cm) ktop = 1;  // found (its index itself is not needed)
    // the round's last level, for the next round's first lane
    Pc = __shfl_sync(FULL, Pl, SRH_SEG - 1, SRH_SEG);
    Tvc = __shfl_sync(FULL, Tvl, SRH_SEG - 1, SRH_SEG);
    uc = __shfl_sync(FULL, ul, SRH_SEG - 1, SRH_SEG);
    vc = __shfl_sync(FULL, vl, SRH_SEG - 1, SRH_SEG);
    Hc = __shfl_sync(FULL, h[SRH_RUN - 1], SRH_SEG - 1, SRH_SEG);
  }
  // utop and vtop live in the crossing lane: the segment's sums
  float ut = utop, vt = vtop;
#pragma unroll
  for (int d = SRH_SEG / 2; d > 0; d >>= 1) {
    A += __shfl_xor_sync(FULL, A, d, SRH_SEG);
    ut += __shfl_xor_sync(FULL, ut, d, SRH_SEG);
    vt += __shfl_xor_sync(FULL, vt, d, SRH_SEG);
  }
  const bool all_mono = (__ballot_sync(FULL, !mono) & seg_mask) == 0;
  __syncwarp();
  if (!active || sl != 0) return;
  if (!all_mono) {
    srh_column_run<float, GRID, true>(a, i);  // any column, the reference's scan rules
    return;
  }
  float u6[12], v6[12];
  for (int k = 0; k < 12; ++k) {
    u6[k] = slot_u[cb][k];
    v6[k] = slot_v[cb][k];
  }
  float rm[2], lm[2], mean[2];
  bunkers_finish(us, vs, u6, v6, rm, lm, mean);
  double srh_rm = -0.0, srh_lm = -0.0;
  if (ktop > 0) {
    const float dv = vt - vs, du = ut - us;
    srh_rm = -(double)(A - nc_mul(rm[0], dv) + nc_mul(rm[1], du));
    srh_lm = -(double)(A - nc_mul(lm[0], dv) + nc_mul(lm[1], du));
  }
  srh_write(a, i, rm, lm, mean, srh_rm, srh_lm);
}

template <int GRID>
static cudaError_t launch_srh_seg(const SrhArgs &a, cudaStream_t s) {
  const long long cols = SRH_SEG_THREADS / SRH_SEG;
  const unsigned blocks = (unsigned)((a.n2 + cols - 1) / cols);
  srh_seg_kernel<GRID><<<blocks, SRH_SEG_THREADS, 0, s>>>(a);
  return cudaGetLastError();
}

template <int GRID>
static cudaError_t launch_srh_tile(const SrhArgs &a, size_t smem, cudaStream_t s) {
  static std::atomic<int> attr[kMaxAttrDevices];
  const cudaError_t e =
      smem_attr_once((const void *)srh_tile_kernel<GRID>, (int)SRH_TILE_SMEM_MAX, attr);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)((a.n2 + SRH_TILE - 1) / SRH_TILE);
  srh_tile_kernel<GRID><<<blocks, SRH_TILE, smem, s>>>(a);
  return cudaGetLastError();
}

static unsigned blocks_for(long long n, int threads) {
  return (unsigned)((n + threads - 1) / threads);
}

template <bool F32>
static void launch_srh_p(const SrhArgs &a, unsigned blocks, cudaStream_t s) {
  if (a.dtype == 0) {
    if (a.grid == 1)
      srh_fused_kernel<float, 1, F32><<<blocks, 128, 0, s>>>(a);
    else
      srh_fused_kernel<float, 2, F32><<<blocks, 128, 0, s>>>(a);
  } else {
    if (a.grid == 1)
      srh_fused_kernel<double, 1, F32><<<blocks, 128, 0, s>>>(a);
    else
      srh_fused_kernel<double, 2, F32><<<blocks, 128, 0, s>>>(a);
  }
}

cudaError_t launch_srh(const SrhArgs &a, cudaStream_t s) {
  const unsigned blocks = blocks_for(a.n2, 128);
  if (blocks == 0) return cudaSuccess;
  if (a.precision == 1 && a.dtype == 0) {
    if (a.srh_kernel == 1) {
      const size_t smem = srh_tile_smem(a.grid, a.nk);
      if (smem <= SRH_TILE_SMEM_MAX)
        return a.grid == 1 ? launch_srh_tile<1>(a, smem, s) : launch_srh_tile<2>(a, smem, s);
    } else {
      return a.grid == 1 ? launch_srh_seg<1>(a, s) : launch_srh_seg<2>(a, s);
    }
  }
  if (a.precision == 1)
    launch_srh_p<true>(a, blocks, s);
  else
    launch_srh_p<false>(a, blocks, s);
  return cudaGetLastError();
}

cudaError_t launch_stdheight(const double *P, long long p_stride, const double *T,
                             const double *Td, const double *Ps, const double *Ts,
                             const double *Tds, const double *Hin, const int *start, int NK,
                             long long NX, double *H, double *Hs, cudaStream_t s) {
  const unsigned blocks = blocks_for(NX, 128);
  if (blocks == 0) return cudaSuccess;
  stdheight_kernel<<<blocks, 128, 0, s>>>(P, p_stride, T, Td, Ps, Ts, Tds, Hin, start, NK, NX,
                                          H, Hs);
  return cudaGetLastError();
}

cudaError_t launch_bunkers(const float *U, const float *V, const float *Z, const float *Us,
                           const float *Vs, const float *Zs, const int *start, int nk,
                           long long n2, float *RM, float *LM, float *Mean, cudaStream_t s) {
  const unsigned blocks = blocks_for(n2, 128);
  if (blocks == 0) return cudaSuccess;
  bunkers_kernel<<<blocks, 128, 0, s>>>(U, V, Z, Us, Vs, Zs, start, nk, n2, RM, LM, Mean);
  return cudaGetLastError();
}

cudaError_t launch_sreh(const double *u, const double *v, const double *aglh, const double *us,
                        const double *vs, const double *aglhs, const double *cu_rm,
                        const double *cv_rm, const double *cu_lm, const double *cv_lm,
                        double top, const int *start, int nk, long long n2, double *sreh_rm,
                        double *sreh_lm, cudaStream_t s) {
  const unsigned blocks = blocks_for(n2, 128);
  if (blocks == 0) return cudaSuccess;
  sreh_kernel<<<blocks, 128, 0, s>>>(u, v, aglh, us, vs, aglhs, cu_rm, cv_rm, cu_lm, cv_lm, top,
                                     start, nk, n2, sreh_rm, sreh_lm);
  return cudaGetLastError();
}

}  // namespace xc
