// guess_mlp.cu -- data, training and batched inference of the learned first
// guess (guess_mlp.cuh), all on the GPU.
//
// * guess_pairs_kernel draws saturated parcel states over the four adiabats
//   and solves one sub-step of each with the plain solver (guess_pair in
//   cape_column.cuh), storing (features, normalised increment, iterations).
// * guess_train_kernel runs forward and backward passes over a batch, with
//   the three 64-wide products on the tensor cores -- mma.sync m16n8k16, BF16
//   operands, FP32 accumulation:
//     forward   Z2 = H1 W2^T                 (samples x 64, K = 64)
//     backward  dW2 += dZ2^T H1               (64 x 64, K = the samples)
//               dH1 = dZ2 W2                  (samples x 64, K = 64)
//   and the rest (the 3-wide first layer, the output layer, the ReLU masks,
//   the bias and first-layer gradients) in FP32 on the CUDA cores.  Each
//   block keeps its share of the gradient in registers over the tiles of
//   samples it processes and adds it to the global gradient once.
// * guess_adam_kernel applies Adam to the FP32 master weights.
// * guess_eval_kernel is the batched inference (the same tensor-core
//   forward pass).
#include <cuda_bf16.h>
#include <stdint.h>

#include "cape_column.cuh"
#include "guess_mlp.cuh"
#include "tc05.cuh"
#include "xc_kernels.h"

namespace xc {

namespace {

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const uint32_t (&a)[4],
                                               const uint32_t (&b)[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int TB = 128;          // samples per tile = threads per block
constexpr int HP = GUESS_H + 1;  // padded row of the activation tiles

struct TrainSmem {
  float w[GUESS_NPARAM + 3];
  __nv_bfloat16 w2bf[GUESS_H * GUESS_H];  // W2 [n][k]: B of the forward product
  __nv_bfloat16 w2t[GUESS_H * GUESS_H];   // W2^T [k][n]: B of dH1 = dZ2 W2
  float h1[TB * HP];  // H1, later dZ1
  float z2[TB * HP];  // Z2, later dZ2
  float x[TB * 3];
  float dy[TB];
};

// Layer 2 on the tensor cores: warp w computes Z2 rows [32w, 32w + 32) =
// H1 (bf16) x W2^T (bf16), FP32 accumulation, into s.z2 (without b2).
__device__ void layer2_mma(TrainSmem &s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  for (int mt = 0; mt < 2; ++mt) {
    const int r = warp * 32 + mt * 16 + gid;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[nt][j] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int c = ks * 16 + tig * 2;
      uint32_t a[4];
      a[0] = pack_bf16x2(s.h1[r * HP + c], s.h1[r * HP + c + 1]);
      a[1] = pack_bf16x2(s.h1[(r + 8) * HP + c], s.h1[(r + 8) * HP + c + 1]);
      a[2] = pack_bf16x2(s.h1[r * HP + c + 8], s.h1[r * HP + c + 9]);
      a[3] = pack_bf16x2(s.h1[(r + 8) * HP + c + 8], s.h1[(r + 8) * HP + c + 9]);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const int n = nt * 8 + gid;
        uint32_t b[2];
        b[0] = *reinterpret_cast<const uint32_t *>(&s.w2bf[n * GUESS_H + c]);
        b[1] = *reinterpret_cast<const uint32_t *>(&s.w2bf[n * GUESS_H + c + 8]);
        mma_bf16_16816(acc[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + tig * 2;
      s.z2[r * HP + col] = acc[nt][0];
      s.z2[r * HP + col + 1] = acc[nt][1];
      s.z2[(r + 8) * HP + col] = acc[nt][2];
      s.z2[(r + 8) * HP + col + 1] = acc[nt][3];
    }
  }
}

// The block's weights in shared memory: FP32 master copy and the two BF16
// operand images of W2.
__device__ void load_weights(TrainSmem &s, const float *weights) {
  for (int i = threadIdx.x; i < GUESS_NPARAM; i += TB) s.w[i] = weights[i];
  for (int i = threadIdx.x; i < GUESS_H * GUESS_H; i += TB) {
    const float v = weights[GUESS_OFF_W2 + i];
    s.w2bf[i] = __float2bfloat16_rn(v);
    s.w2t[(i % GUESS_H) * GUESS_H + i / GUESS_H] = __float2bfloat16_rn(v);
  }
}

// The tile's features (rows beyond n are zero samples), layer 1 (FP32) and
// layer 2 (tensor cores).  The weights must be loaded.
__device__ void forward_hidden(TrainSmem &s, const float *feats, long long row0, long long n) {
  const int t = threadIdx.x;
  const long long g = row0 + t;
  const bool valid = g < n;
  for (int i = 0; i < 3; ++i) s.x[t * 3 + i] = valid ? feats[g * 3 + i] : 0.0f;
  __syncthreads();
  const float f0 = s.x[t * 3], f1 = s.x[t * 3 + 1], f2 = s.x[t * 3 + 2];
  for (int k = 0; k < GUESS_H; ++k) {
    const float z = s.w[GUESS_OFF_B1 + k] + s.w[GUESS_OFF_W1 + 3 * k] * f0 +
                    s.w[GUESS_OFF_W1 + 3 * k + 1] * f1 + s.w[GUESS_OFF_W1 + 3 * k + 2] * f2;
    s.h1[t * HP + k] = z > 0.0f ? z : 0.0f;
  }
  __syncthreads();
  layer2_mma(s);
  __syncthreads();
}

// dW2 (+)= dZ2^T H1 for the tile on the tensor cores: warp w owns rows
// n = 16w .. 16w + 15 of dW2 and all 64 columns k, K runs over the tile's
// TB samples.  acc[nt][j] is the mma C fragment of columns 8 nt .. 8 nt + 7.
__device__ void dw2_mma(const TrainSmem &s, float (&acc)[8][4]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  const int m = warp * 16 + gid;
#pragma unroll 2
  for (int ks = 0; ks < TB / 16; ++ks) {
    const int s0 = ks * 16 + tig * 2;
    uint32_t a[4];  // A[m][sample] = dZ2[sample][m]
    a[0] = pack_bf16x2(s.z2[s0 * HP + m], s.z2[(s0 + 1) * HP + m]);
    a[1] = pack_bf16x2(s.z2[s0 * HP + m + 8], s.z2[(s0 + 1) * HP + m + 8]);
    a[2] = pack_bf16x2(s.z2[(s0 + 8) * HP + m], s.z2[(s0 + 9) * HP + m]);
    a[3] = pack_bf16x2(s.z2[(s0 + 8) * HP + m + 8], s.z2[(s0 + 9) * HP + m + 8]);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int k = nt * 8 + gid;  // B[sample][k] = H1[sample][k]
      uint32_t b[2];
      b[0] = pack_bf16x2(s.h1[s0 * HP + k], s.h1[(s0 + 1) * HP + k]);
      b[1] = pack_bf16x2(s.h1[(s0 + 8) * HP + k], s.h1[(s0 + 9) * HP + k]);
      mma_bf16_16816(acc[nt], a, b);
    }
  }
}

// dZ1 = (dZ2 W2) * [H1 > 0] on the tensor cores, written over H1: warp w
// owns the samples [32w, 32w + 32), as in layer2_mma.
__device__ void dz1_mma(TrainSmem &s) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gid = lane >> 2, tig = lane & 3;
  for (int mt = 0; mt < 2; ++mt) {
    const int r = warp * 32 + mt * 16 + gid;
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[nt][j] = 0.0f;
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const int c = ks * 16 + tig * 2;  // the n (second-layer unit) index
      uint32_t a[4];
      a[0] = pack_bf16x2(s.z2[r * HP + c], s.z2[r * HP + c + 1]);
      a[1] = pack_bf16x2(s.z2[(r + 8) * HP + c], s.z2[(r + 8) * HP + c + 1]);
      a[2] = pack_bf16x2(s.z2[r * HP + c + 8], s.z2[r * HP + c + 9]);
      a[3] = pack_bf16x2(s.z2[(r + 8) * HP + c + 8], s.z2[(r + 8) * HP + c + 9]);
#pragma unroll
      for (int nt = 0; nt < 8; ++nt) {
        const int k = nt * 8 + gid;  // B[n][k] = W2[n][k], read from W2^T [k][n]
        uint32_t b[2];
        b[0] = *reinterpret_cast<const uint32_t *>(&s.w2t[k * GUESS_H + c]);
        b[1] = *reinterpret_cast<const uint32_t *>(&s.w2t[k * GUESS_H + c + 8]);
        mma_bf16_16816(acc[nt], a, b);
      }
    }
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int col = nt * 8 + tig * 2;
      float *h0 = &s.h1[r * HP + col], *h8 = &s.h1[(r + 8) * HP + col];
      h0[0] = h0[0] > 0.0f ? acc[nt][0] : 0.0f;
      h0[1] = h0[1] > 0.0f ? acc[nt][1] : 0.0f;
      h8[0] = h8[0] > 0.0f ? acc[nt][2] : 0.0f;
      h8[1] = h8[1] > 0.0f ? acc[nt][3] : 0.0f;
    }
  }
}

}  // namespace

__global__ void guess_pairs_kernel(long long n, unsigned long long seed, float *feats,
                                   float *targets, int *iters) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  iters[i] = guess_pair(seed, i, feats + 3 * i, targets + i);
}

// Forward and backward passes of the MSE loss over the batch [batch0,
// batch0 + nb): block b processes the tiles of TB samples b, b + gridDim.x,
// ...; its gradient is kept in registers over its tiles (dW2 as the mma
// accumulators, the rest per thread) and added to grad with one atomicAdd
// per parameter and thread at the end; loss likewise.
__global__ void __launch_bounds__(TB) guess_train_kernel(const float *weights, const float *feats,
                                                         const float *targets, long long batch0,
                                                         long long nb, float *grad,
                                                         float *loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem &s = *reinterpret_cast<TrainSmem *>(smem_raw);
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  const int unit = t & (GUESS_H - 1), half = t / GUESS_H;  // (unit, half of the samples)
  const long long end = batch0 + nb;
  const long long ntiles = (nb + TB - 1) / TB;
  load_weights(s, weights);
  float acc_w2[8][4];
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc_w2[nt][j] = 0.0f;
  float g_w1[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // dW1[unit][0..2], db1[unit]
  float g_b2 = 0.0f, g_w3 = 0.0f, g_b3 = 0.0f, l_sum = 0.0f;
  for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const long long row0 = batch0 + tile * TB;
    forward_hidden(s, feats, row0, end);
    // output layer and loss: thread t owns sample t
    const long long g = row0 + t;
    const bool valid = g < end;
    float y = s.w[GUESS_OFF_B3];
    for (int n = 0; n < GUESS_H; ++n) {
      const float z = s.z2[t * HP + n] + s.w[GUESS_OFF_B2 + n];
      s.z2[t * HP + n] = z;  // the pre-activation
      y += s.w[GUESS_OFF_W3 + n] * (z > 0.0f ? z : 0.0f);
    }
    const float err = valid ? y - targets[g] : 0.0f;
    const float dy = 2.0f * err / (float)nb;
    l_sum += err * err / (float)nb;
    s.dy[t] = dy;
    __syncthreads();
    // dW3[n] += sum_s dy_s relu(z2[s][n]), db3 += sum_s dy_s: thread
    // (unit, half) sums its half of the samples
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) {
      const float z = s.z2[r * HP + unit];
      g_w3 += s.dy[r] * (z > 0.0f ? z : 0.0f);
    }
    if (t == 0)
      for (int r = 0; r < TB; ++r) g_b3 += s.dy[r];
    __syncthreads();
    // dZ2 = dy w3 [z2 > 0], over Z2
    for (int n = 0; n < GUESS_H; ++n) {
      const float z = s.z2[t * HP + n];
      s.z2[t * HP + n] = z > 0.0f ? dy * s.w[GUESS_OFF_W3 + n] : 0.0f;
    }
    __syncthreads();
    dw2_mma(s, acc_w2);
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) g_b2 += s.z2[r * HP + unit];
    __syncthreads();  // every warp is done reading H1 for dW2
    dz1_mma(s);
    __syncthreads();
    // dW1[k][i] += sum_s dZ1[s][k] x[s][i], db1[k] += sum_s dZ1[s][k]
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) {
      const float d = s.h1[r * HP + unit];
      g_w1[0] += d * s.x[r * 3];
      g_w1[1] += d * s.x[r * 3 + 1];
      g_w1[2] += d * s.x[r * 3 + 2];
      g_w1[3] += d;
    }
    __syncthreads();  // before the next tile overwrites x, H1 and Z2
  }
  // the block's gradient into the global one
  const int gid = lane >> 2, tig = lane & 3;
#pragma unroll
  for (int nt = 0; nt < 8; ++nt) {
    const int n = warp * 16 + gid, k = nt * 8 + tig * 2;
    atomicAdd(grad + GUESS_OFF_W2 + n * GUESS_H + k, acc_w2[nt][0]);
    atomicAdd(grad + GUESS_OFF_W2 + n * GUESS_H + k + 1, acc_w2[nt][1]);
    atomicAdd(grad + GUESS_OFF_W2 + (n + 8) * GUESS_H + k, acc_w2[nt][2]);
    atomicAdd(grad + GUESS_OFF_W2 + (n + 8) * GUESS_H + k + 1, acc_w2[nt][3]);
  }
  atomicAdd(grad + GUESS_OFF_W1 + 3 * unit, g_w1[0]);
  atomicAdd(grad + GUESS_OFF_W1 + 3 * unit + 1, g_w1[1]);
  atomicAdd(grad + GUESS_OFF_W1 + 3 * unit + 2, g_w1[2]);
  atomicAdd(grad + GUESS_OFF_B1 + unit, g_w1[3]);
  atomicAdd(grad + GUESS_OFF_B2 + unit, g_b2);
  atomicAdd(grad + GUESS_OFF_W3 + unit, g_w3);
  if (t == 0) atomicAdd(grad + GUESS_OFF_B3, g_b3);
  for (int o = 16; o > 0; o >>= 1) l_sum += __shfl_down_sync(0xffffffffu, l_sum, o);
  if (lane == 0) atomicAdd(loss, l_sum);
}

namespace {

// Shared memory of the tcgen05 training kernel: the BF16 operand tiles in
// the canonical K-major layout of tc05.cuh (each a multiple of 128 bytes,
// so the next starts aligned), then the FP32 tiles of the CUDA-core parts.
struct TcTrainSmem {
  __nv_bfloat16 b_w2[GUESS_H * GUESS_H];   // B of Z2 = H1 W2^T: W2 [n][k], K = 64
  __nv_bfloat16 b_w2t[GUESS_H * GUESS_H];  // B of dH1 = dZ2 W2: W2^T [k][n], K = 64
  __nv_bfloat16 a_h1[TB * GUESS_H];        // A of Z2: H1 [sample][k], K = 64
  __nv_bfloat16 a_dz2[TB * GUESS_H];       // A of dH1: dZ2 [sample][n], K = 64
  __nv_bfloat16 a_dz2t[TB * TB];           // A of dW2: dZ2^T [n][sample], rows 64..127 zero, K = 128
  __nv_bfloat16 b_h1t[GUESS_H * TB];       // B of dW2: H1^T [k][sample], K = 128
  float w[GUESS_NPARAM + 3];
  float h1[TB * HP];  // H1, later dZ1
  float z2[TB * HP];  // Z2 (pre-activation), later dZ2
  float x[TB * 3];
  float dy[TB];
  uint64_t bar;
  uint32_t tmem;
  int failed;
};

constexpr uint32_t TC_COLS = 256;           // TMEM columns: Z2 at 0, dH1 at 64, dW2 at 128
constexpr uint32_t TC_WAIT = 1u << 22;      // mbarrier polls before giving up
constexpr uint32_t TC_ID = tc05::idesc_bf16_f32(TB, GUESS_H);

// Waits for the tensor cores' current phase; a wait that runs out marks the
// block failed.  Followed by a block barrier, so s.failed is then uniform.
__device__ __forceinline__ void tc_wait(TcTrainSmem &s, uint32_t &phase) {
  if (!tc05::mbar_wait(&s.bar, phase, TC_WAIT)) s.failed = 1;
  phase ^= 1u;
  __syncthreads();
  tc05::fence_after_sync();
}

}  // namespace

// guess_train_kernel with the three products on the 5th-generation tensor
// cores: tcgen05.mma (kind::f16, BF16 operands in shared memory, FP32
// accumulators in tensor memory), M = 128 samples per tile:
//   Z2  = H1 W2^T       D at TMEM columns 0..63,   K = 64
//   dH1 = dZ2 W2        D at TMEM columns 64..127, K = 64
//   dW2 += dZ2^T H1     D at TMEM columns 128..191, K = 128 samples; M = 128
//                       with dZ2^T's rows padded by 64 zero rows, and the
//                       accumulator kept in TMEM over all the block's tiles.
// Thread t owns sample t of a tile, which is TMEM lane t: warp w reads lanes
// 32w .. 32w + 31, so each thread reads its own sample's rows of Z2 and dH1.
// One thread issues the MMAs and commits them to an mbarrier that every
// thread waits on, for at most TC_WAIT polls; a wait that runs out sets
// *status (when given) and ends the block's work.  Everything else is as in
// guess_train_kernel.
__global__ void __launch_bounds__(TB) guess_train_tc_kernel(const float *weights,
                                                            const float *feats,
                                                            const float *targets, long long batch0,
                                                            long long nb, float *grad, float *loss,
                                                            int *status) {
  extern __shared__ __align__(128) unsigned char tc_smem_raw[];
  TcTrainSmem &s = *reinterpret_cast<TcTrainSmem *>(tc_smem_raw);
  const int t = threadIdx.x;
  const int lane = t & 31, warp = t >> 5;
  const int unit = t & (GUESS_H - 1), half = t / GUESS_H;
  const long long end = batch0 + nb;
  const long long ntiles = (nb + TB - 1) / TB;
  for (int i = t; i < GUESS_NPARAM; i += TB) s.w[i] = weights[i];
  for (int i = t; i < GUESS_H * GUESS_H; i += TB) {
    const int n = i / GUESS_H, k = i % GUESS_H;
    const __nv_bfloat16 v = __float2bfloat16_rn(weights[GUESS_OFF_W2 + i]);
    s.b_w2[tc05::canon(n, k, GUESS_H)] = v;
    s.b_w2t[tc05::canon(k, n, GUESS_H)] = v;
  }
  for (int i = t; i < GUESS_H * TB; i += TB)  // rows 64..127 of dZ2^T
    s.a_dz2t[GUESS_H * TB + i] = __float2bfloat16_rn(0.0f);
  if (t == 0) {
    tc05::mbar_init(&s.bar, 1);
    s.failed = 0;
  }
  if (warp == 0) tc05::tmem_alloc(&s.tmem, TC_COLS);
  tc05::fence_smem_async();
  tc05::fence_before_sync();
  __syncthreads();
  tc05::fence_after_sync();
  const uint32_t tm = s.tmem;
  const uint32_t d_z2 = tm, d_dh1 = tm + 64, d_dw2 = tm + 128;
  const uint32_t my_lanes = (uint32_t)(warp * 32) << 16;  // this warp's TMEM lanes
  uint32_t phase = 0;
  bool any = false;  // the block has accumulated dW2 in TMEM
  float g_w1[4] = {0.0f, 0.0f, 0.0f, 0.0f};  // dW1[unit][0..2], db1[unit]
  float g_b2 = 0.0f, g_w3 = 0.0f, g_b3 = 0.0f, l_sum = 0.0f;
  for (long long tile = blockIdx.x; tile < ntiles && !s.failed; tile += gridDim.x) {
    const long long row0 = batch0 + tile * TB;
    const long long g = row0 + t;
    const bool valid = g < end;
    // layer 1 (FP32) of sample t; H1 into the FP32 tile and the two BF16 operands
    const float f0 = valid ? feats[g * 3] : 0.0f, f1 = valid ? feats[g * 3 + 1] : 0.0f,
                f2 = valid ? feats[g * 3 + 2] : 0.0f;
    s.x[t * 3] = f0;
    s.x[t * 3 + 1] = f1;
    s.x[t * 3 + 2] = f2;
    for (int k = 0; k < GUESS_H; ++k) {
      const float z = s.w[GUESS_OFF_B1 + k] + s.w[GUESS_OFF_W1 + 3 * k] * f0 +
                      s.w[GUESS_OFF_W1 + 3 * k + 1] * f1 + s.w[GUESS_OFF_W1 + 3 * k + 2] * f2;
      const float h = z > 0.0f ? z : 0.0f;
      const __nv_bfloat16 hb = __float2bfloat16_rn(h);
      s.h1[t * HP + k] = h;
      s.a_h1[tc05::canon(t, k, GUESS_H)] = hb;
      s.b_h1t[tc05::canon(k, t, TB)] = hb;
    }
    tc05::fence_smem_async();
    tc05::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc05::fence_after_sync();
      for (int ks = 0; ks < GUESS_H / 16; ++ks)
        tc05::mma_bf16(d_z2, tc05::sdesc(s.a_h1 + ks * 128, 128, 1024),
                       tc05::sdesc(s.b_w2 + ks * 128, 128, 1024), TC_ID, ks > 0);
      tc05::commit(&s.bar);
    }
    tc_wait(s, phase);
    if (s.failed) break;
    // output layer and loss: sample t's row of Z2
    float y = s.w[GUESS_OFF_B3];
    for (int c = 0; c < GUESS_H / 16; ++c) {
      float v[16];
      tc05::tmem_ld16(d_z2 + my_lanes + 16 * c, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        const int n = 16 * c + j;
        const float z = v[j] + s.w[GUESS_OFF_B2 + n];
        s.z2[t * HP + n] = z;
        y += s.w[GUESS_OFF_W3 + n] * (z > 0.0f ? z : 0.0f);
      }
    }
    const float err = valid ? y - targets[g] : 0.0f;
    const float dy = 2.0f * err / (float)nb;
    l_sum += err * err / (float)nb;
    s.dy[t] = dy;
    __syncthreads();
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) {
      const float z = s.z2[r * HP + unit];
      g_w3 += s.dy[r] * (z > 0.0f ? z : 0.0f);
    }
    if (t == 0)
      for (int r = 0; r < TB; ++r) g_b3 += s.dy[r];
    __syncthreads();
    // dZ2 = dy w3 [z2 > 0]: FP32 over Z2, BF16 into the operands of dH1 and dW2
    for (int n = 0; n < GUESS_H; ++n) {
      const float z = s.z2[t * HP + n];
      const float d = z > 0.0f ? dy * s.w[GUESS_OFF_W3 + n] : 0.0f;
      const __nv_bfloat16 db = __float2bfloat16_rn(d);
      s.z2[t * HP + n] = d;
      s.a_dz2[tc05::canon(t, n, GUESS_H)] = db;
      s.a_dz2t[tc05::canon(n, t, TB)] = db;
    }
    tc05::fence_smem_async();
    tc05::fence_before_sync();
    __syncthreads();
    if (t == 0) {
      tc05::fence_after_sync();
      for (int ks = 0; ks < GUESS_H / 16; ++ks)
        tc05::mma_bf16(d_dh1, tc05::sdesc(s.a_dz2 + ks * 128, 128, 1024),
                       tc05::sdesc(s.b_w2t + ks * 128, 128, 1024), TC_ID, ks > 0);
      for (int ks = 0; ks < TB / 16; ++ks)
        tc05::mma_bf16(d_dw2, tc05::sdesc(s.a_dz2t + ks * 128, 128, 2048),
                       tc05::sdesc(s.b_h1t + ks * 128, 128, 2048), TC_ID, any || ks > 0);
      tc05::commit(&s.bar);
    }
    any = true;
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) g_b2 += s.z2[r * HP + unit];
    tc_wait(s, phase);
    if (s.failed) break;
    // dZ1 = dH1 [H1 > 0], over H1: sample t's row
    for (int c = 0; c < GUESS_H / 16; ++c) {
      float v[16];
      tc05::tmem_ld16(d_dh1 + my_lanes + 16 * c, v);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        float *h = &s.h1[t * HP + 16 * c + j];
        *h = *h > 0.0f ? v[j] : 0.0f;
      }
    }
    __syncthreads();
    for (int r = half * (TB / 2); r < (half + 1) * (TB / 2); ++r) {
      const float d = s.h1[r * HP + unit];
      g_w1[0] += d * s.x[r * 3];
      g_w1[1] += d * s.x[r * 3 + 1];
      g_w1[2] += d * s.x[r * 3 + 2];
      g_w1[3] += d;
    }
    tc05::fence_before_sync();
    __syncthreads();  // before the next tile overwrites the tiles and TMEM
    tc05::fence_after_sync();
  }
  const bool failed = s.failed != 0;
  if (!failed) {
    // dW2 rows n = 0..63 are TMEM lanes 0..63: warps 0 and 1, thread t = row n
    if (any && warp < 2) {
      for (int c = 0; c < GUESS_H / 16; ++c) {
        float v[16];
        tc05::tmem_ld16(d_dw2 + my_lanes + 16 * c, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) atomicAdd(grad + GUESS_OFF_W2 + t * GUESS_H + 16 * c + j, v[j]);
      }
    }
    atomicAdd(grad + GUESS_OFF_W1 + 3 * unit, g_w1[0]);
    atomicAdd(grad + GUESS_OFF_W1 + 3 * unit + 1, g_w1[1]);
    atomicAdd(grad + GUESS_OFF_W1 + 3 * unit + 2, g_w1[2]);
    atomicAdd(grad + GUESS_OFF_B1 + unit, g_w1[3]);
    atomicAdd(grad + GUESS_OFF_B2 + unit, g_b2);
    atomicAdd(grad + GUESS_OFF_W3 + unit, g_w3);
    if (t == 0) atomicAdd(grad + GUESS_OFF_B3, g_b3);
    for (int o = 16; o > 0; o >>= 1) l_sum += __shfl_down_sync(0xffffffffu, l_sum, o);
    if (lane == 0) atomicAdd(loss, l_sum);
  } else if (t == 0) {
    // the MMAs may still be in flight: one more bounded wait before the
    // tensor memory is freed
    tc05::mbar_wait(&s.bar, phase ^ 1u, TC_WAIT);
    if (status) atomicExch(status, 1);
  }
  tc05::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc05::fence_after_sync();
    tc05::tmem_free(tm, TC_COLS);
  }
}

__global__ void guess_adam_kernel(float *w, float *grad, float *m, float *v, float lr, float b1,
                                  float b2, float bc1, float bc2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= GUESS_NPARAM) return;
  const float g = grad[i];
  const float mi = b1 * m[i] + (1.0f - b1) * g;
  const float vi = b2 * v[i] + (1.0f - b2) * g * g;
  m[i] = mi;
  v[i] = vi;
  w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
  grad[i] = 0.0f;
}

__global__ void __launch_bounds__(TB) guess_eval_kernel(const float *weights, const float *feats,
                                                        long long n, float *out) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem &s = *reinterpret_cast<TrainSmem *>(smem_raw);
  const int t = threadIdx.x;
  const long long row0 = (long long)blockIdx.x * TB;
  load_weights(s, weights);
  forward_hidden(s, feats, row0, n);
  float y = s.w[GUESS_OFF_B3];
  for (int k = 0; k < GUESS_H; ++k) {
    const float z = s.z2[t * HP + k] + s.w[GUESS_OFF_B2 + k];
    y += s.w[GUESS_OFF_W3 + k] * (z > 0.0f ? z : 0.0f);
  }
  if (row0 + t < n) out[row0 + t] = y;
}

// ---- launchers ---------------------------------------------------------------

size_t guess_smem_bytes() { return sizeof(TrainSmem); }

cudaError_t launch_guess_pairs(long long n, unsigned long long seed, float *feats,
                               float *targets, int *iters, cudaStream_t s) {
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (blocks == 0) return cudaSuccess;
  guess_pairs_kernel<<<blocks, 256, 0, s>>>(n, seed, feats, targets, iters);
  return cudaGetLastError();
}

cudaError_t launch_guess_grad(const float *w, const float *feats, const float *targets,
                              long long batch0, long long nb, float *grad, float *loss,
                              cudaStream_t s) {
  static std::atomic<int> attr[kMaxAttrDevices];
  const cudaError_t ae = smem_attr_once((const void *)guess_train_kernel, (int)sizeof(TrainSmem), attr);
  if (ae != cudaSuccess) return ae;
  const long long tiles = (nb + TB - 1) / TB;
  if (tiles == 0) return cudaSuccess;
  // up to two resident blocks per SM, each over several tiles: fewer
  // blocks, fewer atomics into the gradient
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)(tiles < 2LL * sms ? tiles : 2LL * sms);
  guess_train_kernel<<<blocks, TB, sizeof(TrainSmem), s>>>(w, feats, targets, batch0, nb, grad,
                                                           loss);
  return cudaGetLastError();
}

cudaError_t launch_guess_grad_tc(const float *w, const float *feats, const float *targets,
                                 long long batch0, long long nb, float *grad, float *loss,
                                 int *status, cudaStream_t s) {
  static std::atomic<int> attr[kMaxAttrDevices];
  const cudaError_t ae =
      smem_attr_once((const void *)guess_train_tc_kernel, (int)sizeof(TcTrainSmem), attr);
  if (ae != cudaSuccess) return ae;
  const long long tiles = (nb + TB - 1) / TB;
  if (tiles == 0) return cudaSuccess;
  // one block per SM (its shared memory holds the operand tiles), each over
  // several tiles, so that dW2 stays in its tensor memory between them
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  const unsigned blocks = (unsigned)(tiles < (long long)sms ? tiles : (long long)sms);
  guess_train_tc_kernel<<<blocks, TB, sizeof(TcTrainSmem), s>>>(w, feats, targets, batch0, nb,
                                                                grad, loss, status);
  return cudaGetLastError();
}

cudaError_t launch_guess_adam(float *w, float *grad, float *m, float *v, float lr, int step,
                              cudaStream_t s) {
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.0f - powf(b1, (float)step), bc2 = 1.0f - powf(b2, (float)step);
  guess_adam_kernel<<<(GUESS_NPARAM + 255) / 256, 256, 0, s>>>(w, grad, m, v, lr, b1, b2, bc1,
                                                                bc2);
  return cudaGetLastError();
}

cudaError_t launch_guess_eval(const float *w, const float *feats, long long n, float *out,
                              cudaStream_t s) {
  static std::atomic<int> attr[kMaxAttrDevices];
  const cudaError_t ae = smem_attr_once((const void *)guess_eval_kernel, (int)sizeof(TrainSmem), attr);
  if (ae != cudaSuccess) return ae;
  const unsigned blocks = (unsigned)((n + TB - 1) / TB);
  if (blocks == 0) return cudaSuccess;
  guess_eval_kernel<<<blocks, TB, sizeof(TrainSmem), s>>>(w, feats, n, out);
  return cudaGetLastError();
}

}  // namespace xc
