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
