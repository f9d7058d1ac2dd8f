// guess_mlp.cu -- data, training and batched inference of the learned first
// guess (guess_mlp.cuh), all on the GPU.
//
// * guess_pairs_kernel draws saturated parcel states and solves one sub-step
//   of each with the plain solver (guess_pair in cape_column.cuh), storing
//   (features, normalised increment, iterations).
// * guess_train_kernel runs forward and backward passes over a batch: the
//   64x64 hidden layer on the tensor cores with mma.sync m16n8k16 (BF16
//   operands, FP32 accumulation), the rest and the whole backward pass in
//   FP32 on the CUDA cores; the block's gradient is added to a global
//   gradient with one atomicAdd per parameter.
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

constexpr int TB = 128;          // samples (threads) per block
constexpr int HP = GUESS_H + 1;  // padded row of the activation tiles

struct TrainSmem {
  float w[GUESS_NPARAM + 3];
  __nv_bfloat16 w2bf[GUESS_H * GUESS_H];
  float h1[TB * HP];  // H1, later dZ1
  float z2[TB * HP];  // Z2, later dZ2
  float x[TB * 3];
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

// Loads the weights and the batch's features, runs layer 1 (FP32) and layer
// 2 (tensor cores).  Rows beyond n are zero samples.
__device__ void forward_hidden(TrainSmem &s, const float *weights, const float *feats,
                               long long row0, long long n) {
  const int t = threadIdx.x;
  for (int i = t; i < GUESS_NPARAM; i += TB) s.w[i] = weights[i];
  for (int i = t; i < GUESS_H * GUESS_H; i += TB)
    s.w2bf[i] = __float2bfloat16_rn(weights[GUESS_OFF_W2 + i]);
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

}  // namespace

__global__ void guess_pairs_kernel(long long n, unsigned long long seed, float *feats,
                                   float *targets, int *iters) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  iters[i] = guess_pair(seed, i, feats + 3 * i, targets + i);
}

// One forward/backward pass of the MSE loss over samples [row0, row0 + TB)
// of the batch [batch0, batch0 + nb); grad and loss accumulate atomically.
__global__ void __launch_bounds__(TB) guess_train_kernel(const float *weights, const float *feats,
                                                         const float *targets, long long batch0,
                                                         long long nb, float *grad,
                                                         float *loss) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  TrainSmem &s = *reinterpret_cast<TrainSmem *>(smem_raw);
  const int t = threadIdx.x;
  const long long row0 = batch0 + (long long)blockIdx.x * TB;
  const long long end = batch0 + nb;
  forward_hidden(s, weights, feats, row0, end);
  const long long g = row0 + t;
  const bool valid = g < end;
  // layer 3 and the loss
  float y = s.w[GUESS_OFF_B3];
  for (int n = 0; n < GUESS_H; ++n) {
    const float z = s.z2[t * HP + n] + s.w[GUESS_OFF_B2 + n];
    s.z2[t * HP + n] = z;  // keep the pre-activation
    y += s.w[GUESS_OFF_W3 + n] * (z > 0.0f ? z : 0.0f);
  }
  const float err = valid ? y - targets[g] : 0.0f;
  const float dy = 2.0f * err / (float)nb;
  // loss: warp reduction then one atomic per warp
  float l = err * err / (float)nb;
  for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xffffffffu, l, o);
  if ((t & 31) == 0) atomicAdd(loss, l);
  // dW3, db3 and dZ2 = dy * w3 * [z2 > 0]; z2 is overwritten by dZ2
  __shared__ float red[TB];
  for (int n = 0; n < GUESS_H; ++n) {
    const float z = s.z2[t * HP + n];
    const float h = z > 0.0f ? z : 0.0f;
    s.z2[t * HP + n] = z > 0.0f ? dy * s.w[GUESS_OFF_W3 + n] : 0.0f;
    red[t] = dy * h;
    __syncthreads();
    for (int o = TB / 2; o > 0; o >>= 1) {
      if (t < o) red[t] += red[t + o];
      __syncthreads();
    }
    if (t == 0) atomicAdd(grad + GUESS_OFF_W3 + n, red[0]);
    __syncthreads();
  }
  red[t] = dy;
  __syncthreads();
  for (int o = TB / 2; o > 0; o >>= 1) {
    if (t < o) red[t] += red[t + o];
    __syncthreads();
  }
  if (t == 0) atomicAdd(grad + GUESS_OFF_B3, red[0]);
  __syncthreads();
  // dW2[n][k] = sum_s dZ2[s][n] H1[s][k], db2[n] = sum_s dZ2[s][n]:
  // thread t owns 32 of the 4096 (n, k) entries.
  for (int e = t; e < GUESS_H * GUESS_H; e += TB) {
    const int n = e / GUESS_H, k = e % GUESS_H;
    float acc = 0.0f;
    for (int r = 0; r < TB; ++r) acc += s.z2[r * HP + n] * s.h1[r * HP + k];
    atomicAdd(grad + GUESS_OFF_W2 + e, acc);
  }
  if (t < GUESS_H) {
    float acc = 0.0f;
    for (int r = 0; r < TB; ++r) acc += s.z2[r * HP + t];
    atomicAdd(grad + GUESS_OFF_B2 + t, acc);
  }
  // dZ1 = (dZ2 W2) * [h1 > 0] in FP32 with the master weights
  float dz1[GUESS_H];
#pragma unroll
  for (int k = 0; k < GUESS_H; ++k) dz1[k] = 0.0f;
  for (int n = 0; n < GUESS_H; ++n) {
    const float d = s.z2[t * HP + n];
#pragma unroll
    for (int k = 0; k < GUESS_H; ++k) dz1[k] += d * s.w[GUESS_OFF_W2 + n * GUESS_H + k];
  }
  __syncthreads();  // every thread is done reading h1 for dW2
#pragma unroll
  for (int k = 0; k < GUESS_H; ++k) s.h1[t * HP + k] = s.h1[t * HP + k] > 0.0f ? dz1[k] : 0.0f;
  __syncthreads();
  // dW1[k][i] = sum_s dZ1[s][k] x[s][i], db1[k] = sum_s dZ1[s][k]
  for (int e = t; e < GUESS_H * 4; e += TB) {
    const int k = e / 4, i = e % 4;
    float acc = 0.0f;
    for (int r = 0; r < TB; ++r) acc += s.h1[r * HP + k] * (i < 3 ? s.x[r * 3 + i] : 1.0f);
    atomicAdd(grad + (i < 3 ? GUESS_OFF_W1 + 3 * k + i : GUESS_OFF_B1 + k), acc);
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
  forward_hidden(s, weights, feats, row0, n);
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
  const unsigned blocks = (unsigned)((nb + TB - 1) / TB);
  if (blocks == 0) return cudaSuccess;
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
