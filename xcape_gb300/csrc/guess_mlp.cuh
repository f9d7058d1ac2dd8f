// guess_mlp.cuh -- the learned first guess of the moist-adiabat iteration.
//
// A 3 -> 64 -> 64 -> 1 multilayer perceptron (ReLU) maps a saturated parcel's
// state at the start of a sub-step to its potential temperature at the end
// of it:
//   inputs   f0 = (p2 - 55000 Pa) / 45000 Pa     target pressure
//            f1 = (theta_e - 320 K) / 40 K       parcel theta-e (getthe)
//            f2 = 50 qt - 0.5                    total water
//   output   y, the increment per unit log-pressure:
//            theta2 = theta1 + 50 K * y * ln(p1 / p2)
// so the saturated parcel temperature is T2 = theta2 * pi2.  Predicting the
// increment rather than T2 itself makes the guess error a fraction of one
// sub-step's change instead of a fraction of the whole temperature range
// (BF16 weights carry 8 significant bits).  It is trained on pairs that the
// plain solver (the reference's damped iteration) produces, with the
// project's own GPU kernels (guess_mlp.cu).
//
// Parameters live in one flat float array of GUESS_NPARAM values:
//   W1[64][3] | b1[64] | W2[64][64] (row = output unit) | b2[64] | w3[64] | b3
// The trained network is stored with its weights rounded to BF16.
#pragma once
#include "xc_common.cuh"

namespace xc {

constexpr int GUESS_H = 64;
constexpr int GUESS_IN = 3;
constexpr int GUESS_OFF_W1 = 0;
constexpr int GUESS_OFF_B1 = GUESS_OFF_W1 + GUESS_H * GUESS_IN;   // 192
constexpr int GUESS_OFF_W2 = GUESS_OFF_B1 + GUESS_H;              // 256
constexpr int GUESS_OFF_B2 = GUESS_OFF_W2 + GUESS_H * GUESS_H;    // 4352
constexpr int GUESS_OFF_W3 = GUESS_OFF_B2 + GUESS_H;              // 4416
constexpr int GUESS_OFF_B3 = GUESS_OFF_W3 + GUESS_H;              // 4480
constexpr int GUESS_NPARAM = GUESS_OFF_B3 + 1;                    // 4481

constexpr float GUESS_P_MID = 55000.0f, GUESS_P_SCALE = 45000.0f;
constexpr float GUESS_THE_MID = 320.0f, GUESS_THE_SCALE = 40.0f;
constexpr float GUESS_SLOPE_SCALE = 50.0f;
// outputs outside this range are not used (the caller keeps its own guess)
constexpr float GUESS_Y_MIN = -0.2f, GUESS_Y_MAX = 2.0f;

XC_HD void guess_features(float p2, float the, float qt, float &f0, float &f1, float &f2) {
  f0 = (p2 - GUESS_P_MID) / GUESS_P_SCALE;
  f1 = (the - GUESS_THE_MID) / GUESS_THE_SCALE;
  f2 = 50.0f * qt - 0.5f;
}

// One evaluation, FP32 arithmetic, weights from any memory space (shared
// memory in the CAPE kernel).  Returns the normalised output y.
// The hidden layer is accumulated GUESS_CHUNK output units at a time, each
// pass recomputing the first layer's activations (64 x 3 FMAs against the
// 64 x 64 of the second layer), so that only GUESS_CHUNK accumulators are
// live: the network then fits in the register budget of the CAPE kernel it
// is inlined into.  Every sum is taken in the order of a plain loop
// (z_n = b2_n + sum over k ascending, y = b3 + sum over n ascending).
constexpr int GUESS_CHUNK = 16;
XC_HD float guess_eval(const float *w, float f0, float f1, float f2) {
  float y = w[GUESS_OFF_B3];
  for (int n0 = 0; n0 < GUESS_H; n0 += GUESS_CHUNK) {
    float z[GUESS_CHUNK];
#pragma unroll
    for (int j = 0; j < GUESS_CHUNK; ++j) z[j] = w[GUESS_OFF_B2 + n0 + j];
    for (int k = 0; k < GUESS_H; ++k) {
      float h = w[GUESS_OFF_B1 + k] + w[GUESS_OFF_W1 + 3 * k] * f0 +
                w[GUESS_OFF_W1 + 3 * k + 1] * f1 + w[GUESS_OFF_W1 + 3 * k + 2] * f2;
      h = h > 0.0f ? h : 0.0f;
#pragma unroll
      for (int j = 0; j < GUESS_CHUNK; ++j) z[j] += w[GUESS_OFF_W2 + GUESS_H * (n0 + j) + k] * h;
    }
#pragma unroll
    for (int j = 0; j < GUESS_CHUNK; ++j)
      y += w[GUESS_OFF_W3 + n0 + j] * (z[j] > 0.0f ? z[j] : 0.0f);
  }
  return y;
}

// Packed copy of the parameters for the CAPE kernel's shared memory: the
// first 256 values become one float4 per first-layer unit,
// {W1[k][0], W1[k][1], W1[k][2], b1[k]}; the rest (W2, b2, w3, b3) keeps the
// flat offsets, W2's rows being 16-byte aligned.  Element i of the packed
// array:
XC_HD float guess_packed_value(const float *w, int i) {
  if (i >= 4 * GUESS_H) return w[i];
  const int k = i >> 2, c = i & 3;
  return c < 3 ? w[GUESS_OFF_W1 + 3 * k + c] : w[GUESS_OFF_B1 + k];
}

// guess_eval on the packed parameters (16-byte aligned): the same sums in
// the same order, read four weights per load.
XC_HD float guess_eval_packed(const float *pk, float f0, float f1, float f2) {
  float y = pk[GUESS_OFF_B3];
  for (int n0 = 0; n0 < GUESS_H; n0 += GUESS_CHUNK) {
    float z[GUESS_CHUNK];
#pragma unroll
    for (int j = 0; j < GUESS_CHUNK; ++j) z[j] = pk[GUESS_OFF_B2 + n0 + j];
    for (int k = 0; k < GUESS_H; k += 4) {
      float h[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float4 l = *reinterpret_cast<const float4 *>(pk + 4 * (k + u));
        const float v = l.w + l.x * f0 + l.y * f1 + l.z * f2;
        h[u] = v > 0.0f ? v : 0.0f;
      }
#pragma unroll
      for (int j = 0; j < GUESS_CHUNK; ++j) {
        const float4 r =
            *reinterpret_cast<const float4 *>(pk + GUESS_OFF_W2 + GUESS_H * (n0 + j) + k);
        z[j] += r.x * h[0];
        z[j] += r.y * h[1];
        z[j] += r.z * h[2];
        z[j] += r.w * h[3];
      }
    }
#pragma unroll
    for (int j = 0; j < GUESS_CHUNK; ++j)
      y += pk[GUESS_OFF_W3 + n0 + j] * (z[j] > 0.0f ? z[j] : 0.0f);
  }
  return y;
}

// Deterministic uniform numbers for the training pairs (splitmix64 hash of
// (seed, sample, draw)), the same on the host and the device.
XC_HD uint64_t guess_mix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
XC_HD float guess_uniform01(uint64_t seed, long long i, int k) {
  const uint64_t h = guess_mix64(seed ^ guess_mix64((uint64_t)i * 8ull + (uint64_t)k));
  return (float)(h >> 40) * (1.0f / 16777216.0f);
}

}  // namespace xc
