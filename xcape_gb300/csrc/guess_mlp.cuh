// guess_mlp.cuh -- the learned first guess of the moist-adiabat iteration.
//
// A 3 -> 64 -> 64 -> 1 multilayer perceptron (ReLU) maps a saturated parcel's
// state at the start of a sub-step to the parcel temperature at the end of
// it:
//   inputs   f0 = (p2 - 55000 Pa) / 45000 Pa     target pressure
//            f1 = (theta_e - 330 K) / 60 K       parcel theta-e (getthe)
//            f2 = 50 qt - 0.5                    total water
//   output   y, with T2 = 233.15 K + 50 K * y
// The sub-step guess is then thlast = T2 / pi2.  It is trained on pairs that
// the plain solver (the reference's damped iteration) produces, with the
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
constexpr float GUESS_THE_MID = 330.0f, GUESS_THE_SCALE = 60.0f;
constexpr float GUESS_T_MID = 233.15f, GUESS_T_SCALE = 50.0f;

XC_HD void guess_features(float p2, float the, float qt, float &f0, float &f1, float &f2) {
  f0 = (p2 - GUESS_P_MID) / GUESS_P_SCALE;
  f1 = (the - GUESS_THE_MID) / GUESS_THE_SCALE;
  f2 = 50.0f * qt - 0.5f;
}

// One evaluation, FP32 arithmetic, weights from any memory space (shared
// memory in the CAPE kernel).  Returns the normalised output y.
XC_HD float guess_eval(const float *w, float f0, float f1, float f2) {
  float h1[GUESS_H];  // fully unrolled loops keep it in registers
#pragma unroll
  for (int k = 0; k < GUESS_H; ++k) {
    const float z = w[GUESS_OFF_B1 + k] + w[GUESS_OFF_W1 + 3 * k] * f0 +
                    w[GUESS_OFF_W1 + 3 * k + 1] * f1 + w[GUESS_OFF_W1 + 3 * k + 2] * f2;
    h1[k] = z > 0.0f ? z : 0.0f;
  }
  float y = w[GUESS_OFF_B3];
  for (int n = 0; n < GUESS_H; ++n) {
    const float *row = w + GUESS_OFF_W2 + GUESS_H * n;
    float z = w[GUESS_OFF_B2 + n];
#pragma unroll
    for (int k = 0; k < GUESS_H; ++k) z += row[k] * h1[k];
    y += w[GUESS_OFF_W3 + n] * (z > 0.0f ? z : 0.0f);
  }
  return y;
}

}  // namespace xc
