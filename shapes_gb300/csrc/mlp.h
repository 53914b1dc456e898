/* Learned warm start: the small MLP that predicts the starting normal and
 * friction Lagrangians of contacts without a previous-frame cache entry.
 * Internal interface between the MLP translation unit and the step runtime. */
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

struct shapes_mlp;

namespace mlp {

constexpr int kIn = 16;    /* features per contact */
constexpr int kHid = 64;   /* three hidden layers of 64, ReLU */
constexpr int kOut = 2;    /* normal and friction Lagrangian */
constexpr int kOutPad = 16;
/* FP32 parameter vector: W1[64x16] b1 W2[64x64] b2 W3[64x64] b3 W4[2x64] b4 */
constexpr int oW1 = 0, oB1 = 1024, oW2 = 1088, oB2 = 5184, oW3 = 5248, oB3 = 9344, oW4 = 9408, oB4 = 9536;
constexpr int kParams = 9538;
/* normalisation: feature mean[16], feature 1/scale[16], output mean[2], output scale[2] */
constexpr int kNorm = 36;
/* Normalised inputs are clipped to [-kClip, kClip]: a contact whose features
 * lie far outside the training data (another friction range, another scene)
 * then cannot drive the network arbitrarily far. */
constexpr float kClip = 8.f;
constexpr int kTile = 128;

/* Feature indices (raw, before normalisation). */
enum {
  kFVn = 0,      /* J_n . v (velocities after this step's external acceleration) */
  kFVf = 1,      /* J_f . v */
  kFBias = 2,    /* Baumgarte term b_n */
  kFMn = 3,      /* J_n M^-1 J_n^T */
  kFMf = 4,      /* J_f M^-1 J_f^T */
  kFL0n = 5,     /* -(J_n . v + b_n) / (J_n M^-1 J_n^T): one isolated update */
  kFL0f = 6,     /* -(J_f . v) / (J_f M^-1 J_f^T) */
  kFMu = 7,      /* pair friction coefficient */
  kFDepth = 8,   /* penetration depth */
  kFNx = 9,      /* restitution normal (a -> b) */
  kFNy = 10,
  kFGrav = 11,   /* -(J_n . a dt) / (J_n M^-1 J_n^T): impulse that cancels one step of acceleration */
  kFPairN = 12,  /* contacts of this pair (1 or 2) */
  kFStatic = 13, /* 1 when one body is static */
  kFArmA = 14,   /* angular Jacobian entries of the normal row */
  kFArmB = 15,
};

/* Predicts rows [0, *n_rows) of feat (raw features, kIn floats per row) and
 * writes the clamped Lagrangians of contact ids[r] into lam[2 ids[r] ..],
 * marking info[ids[r]] |= hit_bit; n_pred counts the rows.  Returns a CUDA
 * error code of the launch. */
cudaError_t launch_predict_contacts(const float* params, const float* norm, const float* feat,
                                    const int32_t* n_rows, const int32_t* ids, double* lam, uint8_t* info,
                                    uint8_t hit_bit, unsigned long long* n_pred, int* err, int max_rows,
                                    cudaStream_t stream);

/* Per-device set-up of the network kernels (shared-memory limits); call
 * before capturing a step that launches them. */
cudaError_t prepare_device();

/* Device copies of a network's FP32 parameters and normalisation. */
const float* device_params(const shapes_mlp* m);
const float* device_norm(const shapes_mlp* m);

}  // namespace mlp
