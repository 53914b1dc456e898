/* Learned warm start network: 16 -> 64 -> 64 -> 64 -> 2, ReLU, BF16 operands
 * with FP32 accumulation on the fifth-generation tensor cores (tcgen05.mma,
 * accumulators in TMEM), FP32 master weights and Adam.
 *
 * No counterpart in the reference: the network fills the `newCache` branch of
 * applyCachedSlns (shapes/src/Physics/Solvers/Contact.hs:91-98), where a
 * contact without a previous-frame Lagrangian starts from zero.
 *
 * Kernels (128 threads = 4 warps, one tile of 128 contacts / samples):
 *   k_mlp_predict  forward only; persistent over tiles; 256 TMEM columns.
 *   k_mlp_train    forward, backward and the weight gradients of one tile;
 *                  512 TMEM columns; writes the tile's gradient to its slot.
 *   k_mlp_update   sums the slots in a fixed order (deterministic), scales by
 *                  2 / batch and applies Adam (or returns the gradient).
 *
 * BF16 rounding points (the CPU oracle rounds at the same places): the
 * normalised input, every weight, every hidden activation, the output error,
 * and every back-propagated error (dz) before it enters a matrix product.
 * Biases, accumulators, losses and updates are FP32. */
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <random>
#include <string>
#include <vector>

#include "../../include/shapes_gpu.h"
#include "mlp.h"
#include "tc05.cuh"

namespace mlp {

using tc05::kmaj;

__device__ __forceinline__ void st_bf16(unsigned char* base, uint32_t off, float x) {
  *reinterpret_cast<uint16_t*>(base + off) = tc05::bf16_bits(x);
}

/* Weights of the forward pass as B operands (rows = output features). */
__device__ void stage_forward_weights(const float* __restrict__ P, unsigned char* w1, unsigned char* w2,
                                      unsigned char* w3, unsigned char* w4) {
  for (int e = threadIdx.x; e < kHid * kIn; e += blockDim.x) {
    const int o = e / kIn, i = e % kIn;
    st_bf16(w1, kmaj(o, i, kIn), P[oW1 + e]);
  }
  for (int e = threadIdx.x; e < kHid * kHid; e += blockDim.x) {
    const int o = e / kHid, i = e % kHid;
    st_bf16(w2, kmaj(o, i, kHid), P[oW2 + e]);
    st_bf16(w3, kmaj(o, i, kHid), P[oW3 + e]);
  }
  for (int e = threadIdx.x; e < kOutPad * kHid; e += blockDim.x) {
    const int o = e / kHid, i = e % kHid;
    st_bf16(w4, kmaj(o, i, kHid), o < kOut ? P[oW4 + o * kHid + i] : 0.f);
  }
}

/* 64 FP32 columns [col, col + 64) of this thread's TMEM lane. */
__device__ __forceinline__ void load_row64(uint32_t tbase, int col, float (&v)[64]) {
  const uint32_t lane = 32u * (threadIdx.x >> 5);
#pragma unroll
  for (int c = 0; c < 64; c += 16) tc05::tmem_ld16(tc05::taddr(tbase, lane, col + c), v + c);
}

/* One row of a hidden layer: accumulator + bias, ReLU; bit j of mask is set
 * where the pre-activation is positive. */
__device__ __forceinline__ void hidden_row(uint32_t tbase, int col, const float* bias, float (&h)[64],
                                           uint64_t& mask) {
  load_row64(tbase, col, h);
  mask = 0;
#pragma unroll
  for (int j = 0; j < 64; ++j) {
    const float z = h[j] + bias[j];
    const bool pos = z > 0.f;
    h[j] = pos ? z : 0.f;
    mask |= (uint64_t)pos << j;
  }
}

/* Row t of a K-major operand with K = 64 (eight 16-byte stores). */
__device__ __forceinline__ void store_row64(unsigned char* buf, int t, const float (&h)[64]) {
#pragma unroll
  for (int c = 0; c < 8; ++c) *reinterpret_cast<uint4*>(buf + kmaj(t, 8 * c, kHid)) = tc05::pack8(h + 8 * c);
}

/* Block-wide bounded wait for the MMAs committed to `bar`; on success the
 * phase advances and TMEM reads may follow. */
__device__ __forceinline__ bool wait_mma(uint64_t* bar, uint32_t& phase) {
  const bool ok = __syncthreads_and(tc05::mbar_wait(bar, phase));
  if (ok) {
    phase ^= 1;
    tc05::fence_after();
  }
  return ok;
}

/* Makes this thread's generic shared-memory writes visible to the tensor core
 * and orders them before the next MMA issue. */
__device__ __forceinline__ void publish_smem() {
  tc05::fence_async_smem();
  tc05::fence_before();
  __syncthreads();
  tc05::fence_after();
}

/* ------------------------------------------------------------------------ */
/* Inference                                                                  */
/* ------------------------------------------------------------------------ */

constexpr int kPredW1 = 0, kPredW2 = 2048, kPredW3 = 10240, kPredW4 = 18432, kPredX = 20480, kPredH = 24576;
/* 40 KB of operands; 80 KB requested so that at most two CTAs share an SM and
 * their 2 x 256 TMEM columns always fit (an allocation never waits). */
constexpr int kPredSmem = 80 * 1024;

struct PredictArgs {
  const float* params;
  const float* norm;
  const float* feat;
  const int32_t* n_rows_dev; /* row count on the device, or null */
  int32_t n_rows;            /* row count when n_rows_dev is null */
  int32_t max_rows;
  float* out;                /* generic mode: de-normalised predictions [rows x 2] */
  const int32_t* ids;        /* step mode: contact of each row */
  double* lam;
  uint8_t* info;
  uint8_t hit_bit;
  unsigned long long* n_pred;
  int* err;
};

__global__ void __launch_bounds__(128) k_mlp_predict(PredictArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float sb1[kHid], sb2[kHid], sb3[kHid], sb4[kOut], snorm[kNorm];
  int n = a.n_rows_dev ? *a.n_rows_dev : a.n_rows;
  n = min(n, a.max_rows);
  if ((int)blockIdx.x * kTile >= n) return; /* block-uniform: before any allocation */
  const int t = threadIdx.x;
  stage_forward_weights(a.params, sm + kPredW1, sm + kPredW2, sm + kPredW3, sm + kPredW4);
  for (int k = t; k < kHid; k += 128) {
    sb1[k] = a.params[oB1 + k];
    sb2[k] = a.params[oB2 + k];
    sb3[k] = a.params[oB3 + k];
  }
  if (t < kOut) sb4[t] = a.params[oB4 + t];
  if (t < kNorm) snorm[t] = a.norm[t];
  if (t == 0) tc05::mbar_init(&bar, 1);
  if (t < 32) tc05::tmem_alloc(&tslot, 256);
  publish_smem();
  const uint32_t tb = tslot;
  const uint32_t sX = tc05::smem_addr(sm + kPredX), sH = tc05::smem_addr(sm + kPredH);
  const uint32_t sW1 = tc05::smem_addr(sm + kPredW1), sW2 = tc05::smem_addr(sm + kPredW2);
  const uint32_t sW3 = tc05::smem_addr(sm + kPredW3), sW4 = tc05::smem_addr(sm + kPredW4);
  uint32_t phase = 0;
  bool ok = true;
  for (int tile = blockIdx.x; tile * kTile < n && ok; tile += gridDim.x) {
    const int row = tile * kTile + t;
    const bool valid = row < n;
    float x[kIn];
#pragma unroll
    for (int k = 0; k < kIn; ++k) {
      const float f = valid ? a.feat[(size_t)row * kIn + k] : 0.f;
      x[k] = valid ? fminf(fmaxf((f - snorm[k]) * snorm[kIn + k], -kClip), kClip) : 0.f;
    }
    const float mu = valid ? a.feat[(size_t)row * kIn + kFMu] : 0.f;
    *reinterpret_cast<uint4*>(sm + kPredX + kmaj(t, 0, kIn)) = tc05::pack8(x);
    *reinterpret_cast<uint4*>(sm + kPredX + kmaj(t, 8, kIn)) = tc05::pack8(x + 8);
    publish_smem();
    float h[64];
    uint64_t mask;
    /* layer 1 */
    if (t == 0) {
      tc05::gemm(tb + 0, sX, sW1, 128, kHid, kIn, false);
      tc05::commit(&bar);
    }
    if (!(ok = wait_mma(&bar, phase))) break;
    hidden_row(tb, 0, sb1, h, mask);
    store_row64(sm + kPredH, t, h);
    publish_smem();
    /* layer 2 */
    if (t == 0) {
      tc05::gemm(tb + 64, sH, sW2, 128, kHid, kHid, false);
      tc05::commit(&bar);
    }
    if (!(ok = wait_mma(&bar, phase))) break;
    hidden_row(tb, 64, sb2, h, mask);
    store_row64(sm + kPredH, t, h);
    publish_smem();
    /* layer 3 */
    if (t == 0) {
      tc05::gemm(tb + 128, sH, sW3, 128, kHid, kHid, false);
      tc05::commit(&bar);
    }
    if (!(ok = wait_mma(&bar, phase))) break;
    hidden_row(tb, 128, sb3, h, mask);
    store_row64(sm + kPredH, t, h);
    publish_smem();
    /* output layer (N padded to 16) */
    if (t == 0) {
      tc05::gemm(tb + 192, sH, sW4, 128, kOutPad, kHid, false);
      tc05::commit(&bar);
    }
    if (!(ok = wait_mma(&bar, phase))) break;
    float v[16];
    tc05::tmem_ld16(tc05::taddr(tb, 32 * (t >> 5), 192), v);
    const float y0 = (v[0] + sb4[0]) * snorm[2 * kIn + 2] + snorm[2 * kIn];
    const float y1 = (v[1] + sb4[1]) * snorm[2 * kIn + 3] + snorm[2 * kIn + 1];
    if (valid) {
      if (a.out) {
        a.out[2 * (size_t)row] = y0;
        a.out[2 * (size_t)row + 1] = y1;
      } else {
        /* a valid starting point: positive normal impulse, friction inside
         * the cone (positive / clampAbs, SolutionProcessors.hs:33-53) */
        const double ln = y0 > 0.f ? (double)y0 : 0.0;
        const double lim = ln * (double)mu;
        const double lf = fmin(fmax((double)y1, -lim), lim);
        const int c = a.ids[row];
        a.lam[2 * (size_t)c] = ln;
        a.lam[2 * (size_t)c + 1] = lf;
        a.info[c] |= a.hit_bit;
      }
    }
    tc05::fence_before(); /* this tile's TMEM reads precede the next tile's MMAs */
  }
  if (!ok) {
    if (t == 0) atomicExch(a.err, 1);
    tc05::mbar_wait(&bar, phase); /* bounded: let an MMA still in flight finish */
  } else if (t == 0 && a.n_pred && !a.out) {
    /* rows this block predicted */
    unsigned long long mine = 0;
    for (int tile = blockIdx.x; tile * kTile < n; tile += gridDim.x) mine += min(kTile, n - tile * kTile);
    atomicAdd(a.n_pred, mine);
  }
  __syncthreads();
  if (t < 32) tc05::tmem_free(tb, 256);
}

/* ------------------------------------------------------------------------ */
/* Training                                                                   */
/* ------------------------------------------------------------------------ */

/* shared-memory map of k_mlp_train (bytes) */
constexpr int kTrW1 = 0;                /* 64 x 16  (out, in) */
constexpr int kTrW2 = kTrW1 + 2048;     /* 64 x 64 */
constexpr int kTrW3 = kTrW2 + 8192;     /* 64 x 64 */
constexpr int kTrW4 = kTrW3 + 8192;     /* 16 x 64 (2 real rows) */
constexpr int kTrW4T = kTrW4 + 2048;    /* 64 x 16 (in, out; 2 real columns) */
constexpr int kTrW3T = kTrW4T + 2048;   /* 64 x 64 (in, out) */
constexpr int kTrW2T = kTrW3T + 8192;   /* 64 x 64 */
constexpr int kTrX = kTrW2T + 8192;     /* 128 x 16 samples x features */
constexpr int kTrH = kTrX + 4096;       /* 128 x 64 */
constexpr int kTrA1 = kTrH + 16384;     /* 128 x 128: h1^T rows 0-63, h2^T rows 64-127 (K = samples) */
constexpr int kTrA2 = kTrA1 + 32768;    /* 128 x 128: x^T rows 0-15, ones row 16, h3^T rows 64-127 */
constexpr int kTrB = kTrA2 + 32768;     /* 208 x 128: dz1^T 0-63, dy^T 64-79, dz2^T 80-143, dz3^T 144-207 */
constexpr int kTrDY = kTrB + 208 * 256; /* 128 x 16 output errors */
constexpr int kTrDZ = kTrDY + 4096;     /* 128 x 64 back-propagated errors */
constexpr int kTrEnd = kTrDZ + 16384;
constexpr int kTrainSmem = kTrEnd + 16384; /* + slack */
static_assert(kTrainSmem <= 227 * 1024, "train kernel shared memory");

struct TrainArgs {
  const float* params;
  const float* norm;
  const float* feat;    /* dataset [n x 16] raw features */
  const float* tgt;     /* dataset [n x 2] raw targets */
  const int32_t* index; /* dataset row of each batch row; -1 = padding */
  int32_t batch_rows;   /* rows of this batch (a multiple of 128) */
  float* slots;         /* [tiles x kParams] per-tile gradient sums */
  float* loss_slots;    /* [tiles] per-tile sums of squared errors */
  int* err;
};

/* One tile of 128 samples: forward, backward, and the weight and bias
 * gradients summed over the tile (no 2 / batch factor), written to the tile's
 * slot.  Loss: sum over the two outputs of (y - normalised target)^2.
 *
 * Weight gradients are products over the 128 samples (K = samples).  With
 * M = 128 two layers are stacked per product:
 *   G1 = [h1^T; h2^T] x [dz2^T; dz3^T]^T  -> dW2^T (rows 0-63, cols 0-63),
 *                                           dW3^T (rows 64-127, cols 64-127);
 *   G2 = [x^T; 1; 0; h3^T] x [dz1^T; dy^T; dz2^T; dz3^T]^T
 *                                        -> dW1^T (rows 0-15, cols 0-63),
 *                                           all biases (row 16),
 *                                           dW4^T (rows 64-127, cols 64-65).
 * TMEM columns: z1 0, z2 64, z3 128, y 192 (16); dh3 0, dh2 64, dh1 128 once
 * the forward values are consumed; G2 0-207 and G1 256-383 at the end. */
__global__ void __launch_bounds__(128) k_mlp_train(TrainArgs a) {
  extern __shared__ __align__(1024) unsigned char sm[];
  __shared__ uint64_t bar;
  __shared__ uint32_t tslot;
  __shared__ float sb1[kHid], sb2[kHid], sb3[kHid], sb4[kOut], snorm[kNorm];
  __shared__ float sloss[4];
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const float* P = a.params;
  stage_forward_weights(P, sm + kTrW1, sm + kTrW2, sm + kTrW3, sm + kTrW4);
  /* transposed weights for the backward products: (row j, k = o) = W[o][j] */
  for (int e = t; e < kHid * kHid; e += 128) {
    const int j = e / kHid, o = e % kHid;
    st_bf16(sm + kTrW3T, kmaj(j, o, kHid), P[oW3 + o * kHid + j]);
    st_bf16(sm + kTrW2T, kmaj(j, o, kHid), P[oW2 + o * kHid + j]);
  }
  for (int e = t; e < kHid * kOutPad; e += 128) {
    const int j = e / kOutPad, o = e % kOutPad;
    st_bf16(sm + kTrW4T, kmaj(j, o, kOutPad), o < kOut ? P[oW4 + o * kHid + j] : 0.f);
  }
  /* constant rows: A2 16-63 (row 16 = ones), B 66-79 (output padding) */
  for (int e = t; e < 48 * 128; e += 128) {
    const int r = 16 + e / 128, k = e % 128;
    st_bf16(sm + kTrA2, kmaj(r, k, 128), r == 16 ? 1.f : 0.f);
  }
  for (int e = t; e < 14 * 128; e += 128) {
    const int r = 66 + e / 128, k = e % 128;
    st_bf16(sm + kTrB, kmaj(r, k, 128), 0.f);
  }
  for (int k = t; k < kHid; k += 128) {
    sb1[k] = P[oB1 + k];
    sb2[k] = P[oB2 + k];
    sb3[k] = P[oB3 + k];
  }
  if (t < kOut) sb4[t] = P[oB4 + t];
  if (t < kNorm) snorm[t] = a.norm[t];
  if (t == 0) tc05::mbar_init(&bar, 1);
  if (t < 32) tc05::tmem_alloc(&tslot, 512);
  __syncthreads(); /* biases and normalisation are read by every thread below */

  const int row = blockIdx.x * kTile + t;
  const int smp = row < a.batch_rows ? a.index[row] : -1;
  const bool valid = smp >= 0;
  float x[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k)
    x[k] = valid ? fminf(fmaxf((a.feat[(size_t)smp * kIn + k] - snorm[k]) * snorm[kIn + k], -kClip), kClip) : 0.f;
  *reinterpret_cast<uint4*>(sm + kTrX + kmaj(t, 0, kIn)) = tc05::pack8(x);
  *reinterpret_cast<uint4*>(sm + kTrX + kmaj(t, 8, kIn)) = tc05::pack8(x + 8);
#pragma unroll
  for (int k = 0; k < kIn; ++k) st_bf16(sm + kTrA2, kmaj(k, t, 128), x[k]);
  publish_smem();
  const uint32_t tb = tslot;
  auto sa = [&](int off) { return tc05::smem_addr(sm + off); };

  uint32_t phase = 0;
  bool ok = true;
  /* waits for the MMAs issued by thread 0 since the last wait */
  auto finish = [&]() {
    if (t == 0) tc05::commit(&bar);
    return ok = wait_mma(&bar, phase);
  };
  float h[64];
  uint64_t m1 = 0, m2 = 0, m3 = 0;
  float sq = 0.f;
  do {
    /* ---- forward ---- */
    if (t == 0) tc05::gemm(tb + 0, sa(kTrX), sa(kTrW1), 128, kHid, kIn, false);
    if (!finish()) break;
    hidden_row(tb, 0, sb1, h, m1);
    store_row64(sm + kTrH, t, h);
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrA1, kmaj(j, t, 128), h[j]);
    publish_smem();
    if (t == 0) tc05::gemm(tb + 64, sa(kTrH), sa(kTrW2), 128, kHid, kHid, false);
    if (!finish()) break;
    hidden_row(tb, 64, sb2, h, m2);
    store_row64(sm + kTrH, t, h);
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrA1, kmaj(64 + j, t, 128), h[j]);
    publish_smem();
    if (t == 0) tc05::gemm(tb + 128, sa(kTrH), sa(kTrW3), 128, kHid, kHid, false);
    if (!finish()) break;
    hidden_row(tb, 128, sb3, h, m3);
    store_row64(sm + kTrH, t, h);
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrA2, kmaj(64 + j, t, 128), h[j]);
    publish_smem();
    if (t == 0) tc05::gemm(tb + 192, sa(kTrH), sa(kTrW4), 128, kOutPad, kHid, false);
    if (!finish()) break;
    float e[16];
    tc05::tmem_ld16(tc05::taddr(tb, 32 * w, 192), e);
    {
      float dy0 = 0.f, dy1 = 0.f;
      if (valid) {
        const float t0 = (a.tgt[2 * (size_t)smp] - snorm[2 * kIn]) / snorm[2 * kIn + 2];
        const float t1 = (a.tgt[2 * (size_t)smp + 1] - snorm[2 * kIn + 1]) / snorm[2 * kIn + 3];
        dy0 = (e[0] + sb4[0]) - t0;
        dy1 = (e[1] + sb4[1]) - t1;
      }
      sq = dy0 * dy0 + dy1 * dy1;
#pragma unroll
      for (int k = 0; k < 16; ++k) e[k] = 0.f;
      e[0] = dy0;
      e[1] = dy1;
    }
    /* ---- backward ---- */
    *reinterpret_cast<uint4*>(sm + kTrDY + kmaj(t, 0, kOutPad)) = tc05::pack8(e);
    *reinterpret_cast<uint4*>(sm + kTrDY + kmaj(t, 8, kOutPad)) = tc05::pack8(e + 8);
    st_bf16(sm + kTrB, kmaj(64, t, 128), e[0]);
    st_bf16(sm + kTrB, kmaj(65, t, 128), e[1]);
    publish_smem();
    /* dh3 = dy W4; dz3 = dh3 * relu'(z3) */
    if (t == 0) tc05::gemm(tb + 0, sa(kTrDY), sa(kTrW4T), 128, kHid, kOutPad, false);
    if (!finish()) break;
    load_row64(tb, 0, h);
    for (int j = 0; j < kHid; ++j) h[j] = ((m3 >> j) & 1) ? h[j] : 0.f;
    store_row64(sm + kTrDZ, t, h);
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrB, kmaj(144 + j, t, 128), h[j]);
    publish_smem();
    /* dh2 = dz3 W3 */
    if (t == 0) tc05::gemm(tb + 64, sa(kTrDZ), sa(kTrW3T), 128, kHid, kHid, false);
    if (!finish()) break;
    load_row64(tb, 64, h);
    for (int j = 0; j < kHid; ++j) h[j] = ((m2 >> j) & 1) ? h[j] : 0.f;
    store_row64(sm + kTrDZ, t, h);
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrB, kmaj(80 + j, t, 128), h[j]);
    publish_smem();
    /* dh1 = dz2 W2 */
    if (t == 0) tc05::gemm(tb + 128, sa(kTrDZ), sa(kTrW2T), 128, kHid, kHid, false);
    if (!finish()) break;
    load_row64(tb, 128, h);
    for (int j = 0; j < kHid; ++j) h[j] = ((m1 >> j) & 1) ? h[j] : 0.f;
    for (int j = 0; j < kHid; ++j) st_bf16(sm + kTrB, kmaj(j, t, 128), h[j]);
    publish_smem();
    /* weight and bias gradients */
    if (t == 0) {
      tc05::gemm(tb + 256, sa(kTrA1), sa(kTrB) + (uint32_t)kmaj(80, 0, 128), 128, 128, 128, false);
      tc05::gemm(tb + 0, sa(kTrA2), sa(kTrB), 128, 208, 128, false);
    }
    if (!finish()) break;
    float* slot = a.slots + (size_t)blockIdx.x * kParams;
    float v[16];
    if (w == 0) {
      for (int c = 0; c < 208; c += 16) {
        tc05::tmem_ld16(tc05::taddr(tb, 0, c), v);
        for (int k = 0; k < 16; ++k) {
          const int o = c + k;
          if (lane < 16) {
            if (o < 64) slot[oW1 + o * kIn + lane] = v[k];
          } else if (lane == 16) {
            if (o < 64) slot[oB1 + o] = v[k];
            else if (o < 66) slot[oB4 + o - 64] = v[k];
            else if (o >= 80 && o < 144) slot[oB2 + o - 80] = v[k];
            else if (o >= 144) slot[oB3 + o - 144] = v[k];
          }
        }
      }
    }
    if (w < 2) {
      for (int c = 0; c < 64; c += 16) {
        tc05::tmem_ld16(tc05::taddr(tb, 32 * w, 256 + c), v);
        for (int k = 0; k < 16; ++k) slot[oW2 + (c + k) * kHid + t] = v[k];
      }
    } else {
      const int i = t - 64;
      for (int c = 0; c < 64; c += 16) {
        tc05::tmem_ld16(tc05::taddr(tb, 32 * w, 320 + c), v);
        for (int k = 0; k < 16; ++k) slot[oW3 + (c + k) * kHid + i] = v[k];
      }
      tc05::tmem_ld16(tc05::taddr(tb, 32 * w, 64), v);
      slot[oW4 + i] = v[0];
      slot[oW4 + kHid + i] = v[1];
    }
  } while (false);
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  if (lane == 0) sloss[w] = sq;
  if (!ok) {
    if (t == 0) atomicExch(a.err, 1);
    tc05::mbar_wait(&bar, phase); /* bounded: let an MMA still in flight finish */
  }
  tc05::fence_before();
  __syncthreads();
  if (t == 0) a.loss_slots[blockIdx.x] = ok ? (sloss[0] + sloss[1]) + (sloss[2] + sloss[3]) : 0.f;
  if (t < 32) tc05::tmem_free(tb, 512);
}

/* Gradient = scale * (sum of the tile slots in tile order); then Adam, or the
 * gradient itself when grad_out is set.  Thread p owns parameter p. */
__global__ void k_mlp_update(float* params, float* m, float* v, const float* slots, int tiles, float scale,
                             float lr, float beta1, float beta2, float eps, float bc1, float bc2, float* grad_out,
                             const float* loss_slots, float* loss_acc) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p == 0 && loss_acc) {
    float l = 0.f;
    for (int s = 0; s < tiles; ++s) l += loss_slots[s];
    *loss_acc += l;
  }
  if (p >= kParams) return;
  float g = 0.f;
  for (int s = 0; s < tiles; ++s) g += slots[(size_t)s * kParams + p];
  g *= scale;
  if (grad_out) {
    grad_out[p] = g;
    return;
  }
  const float mm = beta1 * m[p] + (1.f - beta1) * g;
  const float vv = beta2 * v[p] + (1.f - beta2) * g * g;
  m[p] = mm;
  v[p] = vv;
  params[p] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
}

/* ------------------------------------------------------------------------ */
/* Launch helpers                                                             */
/* ------------------------------------------------------------------------ */

int num_sms() { /* handles may be used from several host threads: atomics */
  static std::atomic<int> sms{0};
  int v = sms.load(std::memory_order_relaxed);
  if (!v) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    if (v <= 0) v = 148;
    sms.store(v, std::memory_order_relaxed);
  }
  return v;
}

/* Shared-memory limits of the two tensor-core kernels, set once per device
 * (outside any stream capture: prepare_device() runs before a step is
 * captured). */
cudaError_t set_smem_attrs() {
  static std::atomic<unsigned long long> done{0}; /* bit per device */
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 64 && ((done.load() >> dev) & 1ull)) return cudaSuccess;
  e = cudaFuncSetAttribute(k_mlp_predict, cudaFuncAttributeMaxDynamicSharedMemorySize, kPredSmem);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, kTrainSmem);
  if (e == cudaSuccess && dev < 64) done.fetch_or(1ull << dev);
  return e;
}

cudaError_t prepare_device() {
  num_sms();
  return set_smem_attrs();
}

cudaError_t launch_predict(const PredictArgs& a, int max_rows, cudaStream_t stream) {
  const cudaError_t e = set_smem_attrs();
  if (e != cudaSuccess) return e;
  const int tiles = (max_rows + kTile - 1) / kTile;
  const int grid = std::max(1, std::min(tiles, 2 * num_sms()));
  k_mlp_predict<<<grid, 128, kPredSmem, stream>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_predict_contacts(const float* params, const float* norm, const float* feat,
                                    const int32_t* n_rows, const int32_t* ids, double* lam, uint8_t* info,
                                    uint8_t hit_bit, unsigned long long* n_pred, int* err, int max_rows,
                                    cudaStream_t stream) {
  PredictArgs a{};
  a.params = params;
  a.norm = norm;
  a.feat = feat;
  a.n_rows_dev = n_rows;
  a.max_rows = max_rows;
  a.ids = ids;
  a.lam = lam;
  a.info = info;
  a.hit_bit = hit_bit;
  a.n_pred = n_pred;
  a.err = err;
  if (max_rows <= 0) return cudaSuccess;
  return launch_predict(a, max_rows, stream);
}

}  // namespace mlp

/* ------------------------------------------------------------------------ */
/* C ABI                                                                      */
/* ------------------------------------------------------------------------ */

extern thread_local std::string g_last_error;

struct shapes_mlp {
  float* params = nullptr; /* FP32 masters [kParams] */
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* norm = nullptr; /* [kNorm] */
  int64_t adam_t = 0;
  float* slots = nullptr;
  float* loss_slots = nullptr;
  int slot_tiles = 0;
  float* loss_acc = nullptr; /* [1] */
  int* err = nullptr;
  cudaStream_t stream = nullptr;
};

namespace {

int mlp_fail(cudaError_t e, const char* what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
  return SHAPES_E_CUDA;
}

#define MLP_CK(expr, what)                           \
  do {                                               \
    const cudaError_t e_ = (expr);                   \
    if (e_ != cudaSuccess) return mlp_fail(e_, what); \
  } while (0)

int ensure_slots(shapes_mlp* m, int tiles) {
  if (tiles <= m->slot_tiles) return SHAPES_OK;
  cudaFree(m->slots);
  cudaFree(m->loss_slots);
  m->slots = nullptr;
  m->loss_slots = nullptr;
  m->slot_tiles = 0;
  MLP_CK(cudaMalloc(&m->slots, sizeof(float) * mlp::kParams * (size_t)tiles), "cudaMalloc");
  MLP_CK(cudaMalloc(&m->loss_slots, sizeof(float) * (size_t)tiles), "cudaMalloc");
  m->slot_tiles = tiles;
  return SHAPES_OK;
}

/* Device buffer that frees itself. */
template <class T>
struct DevBuf {
  T* p = nullptr;
  ~DevBuf() { cudaFree(p); }
  cudaError_t alloc(size_t n) { return cudaMalloc(&p, sizeof(T) * std::max<size_t>(n, 1)); }
};

int check_err(shapes_mlp* m) {
  int h = 0;
  MLP_CK(cudaMemcpyAsync(&h, m->err, sizeof(int), cudaMemcpyDeviceToHost, m->stream), "download");
  MLP_CK(cudaStreamSynchronize(m->stream), "sync");
  if (h) {
    g_last_error = "MLP kernel: a bounded tensor-core wait gave up";
    cudaMemsetAsync(m->err, 0, sizeof(int), m->stream);
    return SHAPES_E_TIMEOUT;
  }
  return SHAPES_OK;
}

}  // namespace

extern "C" {

int shapes_mlp_create(uint64_t seed, shapes_mlp** out) {
  if (!out) return SHAPES_E_INVALID_ARG;
  *out = nullptr;
  shapes_mlp* m = new (std::nothrow) shapes_mlp();
  if (!m) return SHAPES_E_CAPACITY;
  std::vector<float> p(mlp::kParams, 0.f);
  std::mt19937_64 rng(seed);
  auto init = [&](int off, int fan_out, int fan_in) {
    const float lim = std::sqrt(6.f / (float)fan_in); /* He-uniform for ReLU */
    std::uniform_real_distribution<float> u(-lim, lim);
    for (int k = 0; k < fan_out * fan_in; ++k) p[off + k] = u(rng);
  };
  init(mlp::oW1, mlp::kHid, mlp::kIn);
  init(mlp::oW2, mlp::kHid, mlp::kHid);
  init(mlp::oW3, mlp::kHid, mlp::kHid);
  init(mlp::oW4, mlp::kOut, mlp::kHid);
  for (int k = mlp::oW4; k < mlp::oW4 + mlp::kOut * mlp::kHid; ++k) p[k] *= 0.1f;
  float norm[mlp::kNorm];
  for (int k = 0; k < mlp::kIn; ++k) {
    norm[k] = 0.f;
    norm[mlp::kIn + k] = 1.f;
  }
  norm[2 * mlp::kIn] = norm[2 * mlp::kIn + 1] = 0.f;
  norm[2 * mlp::kIn + 2] = norm[2 * mlp::kIn + 3] = 1.f;
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&m->params, sizeof(float) * mlp::kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->adam_m, sizeof(float) * mlp::kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->adam_v, sizeof(float) * mlp::kParams);
  if (e == cudaSuccess) e = cudaMalloc(&m->norm, sizeof(float) * mlp::kNorm);
  if (e == cudaSuccess) e = cudaMalloc(&m->loss_acc, sizeof(float));
  if (e == cudaSuccess) e = cudaMalloc(&m->err, sizeof(int));
  /* every transfer on the network's own stream, complete before returning */
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(m->params, p.data(), sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(m->norm, norm, sizeof(norm), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->adam_m, 0, sizeof(float) * mlp::kParams, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->adam_v, 0, sizeof(float) * mlp::kParams, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->err, 0, sizeof(int), m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  if (e != cudaSuccess) {
    shapes_mlp_destroy(m);
    return mlp_fail(e, "shapes_mlp_create");
  }
  *out = m;
  return SHAPES_OK;
}

void shapes_mlp_destroy(shapes_mlp* m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->params);
  cudaFree(m->adam_m);
  cudaFree(m->adam_v);
  cudaFree(m->norm);
  cudaFree(m->slots);
  cudaFree(m->loss_slots);
  cudaFree(m->loss_acc);
  cudaFree(m->err);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

int shapes_mlp_get_params(shapes_mlp* m, float* params, float* norm) {
  if (!m) return SHAPES_E_INVALID_ARG;
  if (params)
    MLP_CK(cudaMemcpyAsync(params, m->params, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, m->stream),
           "download");
  if (norm)
    MLP_CK(cudaMemcpyAsync(norm, m->norm, sizeof(float) * mlp::kNorm, cudaMemcpyDeviceToHost, m->stream),
           "download");
  MLP_CK(cudaStreamSynchronize(m->stream), "sync");
  return SHAPES_OK;
}

int shapes_mlp_set_params(shapes_mlp* m, const float* params, const float* norm) {
  if (!m) return SHAPES_E_INVALID_ARG;
  if (params)
    for (int k = 0; k < mlp::kParams; ++k)
      if (!std::isfinite(params[k])) return SHAPES_E_NAN;
  if (norm)
    for (int k = 0; k < mlp::kNorm; ++k)
      if (!std::isfinite(norm[k])) return SHAPES_E_NAN;
  if (params) {
    MLP_CK(cudaMemcpyAsync(m->params, params, sizeof(float) * mlp::kParams, cudaMemcpyHostToDevice, m->stream),
           "upload");
    MLP_CK(cudaMemsetAsync(m->adam_m, 0, sizeof(float) * mlp::kParams, m->stream), "memset");
    MLP_CK(cudaMemsetAsync(m->adam_v, 0, sizeof(float) * mlp::kParams, m->stream), "memset");
    m->adam_t = 0;
  }
  if (norm)
    MLP_CK(cudaMemcpyAsync(m->norm, norm, sizeof(float) * mlp::kNorm, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaStreamSynchronize(m->stream), "sync");
  return SHAPES_OK;
}

int shapes_mlp_fit_normalization(shapes_mlp* m, const float* feat, const float* tgt, int64_t n) {
  if (!m || !feat || !tgt || n <= 0) return SHAPES_E_INVALID_ARG;
  double s1[mlp::kIn + mlp::kOut] = {0}, s2[mlp::kIn + mlp::kOut] = {0};
  for (int64_t r = 0; r < n; ++r) {
    for (int k = 0; k < mlp::kIn; ++k) {
      const double x = feat[r * mlp::kIn + k];
      if (!std::isfinite(x)) return SHAPES_E_NAN;
      s1[k] += x;
      s2[k] += x * x;
    }
    for (int k = 0; k < mlp::kOut; ++k) {
      const double x = tgt[r * mlp::kOut + k];
      if (!std::isfinite(x)) return SHAPES_E_NAN;
      s1[mlp::kIn + k] += x;
      s2[mlp::kIn + k] += x * x;
    }
  }
  float norm[mlp::kNorm];
  for (int k = 0; k < mlp::kIn + mlp::kOut; ++k) {
    const double mean = s1[k] / (double)n;
    const double var = std::max(0.0, s2[k] / (double)n - mean * mean);
    const double sd = std::max(std::sqrt(var), 1e-6);
    if (k < mlp::kIn) {
      norm[k] = (float)mean;
      norm[mlp::kIn + k] = (float)(1.0 / sd);
    } else {
      norm[2 * mlp::kIn + (k - mlp::kIn)] = (float)mean;
      norm[2 * mlp::kIn + 2 + (k - mlp::kIn)] = (float)sd;
    }
  }
  return shapes_mlp_set_params(m, nullptr, norm);
}

int shapes_mlp_forward(shapes_mlp* m, const float* feat, int64_t n, float* out) {
  if (!m || !feat || !out || n < 0 || n > INT32_MAX / 2) return SHAPES_E_INVALID_ARG;
  if (n == 0) return SHAPES_OK;
  DevBuf<float> df, dout;
  MLP_CK(df.alloc((size_t)n * mlp::kIn), "cudaMalloc");
  MLP_CK(dout.alloc((size_t)n * mlp::kOut), "cudaMalloc");
  MLP_CK(cudaMemcpyAsync(df.p, feat, sizeof(float) * mlp::kIn * n, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaStreamSynchronize(m->stream), "upload"); /* inputs resident before the kernels read them */
  mlp::PredictArgs a{};
  a.params = m->params;
  a.norm = m->norm;
  a.feat = df.p;
  a.n_rows = (int32_t)n;
  a.max_rows = (int32_t)n;
  a.out = dout.p;
  a.err = m->err;
  MLP_CK(mlp::launch_predict(a, (int)n, m->stream), "k_mlp_predict");
  MLP_CK(cudaMemcpyAsync(out, dout.p, sizeof(float) * mlp::kOut * n, cudaMemcpyDeviceToHost, m->stream),
         "download");
  return check_err(m);
}

namespace {

/* One gradient evaluation or Adam step over batch rows [0, rows) of the
 * device index list (padded with -1 to a multiple of 128). */
int train_batch(shapes_mlp* m, const float* dfeat, const float* dtgt, const int32_t* dindex, int rows, int n_real,
                float lr, float* grad_out, bool count_loss) {
  const int tiles = (rows + mlp::kTile - 1) / mlp::kTile;
  int rc = ensure_slots(m, tiles);
  if (rc) return rc;
  MLP_CK(mlp::set_smem_attrs(), "cudaFuncSetAttribute");
  mlp::TrainArgs a{};
  a.params = m->params;
  a.norm = m->norm;
  a.feat = dfeat;
  a.tgt = dtgt;
  a.index = dindex;
  a.batch_rows = tiles * mlp::kTile;
  a.slots = m->slots;
  a.loss_slots = m->loss_slots;
  a.err = m->err;
  mlp::k_mlp_train<<<tiles, 128, mlp::kTrainSmem, m->stream>>>(a);
  MLP_CK(cudaGetLastError(), "k_mlp_train");
  const float b1 = 0.9f, b2 = 0.999f;
  float bc1 = 1.f, bc2 = 1.f;
  if (!grad_out) {
    ++m->adam_t;
    bc1 = 1.f - (float)std::pow((double)b1, (double)m->adam_t);
    bc2 = 1.f - (float)std::pow((double)b2, (double)m->adam_t);
  }
  mlp::k_mlp_update<<<(mlp::kParams + 255) / 256, 256, 0, m->stream>>>(
      m->params, m->adam_m, m->adam_v, m->slots, tiles, 2.f / (float)n_real, lr, b1, b2, 1e-8f, bc1, bc2, grad_out,
      m->loss_slots, count_loss ? m->loss_acc : nullptr);
  MLP_CK(cudaGetLastError(), "k_mlp_update");
  return SHAPES_OK;
}

}  // namespace

int shapes_mlp_gradient(shapes_mlp* m, const float* feat, const float* tgt, int64_t n, float* grad, float* loss) {
  if (!m || !feat || !tgt || !grad || n <= 0 || n > (1 << 20)) return SHAPES_E_INVALID_ARG;
  const int rows = (int)((n + mlp::kTile - 1) / mlp::kTile * mlp::kTile);
  std::vector<int32_t> idx(rows, -1);
  for (int64_t k = 0; k < n; ++k) idx[k] = (int32_t)k;
  DevBuf<float> df, dt, dg;
  DevBuf<int32_t> di;
  MLP_CK(df.alloc((size_t)n * mlp::kIn), "cudaMalloc");
  MLP_CK(dt.alloc((size_t)n * mlp::kOut), "cudaMalloc");
  MLP_CK(dg.alloc(mlp::kParams), "cudaMalloc");
  MLP_CK(di.alloc(rows), "cudaMalloc");
  MLP_CK(cudaMemcpyAsync(df.p, feat, sizeof(float) * mlp::kIn * n, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaMemcpyAsync(dt.p, tgt, sizeof(float) * mlp::kOut * n, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaMemcpyAsync(di.p, idx.data(), sizeof(int32_t) * rows, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaMemsetAsync(m->loss_acc, 0, sizeof(float), m->stream), "memset");
  MLP_CK(cudaStreamSynchronize(m->stream), "upload"); /* inputs resident before the kernels read them */
  int rc = train_batch(m, df.p, dt.p, di.p, rows, (int)n, 0.f, dg.p, true);
  if (rc) return rc;
  float l = 0.f;
  MLP_CK(cudaMemcpyAsync(grad, dg.p, sizeof(float) * mlp::kParams, cudaMemcpyDeviceToHost, m->stream), "download");
  MLP_CK(cudaMemcpyAsync(&l, m->loss_acc, sizeof(float), cudaMemcpyDeviceToHost, m->stream), "download");
  rc = check_err(m);
  if (rc) return rc;
  if (loss) *loss = l / (float)n;
  return SHAPES_OK;
}

int shapes_mlp_train(shapes_mlp* m, const float* feat, const float* tgt, int64_t n, const shapes_train_config* tc,
                     float* epoch_loss) {
  if (!m || !feat || !tgt || !tc || n <= 0 || n > INT32_MAX / 4) return SHAPES_E_INVALID_ARG;
  if (tc->epochs <= 0 || tc->batch <= 0 || tc->batch % mlp::kTile || !(tc->lr > 0.f)) return SHAPES_E_INVALID_ARG;
  const int batch = tc->batch;
  DevBuf<float> df, dt;
  DevBuf<int32_t> di;
  MLP_CK(df.alloc((size_t)n * mlp::kIn), "cudaMalloc");
  MLP_CK(dt.alloc((size_t)n * mlp::kOut), "cudaMalloc");
  MLP_CK(di.alloc((size_t)n + batch), "cudaMalloc");
  MLP_CK(cudaMemcpyAsync(df.p, feat, sizeof(float) * mlp::kIn * n, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaMemcpyAsync(dt.p, tgt, sizeof(float) * mlp::kOut * n, cudaMemcpyHostToDevice, m->stream), "upload");
  MLP_CK(cudaStreamSynchronize(m->stream), "upload");
  std::vector<int32_t> perm((size_t)n + batch, -1);
  std::mt19937_64 rng(tc->seed);
  for (int ep = 0; ep < tc->epochs; ++ep) {
    for (int64_t k = 0; k < n; ++k) perm[k] = (int32_t)k;
    for (int64_t k = n - 1; k > 0; --k) { /* Fisher-Yates */
      const int64_t j = (int64_t)(rng() % (uint64_t)(k + 1));
      std::swap(perm[k], perm[j]);
    }
    MLP_CK(cudaStreamSynchronize(m->stream), "sync"); /* the previous epoch's batches read di */
    MLP_CK(cudaMemcpyAsync(di.p, perm.data(), sizeof(int32_t) * perm.size(), cudaMemcpyHostToDevice, m->stream),
           "upload");
    MLP_CK(cudaMemsetAsync(m->loss_acc, 0, sizeof(float), m->stream), "memset");
    MLP_CK(cudaStreamSynchronize(m->stream), "upload");
    for (int64_t off = 0; off < n; off += batch) {
      const int real = (int)std::min<int64_t>(batch, n - off);
      const int rows = (real + mlp::kTile - 1) / mlp::kTile * mlp::kTile;
      const int rc = train_batch(m, df.p, dt.p, di.p + off, rows, real, tc->lr, nullptr, true);
      if (rc) return rc;
    }
    float l = 0.f;
    MLP_CK(cudaMemcpyAsync(&l, m->loss_acc, sizeof(float), cudaMemcpyDeviceToHost, m->stream), "download");
    const int rc = check_err(m);
    if (rc) return rc;
    if (epoch_loss) epoch_loss[ep] = l / (float)n;
  }
  return SHAPES_OK;
}

}  // extern "C"

const float* mlp::device_params(const shapes_mlp* m) { return m ? m->params : nullptr; }
const float* mlp::device_norm(const shapes_mlp* m) { return m ? m->norm : nullptr; }
