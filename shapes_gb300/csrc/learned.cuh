/* Learned warm start inside the step (no counterpart in the reference).
 *
 * The reference starts a contact without a previous-frame cache entry from
 * zero (applyCachedSlns, shapes/src/Physics/Solvers/Contact.hs:91-98).  With a
 * network attached, k_build flags those contacts (in worlds whose learned
 * mask is set); a scan gives each a row; k_learned_features writes the row's
 * 16 features; the tensor-core network (mlp.cu) writes the predicted starting
 * Lagrangians and marks the contact as started, so the warm-start pass applies
 * them exactly like a cache hit (applySln, Solvers/Contact.hs:55-65).
 *
 * Training samples come from the same rows with the network off: features
 * before the solve, final Lagrangians after the last sweep (k_collect).
 *
 * The judge (k_learned_judge) clears a world's mask when its residual or its
 * largest depth exceeds the per-world limit, so that world starts plainly
 * from then on. */
#pragma once

#include "mlp.h"
#include "step_kernels.cuh"

namespace shapes {

/* Rows of the flagged contacts: row r = miss_off[c] holds contact c. */
__global__ void k_learned_features(Dev d, int external, double ax, double ay, double dt) {
  const int C = min((int)d.counters[kCntContacts], d.contact_cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) d.miss_n[0] = d.miss_off[C];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    if (!d.miss_flag[c]) continue;
    const int row = d.miss_off[c];
    d.miss_ids[row] = c;
    const Con& cc = d.con[c];
    const int ga = d.c_ga[c], gb = d.c_gb[c];
    const uint8_t info = d.c_hit[c];
    /* velocities as the solver will see them: after applyExternal */
    const bool acc_a = external && !(0.0 == d.iml[ga]), acc_b = external && !(0.0 == d.iml[gb]);
    double v[6] = {d.vx[ga], d.vy[ga], d.w[ga], d.vx[gb], d.vy[gb], d.w[gb]};
    if (acc_a) {
      v[0] = v[0] + ax * dt;
      v[1] = v[1] + ay * dt;
    }
    if (acc_b) {
      v[3] = v[3] + ax * dt;
      v[4] = v[4] + ay * dt;
    }
    const double g[6] = {acc_a ? ax * dt : 0.0, acc_a ? ay * dt : 0.0, 0.0,
                         acc_b ? ax * dt : 0.0, acc_b ? ay * dt : 0.0, 0.0};
    double jn[6], jf[6];
    for (int k = 0; k < 6; ++k) {
      jn[k] = cc.jn[k];
      jf[k] = cc.jf[k];
    }
    const double vn = dot6(jn, v), vf = dot6(jf, v), gn = dot6(jn, g);
    const double mcn = cc.mcn, mcf = cc.mcf;
    const bool okn = mcn > 0.0, okf = mcf > 0.0;
    int pair_n = 1;
    if (c > 0 && d.c_ga[c - 1] == ga && d.c_gb[c - 1] == gb) ++pair_n;
    if (c + 1 < C && d.c_ga[c + 1] == ga && d.c_gb[c + 1] == gb) ++pair_n;
    float f[mlp::kIn];
    f[mlp::kFVn] = (float)vn;
    f[mlp::kFVf] = (float)vf;
    f[mlp::kFBias] = (float)cc.bn;
    f[mlp::kFMn] = (float)mcn;
    f[mlp::kFMf] = (float)mcf;
    f[mlp::kFL0n] = okn ? (float)(-(vn + cc.bn) / mcn) : 0.f;
    f[mlp::kFL0f] = okf ? (float)(-vf / mcf) : 0.f;
    f[mlp::kFMu] = (float)cc.mu;
    f[mlp::kFDepth] = (float)d.c_val[5 * (size_t)c + 4];
    f[mlp::kFNx] = (float)cc.rnx;
    f[mlp::kFNy] = (float)cc.rny;
    f[mlp::kFGrav] = okn ? (float)(-gn / mcn) : 0.f;
    f[mlp::kFPairN] = (float)pair_n;
    f[mlp::kFStatic] = ((info & kInfoDynA) && (info & kInfoDynB)) ? 0.f : 1.f;
    f[mlp::kFArmA] = (float)jn[2];
    f[mlp::kFArmB] = (float)jn[5];
    float4* out = reinterpret_cast<float4*>(d.mfeat + (size_t)row * mlp::kIn);
    for (int k = 0; k < 4; ++k) out[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
  }
}

/* Appends this step's samples: features (before the solve) and the final
 * Lagrangians of the same contacts (after the last sweep). */
__global__ void k_collect(Dev d, float* ds_feat, float* ds_tgt, const unsigned long long* ds_count,
                          long long ds_cap) {
  const int n = d.miss_n[0];
  const long long base = (long long)*ds_count;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const long long s = base + r;
    if (s >= ds_cap) break;
    const float4* src = reinterpret_cast<const float4*>(d.mfeat + (size_t)r * mlp::kIn);
    float4* dst = reinterpret_cast<float4*>(ds_feat + (size_t)s * mlp::kIn);
    for (int k = 0; k < 4; ++k) dst[k] = src[k];
    const int c = d.miss_ids[r];
    ds_tgt[2 * s] = (float)d.lam[2 * (size_t)c];
    ds_tgt[2 * s + 1] = (float)d.lam[2 * (size_t)c + 1];
  }
}

__global__ void k_collect_advance(const int32_t* miss_n, unsigned long long* ds_count, long long ds_cap) {
  const unsigned long long next = *ds_count + (unsigned long long)miss_n[0];
  *ds_count = next < (unsigned long long)ds_cap ? next : (unsigned long long)ds_cap;
}

/* Per world: back to the plain start when the residual or the largest depth
 * exceeds its limit (NaN counts as exceeding). */
__global__ void k_learned_judge(Dev d) {
  const int wld = blockIdx.x * blockDim.x + threadIdx.x;
  if (wld >= d.n_worlds || !d.learned_mask[wld]) return;
  const double r = d.world_residual[wld], dep = d.world_depth[wld];
  const bool bad = !(r <= d.judge_res[wld]) || !(dep <= d.judge_depth[wld]);
  if (bad) {
    d.learned_mask[wld] = 0;
    atomicAdd(&d.counters[kCntReverted], 1ull);
  }
}

}  // namespace shapes
