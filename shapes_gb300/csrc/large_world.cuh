/*
 * Solver paths for one very large world (hundreds of thousands of bodies),
 * where a warp per world cannot expose the parallelism.
 *
 * Ordered (exact): the reference's sequence of updates — warm-start pass over
 * the cache hits, then `iterations` sweeps, each in contact order
 * (Solvers/Contact.hs:74-157) — is executed as a dataflow.  Update u touching
 * body a must run after every earlier update on a.  If r_a(u) is the number of
 * earlier updates on a, u may run exactly when a's completion counter equals
 * r_a(u).  The ranks come from each body's contacts sorted by contact order:
 * for a contact k at position r_a(k) in a's list, with h_a of a's contacts
 * being cache hits (hr_a(k) of them before k) and n_a contacts in all,
 *   warm-start pass:  r = hr_a(k)
 *   sweep p (1-based): r = h_a + (p - 1) n_a + r_a(k).
 * A persistent kernel hands out updates in sequential order; every update
 * waits only on earlier ones, all of which are already held by resident warps,
 * so the earliest unfinished update can always run.  Waits are bounded: past
 * the limit the kernel raises an error flag (SHAPES_E_TIMEOUT) and stops.
 * Velocities and Lagrangians are read and written at L2 (no stale L1 lines
 * across SMs); a release fence precedes each counter increment and an acquire
 * fence follows each successful wait.  Static bodies take no part in the
 * ordering (they are never written).  Results are bit-identical to the
 * sequential sweep.
 *
 * Coloured (not the reference's order): contacts are coloured so that no two
 * contacts of a colour share a dynamic body (Jones-Plassmann: a contact takes
 * the smallest colour free among its neighbours once its hash priority beats
 * all uncoloured neighbours), then each pass updates one colour at a time,
 * every contact of a colour in parallel.  Judged against the ordered path by
 * residual and penetration.
 */
#pragma once
#include "step_kernels.cuh"

namespace shapes {

/* Per large world scratch (device). */
struct LW {
  int wld;                  /* the world */
  int b0, nb;               /* bodies [b0, b0 + nb) */
  int c0, nc;               /* contacts [c0, c0 + nc): set on the device by k_lw_setup */
  int32_t* bcnt;            /* [nb + 1] refs per body, then scanned starts, then ends */
  int32_t* bstart;          /* [nb + 1] */
  int32_t* refs;            /* [2 nc] (local contact << 1 | side), grouped by body */
  int32_t* rank;            /* [2 nc] r_s(k) */
  int32_t* hrank;           /* [2 nc] hr_s(k) */
  int32_t* bh;              /* [nb] hits per body */
  int32_t* bn;              /* [nb] contacts per body */
  int32_t* done;            /* [nb] completed updates per body */
  int32_t* hitflag;         /* [nc] */
  int32_t* hitoff;          /* [nc + 1] scanned */
  int32_t* hit_idx;         /* [nc] local contact of the h-th hit */
  int32_t* color;           /* [nc] */
  int32_t* color_cnt;       /* [kMaxColors + 1] then scanned */
  int32_t* color_list;      /* [nc] contacts grouped by colour */
  int32_t* seqflag;         /* [nc] 1 = left over by the colouring */
  int32_t* seqoff;          /* [nc + 1] scanned seqflag */
  int32_t* seq_list;        /* [nc] left-over contacts in contact order */
  unsigned long long* ctl;  /* [8] ticket, timeout flag, round counter, colours used, nc, c0, round counters */
};

__device__ __forceinline__ int32_t ld_acquire_gpu(const int32_t* p) {
  int32_t v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void red_release_gpu_add(int32_t* p, int32_t v) {
  asm volatile("red.release.gpu.global.add.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int kMaxColors = 64;
constexpr int kSeqColor = kMaxColors - 1; /* contacts left over by the colouring: updated one by one */

/* Reads the world's contact range from the device (kernels read w.c0 / w.nc
 * through lw_range) and resets the per-step state. */
__global__ void k_lw_setup(Dev d, LW w) {
  const int c0 = d.world_contact_off[w.wld], c1 = d.world_contact_off[w.wld + 1];
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= w.nb; b += gridDim.x * blockDim.x) w.bcnt[b] = 0;
  if (blockIdx.x == 0 && threadIdx.x < 8) {
    const int t = threadIdx.x;
    w.ctl[t] = t == 4 ? (unsigned long long)(c1 - c0) : (t == 5 ? (unsigned long long)c0 : 0ull);
  }
  if (blockIdx.x == 0) {
    for (int t = threadIdx.x; t <= kMaxColors; t += blockDim.x) w.color_cnt[t] = 0;
  }
}

__device__ __forceinline__ void lw_range(LW& w) {
  w.nc = (int)w.ctl[4];
  w.c0 = (int)w.ctl[5];
}
constexpr long long kSpinLimit = 1ll << 26;

/* Body of a contact side, or -1 for a static body (no ordering). */
__device__ __forceinline__ int lw_body(const Dev& d, const LW& w, int k, int side) {
  const int c = w.c0 + k;
  const uint8_t info = d.c_hit[c];
  if (side == 0) return (info & kInfoDynA) ? d.c_ga[c] - w.b0 : -1;
  return (info & kInfoDynB) ? d.c_gb[c] - w.b0 : -1;
}

__global__ void k_lw_count(Dev d, LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) {
    const int c = w.c0 + k;
    w.hitflag[k] = (d.c_hit[c] & kInfoHit) ? 1 : 0;
    for (int s = 0; s < 2; ++s) {
      const int b = lw_body(d, w, k, s);
      if (b >= 0) atomicAdd(&w.bcnt[b], 1);
    }
  }
}

/* bstart holds exclusive starts; the atomics turn them into ends. */
__global__ void k_lw_scatter(Dev d, LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) {
    for (int s = 0; s < 2; ++s) {
      const int b = lw_body(d, w, k, s);
      if (b >= 0) w.refs[atomicAdd(&w.bstart[b], 1)] = (k << 1) | s;
    }
  }
}

/* One thread per body: sort its refs by contact order, then ranks. */
__global__ void k_lw_rank(Dev d, LW w) {
  lw_range(w);
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.nb; b += gridDim.x * blockDim.x) {
    const int r0 = b > 0 ? w.bstart[b - 1] : 0, r1 = w.bstart[b];
    for (int x = r0 + 1; x < r1; ++x) {
      const int v = w.refs[x];
      int y = x - 1;
      while (y >= r0 && w.refs[y] > v) {
        w.refs[y + 1] = w.refs[y];
        --y;
      }
      w.refs[y + 1] = v;
    }
    int hits = 0;
    for (int x = r0; x < r1; ++x) {
      const int ref = w.refs[x];
      w.rank[ref] = x - r0;
      w.hrank[ref] = hits;
      hits += w.hitflag[ref >> 1];
    }
    w.bh[b] = hits;
    w.bn[b] = r1 - r0;
    w.done[b] = 0;
  }
}

__global__ void k_lw_hit_list(LW w, unsigned long long* hits, unsigned long long* items, int iterations) {
  lw_range(w);
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    atomicAdd(hits, (unsigned long long)w.hitoff[w.nc]);
    atomicAdd(items, (unsigned long long)w.hitoff[w.nc] + (unsigned long long)iterations * (unsigned long long)w.nc);
  }
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x)
    if (w.hitflag[k]) w.hit_idx[w.hitoff[k]] = k;
}

__global__ void k_lw_gravity(Dev d, LW w, double ax, double ay, double dt) {
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b < w.nb; b += gridDim.x * blockDim.x) {
    const int g = w.b0 + b;
    if (!(0.0 == d.iml[g]) && !(d.flags[g] & kFlagInactive)) {
      d.vx[g] = d.vx[g] + ax * dt;
      d.vy[g] = d.vy[g] + ay * dt;
    }
  }
}

/* Global velocities read and written at L2, for updates running on any SM. */
struct L2Vel {
  const Dev* d;
  __device__ __forceinline__ void load(int g, int, double& x, double& y, double& w) const {
    x = __ldcg(d->vx + g);
    y = __ldcg(d->vy + g);
    w = __ldcg(d->w + g);
  }
  __device__ __forceinline__ void store(int g, int, double x, double y, double w) const {
    __stcg(d->vx + g, x);
    __stcg(d->vy + g, y);
    __stcg(d->w + g, w);
  }
};

/* The update of contact c (global index), with the generic velocity store. */
template <typename Store>
__device__ __forceinline__ void lw_solve_item(const Dev& d, uint32_t item, const Store& vs) {
  const int c = (int)(item & ~kWarmBit);
  const int ga = d.c_ga[c], gb = d.c_gb[c];
  const double2* cp = reinterpret_cast<const double2*>(d.con + c);
  double j_n[6], j_f[6];
  const double2 a0 = cp[0], a1 = cp[1], a2 = cp[2], a3 = cp[3], a4 = cp[4], a5 = cp[5];
  j_n[0] = a0.x; j_n[1] = a0.y; j_n[2] = a1.x; j_n[3] = a1.y; j_n[4] = a2.x; j_n[5] = a2.y;
  j_f[0] = a3.x; j_f[1] = a3.y; j_f[2] = a4.x; j_f[3] = a4.y; j_f[4] = a5.x; j_f[5] = a5.y;
  double v[6];
  vs.load(ga, 0, v[0], v[1], v[2]);
  vs.load(gb, 0, v[3], v[4], v[5]);
  const double ima = __ldg(d.iml + ga), ira = __ldg(d.imr + ga), imb = __ldg(d.iml + gb), irb = __ldg(d.imr + gb);
  const double m[6] = {ima, ima, ira, imb, imb, irb};
  double2* lam2 = reinterpret_cast<double2*>(d.lam) + c;
  const double2 cached = __ldcg(lam2);
  double ln_apply, lf_apply;
  if (item & kWarmBit) {
    ln_apply = cached.x;
    lf_apply = cached.y;
  } else {
    const double2 b6 = cp[6], b9 = cp[9], b10 = cp[10], b11 = cp[11], b12 = cp[12];
    const double cn = cached.x, cf = cached.y;
    const uint64_t ebits = (uint64_t)__double_as_longlong(b11.y) & 0x7fffffffffffffffull;
    const bool fastflag = __double_as_longlong(cp[13].x) != 0;
    double bias;
    if (ebits == 0 && fastflag && small_mag(v[0]) && small_mag(v[1]) && small_mag(v[2]) && small_mag(v[3]) &&
        small_mag(v[4]) && small_mag(v[5])) {
      bias = b6.y;
    } else {
      const double2 b7 = cp[7], b8 = cp[8];
      const double nwa = -v[2];
      const double cvx = ((-v[0] + (-(nwa * b7.y))) + v[3]) + (-(v[5] * b8.y));
      const double cvy = ((-v[1] + nwa * b7.x) + v[4]) + v[5] * b8.x;
      const double tb = b11.y * (cvx * b9.x + cvy * b9.y);
      bias = b6.x + (f_le(0.0, tb) ? 0.0 : tb);
    }
    const double ln_new = div_rn(-(dot6(j_n, v) + bias), b10.x, b12.x);
    const double lf_new = div_rn(-plus_zero(dot6(j_f, v)), b10.y, b12.y);
    const double neg_cn = -cn;
    ln_apply = f_le(ln_new, neg_cn) ? neg_cn : ln_new;
    const double ln_cache = cn + ln_apply;
    const double thr = ln_cache * b11.x;
    const double acc = cf + lf_new;
    const double acc2 = f_lt(thr, acc) ? thr : (f_lt(acc, -thr) ? -thr : acc);
    lf_apply = acc2 - cf;
    __stcg(lam2, make_double2(ln_cache, acc2));
  }
  apply_impulse(j_n, ln_apply, v, m);
  apply_impulse(j_f, lf_apply, v, m);
  const uint8_t info = d.c_hit[c];
  if (info & kInfoDynA) vs.store(ga, 0, v[0], v[1], v[2]);
  if (info & kInfoDynB) vs.store(gb, 0, v[3], v[4], v[5]);
}

/* Persistent dataflow solver for one large world: updates in the reference's
 * sequential order, each waiting (bounded) for its bodies' earlier updates. */
__global__ void k_lw_ordered(Dev d, LW w, int iterations, int warm_start) {
  if (d.counters[kCntOverflow]) return;
  lw_range(w);
  const int lane = threadIdx.x & 31;
  const long long H = warm_start ? (long long)w.hitoff[w.nc] : 0;
  const long long total = H + (long long)iterations * w.nc;
  for (;;) {
    long long base = 0;
    if (lane == 0) base = (long long)atomicAdd(&w.ctl[0], 32ull);
    base = __shfl_sync(0xffffffffu, base, 0);
    if (base >= total) break;
    if (*reinterpret_cast<volatile unsigned long long*>(&w.ctl[1])) break; /* another update timed out */
    const long long u = base + lane;
    if (u < total) {
      int k, pass;
      if (u < H) {
        pass = 0;
        k = w.hit_idx[u];
      } else {
        pass = 1 + (int)((u - H) / w.nc);
        k = (int)((u - H) % w.nc);
      }
      int body[2], want[2];
      for (int s = 0; s < 2; ++s) {
        body[s] = lw_body(d, w, k, s);
        if (body[s] >= 0) {
          const int ref = (k << 1) | s;
          want[s] = pass == 0 ? w.hrank[ref] : w.bh[body[s]] + (pass - 1) * w.bn[body[s]] + w.rank[ref];
        }
      }
      /* acquire loads of the predecessors' counters (their velocity writes,
       * released with the counter increment, are visible after the load
       * that sees the wanted count); a short tight spin, then backing off */
      bool ok = true;
      for (int s = 0; s < 2 && ok; ++s) {
        if (body[s] < 0) continue;
        const int32_t* cnt = w.done + body[s];
        long long spins = 0;
        while (ld_acquire_gpu(cnt) != want[s]) {
          if (++spins > kSpinLimit) {
            ok = false;
            break;
          }
          if (spins > 64) __nanosleep(32);
        }
      }
      if (!ok) {
        atomicExch(&w.ctl[1], 1ull);
      } else {
        lw_solve_item(d, (uint32_t)(w.c0 + k) | (pass == 0 ? kWarmBit : 0u), L2Vel{&d});
        /* release: this update's velocity writes before the counters move */
        for (int s = 0; s < 2; ++s)
          if (body[s] >= 0) red_release_gpu_add(w.done + body[s], 1);
      }
    }
    __syncwarp();
  }
}

/* Jones-Plassmann colouring round over the contact graph. */
__device__ __forceinline__ uint32_t lw_prio(int k) {
  uint32_t x = (uint32_t)k * 0x9e3779b1u;
  x ^= x >> 15;
  x *= 0x85ebca6bu;
  x ^= x >> 13;
  return x;
}

/* Round r of the colouring counts the contacts it leaves uncoloured in
 * ctl[slot(r)], slots rotating over ctl[2], ctl[6], ctl[7]: round r reads
 * slot(r - 1) (a round after one that left none returns at once, so the host
 * can launch a generous number of rounds), counts into slot(r), and clears
 * slot(r + 1), which no block of round r reads. */
__device__ __forceinline__ unsigned long long* lw_round_slot(const LW& w, int round) {
  const int m = round % 3;
  return w.ctl + (m == 0 ? 2 : (m == 1 ? 6 : 7));
}

__global__ void k_lw_color_round(Dev d, LW w, int round) {
  lw_range(w);
  if (round > 0 && *lw_round_slot(w, round - 1) == 0) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) *lw_round_slot(w, round + 1) = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) {
    if (w.color[k] >= 0) continue;
    const uint64_t mine = ((uint64_t)lw_prio(k) << 32) | (uint32_t)k;
    bool top = true;
    uint64_t used = 0;
    for (int s = 0; s < 2 && top; ++s) {
      const int b = lw_body(d, w, k, s);
      if (b < 0) continue;
      const int r0 = b > 0 ? w.bstart[b - 1] : 0, r1 = w.bstart[b];
      for (int x = r0; x < r1; ++x) {
        const int k2 = w.refs[x] >> 1;
        if (k2 == k) continue;
        const int col = w.color[k2];
        if (col < 0) {
          const uint64_t other = ((uint64_t)lw_prio(k2) << 32) | (uint32_t)k2;
          if (other > mine) {
            top = false;
            break;
          }
        } else if (col < kSeqColor) {
          used |= 1ull << col;
        }
      }
    }
    if (!top) {
      atomicAdd(lw_round_slot(w, round), 1ull);
      continue;
    }
    int col = __ffsll((long long)~used) - 1;
    if (col < 0 || col >= kSeqColor) col = kSeqColor;
    w.color[k] = col;
    atomicMax(&w.ctl[3], (unsigned long long)(col + 1));
  }
}

/* After the rounds, contacts still uncoloured go to the sequential colour. */
__global__ void k_lw_color_count(LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) {
    if (w.color[k] < 0) w.color[k] = kSeqColor;
    atomicAdd(&w.color_cnt[w.color[k]], 1);
    w.seqflag[k] = w.color[k] == kSeqColor ? 1 : 0;
  }
}

__global__ void k_lw_color_init(LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) w.color[k] = -1;
}

__global__ void k_lw_color_scatter(LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x)
    w.color_list[atomicAdd(&w.color_cnt[w.color[k]], 1)] = k;
}

/* Global velocities with plain loads/stores (one colour per launch: no other
 * update of the launch touches the same body). */
struct GlobalVel {
  const Dev* d;
  __device__ __forceinline__ void load(int g, int, double& x, double& y, double& w) const {
    x = d->vx[g];
    y = d->vy[g];
    w = d->w[g];
  }
  __device__ __forceinline__ void store(int g, int, double x, double y, double w) const {
    d->vx[g] = x;
    d->vy[g] = y;
    d->w[g] = w;
  }
};

/* The left-over contacts, in contact order (ordered compaction of seqflag). */
__global__ void k_lw_seq_list(LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x)
    if (w.seqflag[k]) w.seq_list[w.seqoff[k]] = k;
}

/* One colour of one pass: contacts [lo, hi) of the colour list.  The
 * left-over contacts run on one thread in contact order. */
__global__ void k_lw_color_seq(Dev d, LW w, int warm) {
  if (d.counters[kCntOverflow]) return;
  lw_range(w);
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int n = w.seqoff[w.nc];
  for (int t = 0; t < n; ++t) {
    const int k = w.seq_list[t];
    const int c = w.c0 + k;
    if (warm && !(d.c_hit[c] & kInfoHit)) continue;
    lw_solve_item(d, (uint32_t)c | (warm ? kWarmBit : 0u), GlobalVel{&d});
  }
}

__global__ void k_lw_color_pass(Dev d, LW w, int lo_color, int warm) {
  if (d.counters[kCntOverflow]) return;
  lw_range(w);
  const int lo = lo_color > 0 ? w.color_cnt[lo_color - 1] : 0, hi = w.color_cnt[lo_color];
  for (int t = lo + blockIdx.x * blockDim.x + threadIdx.x; t < hi; t += gridDim.x * blockDim.x) {
    const int k = w.color_list[t];
    const int c = w.c0 + k;
    if (warm && !(d.c_hit[c] & kInfoHit)) continue;
    lw_solve_item(d, (uint32_t)c | (warm ? kWarmBit : 0u), GlobalVel{&d});
  }
}

}  // namespace shapes
