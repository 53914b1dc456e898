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
 * Contacts are in descending (i, j) order with i > j the first body, so a
 * pass is a sequence of rows, one per first body i; within a pass no update
 * after i's row touches i.  A row is one unit of work ("ticket"): one lane
 * waits once for i's earlier updates, keeps i's velocity in registers through
 * the row and waits per contact only for the second body's.  Tickets are
 * handed out in the order p S + r (pass p, row r, S the pass skew: row r of
 * pass p + 1 waits on nothing of pass p at a row >= r + S), which puts every
 * wait on an earlier ticket and lets the tickets in flight cover several
 * passes' wavefronts; the earliest unfinished ticket can always run.  Lanes
 * never block: a warp polls each lane's next dependency once and all lanes
 * whose dependency is met run their update together.  Waits are bounded: past
 * the limit the kernel raises an error flag (SHAPES_E_TIMEOUT) that stays set
 * for the rest of the run, and stops.  Velocities and Lagrangians are read
 * and written at L2 (no stale L1 lines across SMs); a release precedes each
 * counter increment and each met count is read with acquire semantics.
 * Static bodies take no part in the ordering (they are never written).
 * Results are bit-identical to the sequential sweep.
 *
 * Coloured (not the reference's order): contacts are coloured so that no two
 * contacts of a colour share a dynamic body (Jones-Plassmann: a contact takes
 * the smallest colour free among its neighbours once its hash priority beats
 * all uncoloured neighbours), then each pass updates one colour at a time,
 * every contact of a colour in parallel.  Judged against the ordered path by
 * residual and penetration.
 */
#pragma once
#include "lw_order.cuh"
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
  int32_t* color;           /* [nc] */
  int32_t* color_cnt;       /* [kMaxColors + 1] then scanned */
  int32_t* color_list;      /* [nc] contacts grouped by colour */
  int32_t* seqflag;         /* [nc] 1 = left over by the colouring */
  int32_t* seqoff;          /* [nc + 1] scanned seqflag */
  int32_t* seq_list;        /* [nc] left-over contacts in contact order */
  unsigned long long* ctl;  /* [8] ticket, timeout flag, round counter, colours used (coloured) or pass skew
                               (ordered by rows), nc, c0, round counters */
  int32_t* rowflag;         /* [nc] 1 where a contact starts a row (a run of contacts with one first body) */
  int32_t* rowoff;          /* [nc + 1] scanned rowflag: rowoff[nc] rows */
  int32_t* row_start;       /* [rows] first local contact of each row */
  int4* side;               /* [2 nc] per contact side: see k_lw_side */
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
 * through lw_range) and resets the per-step state.  A timeout (ctl[1]) stays
 * raised for the rest of the run: later steps' ordered solves return at once
 * and the host reports the error. */
__global__ void k_lw_setup(Dev d, LW w) {
  const int c0 = d.world_contact_off[w.wld], c1 = d.world_contact_off[w.wld + 1];
  for (int b = blockIdx.x * blockDim.x + threadIdx.x; b <= w.nb; b += gridDim.x * blockDim.x) w.bcnt[b] = 0;
  if (blockIdx.x == 0 && threadIdx.x < 8 && threadIdx.x != 1) { /* ctl[1], the timeout flag, is cleared per run */
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

/* The step's statistics: cache hits and updates (hits + iterations x contacts). */
__global__ void k_lw_item_counts(LW w, unsigned long long* hits, unsigned long long* items, int iterations) {
  lw_range(w);
  atomicAdd(hits, (unsigned long long)w.hitoff[w.nc]);
  atomicAdd(items, (unsigned long long)w.hitoff[w.nc] + (unsigned long long)iterations * (unsigned long long)w.nc);
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

/* One update of a contact from its constants cp, the velocities v of its two
 * bodies (updated in place), the inverse masses m and its accumulated
 * Lagrangians lam2 (Solvers/Contact.hs:74-157; warm = the warm-start pass's
 * application of the cached impulses). */
__device__ __forceinline__ void lw_contact_math(const double2* cp, double v[6], const double m[6], double2* lam2,
                                                bool warm) {
  double j_n[6], j_f[6];
  const double2 a0 = cp[0], a1 = cp[1], a2 = cp[2], a3 = cp[3], a4 = cp[4], a5 = cp[5];
  j_n[0] = a0.x; j_n[1] = a0.y; j_n[2] = a1.x; j_n[3] = a1.y; j_n[4] = a2.x; j_n[5] = a2.y;
  j_f[0] = a3.x; j_f[1] = a3.y; j_f[2] = a4.x; j_f[3] = a4.y; j_f[4] = a5.x; j_f[5] = a5.y;
  const double2 cached = __ldcg(lam2);
  double ln_apply, lf_apply;
  if (warm) {
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
}

/* The update of contact c (global index), with the generic velocity store. */
template <typename Store>
__device__ __forceinline__ void lw_solve_item(const Dev& d, uint32_t item, const Store& vs) {
  const int c = (int)(item & ~kWarmBit);
  const int ga = d.c_ga[c], gb = d.c_gb[c];
  double v[6];
  vs.load(ga, 0, v[0], v[1], v[2]);
  vs.load(gb, 0, v[3], v[4], v[5]);
  const double ima = __ldg(d.iml + ga), ira = __ldg(d.imr + ga), imb = __ldg(d.iml + gb), irb = __ldg(d.imr + gb);
  const double m[6] = {ima, ima, ira, imb, imb, irb};
  lw_contact_math(reinterpret_cast<const double2*>(d.con + c), v, m, reinterpret_cast<double2*>(d.lam) + c,
                  (item & kWarmBit) != 0);
  const uint8_t info = d.c_hit[c];
  if (info & kInfoDynA) vs.store(ga, 0, v[0], v[1], v[2]);
  if (info & kInfoDynB) vs.store(gb, 0, v[3], v[4], v[5]);
}

/* Rows: contacts are in the reference's order, descending (i, j) with i the
 * first body, so the contacts of one first body form a contiguous run. */
__global__ void k_lw_rowflag(Dev d, LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x)
    w.rowflag[k] = (k == 0 || d.c_ga[w.c0 + k] != d.c_ga[w.c0 + k - 1]) ? 1 : 0;
}

__global__ void k_lw_row_list(LW w) {
  lw_range(w);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x)
    if (w.rowflag[k]) w.row_start[w.rowoff[k]] = k;
}

__device__ __forceinline__ int lw_row_of(const LW& w, int k) { return w.rowoff[k] + w.rowflag[k] - 1; }

/* Pass skew S = 1 + the largest (last row of the pass touching body b) - (row
 * of a contact on b), over the contacts' dynamic bodies (ctl[3]).  A body's
 * contacts are refs[bstart[b - 1] .. bstart[b]) in contact order, so its last
 * row is the row of its last ref.  Row r of pass p + 1 then waits on nothing
 * of pass p at a row >= r + S. */
__global__ void k_lw_skew(Dev d, LW w) {
  lw_range(w);
  int best = 0;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < w.nc; k += gridDim.x * blockDim.x) {
    const int r = lw_row_of(w, k);
    for (int s = 0; s < 2; ++s) {
      const int b = lw_body(d, w, k, s);
      if (b >= 0) best = max(best, lw_row_of(w, w.refs[w.bstart[b] - 1] >> 1) - r + 1);
    }
  }
  for (int o = 16; o; o >>= 1) best = max(best, __shfl_xor_sync(0xffffffffu, best, o));
  if ((threadIdx.x & 31) == 0 && best > 0) atomicMax(&w.ctl[3], (unsigned long long)best);
}

/* Per contact side (ref = k << 1 | side): {global body, hr_b(k) or -1 for a
 * static body, h_b - n_b + r_b(k), n_b}, so that the body's completed count
 * wanted before the update of pass p is lw_want(e, p) with one load. */
__global__ void k_lw_side(Dev d, LW w) {
  lw_range(w);
  for (int ref = blockIdx.x * blockDim.x + threadIdx.x; ref < 2 * w.nc; ref += gridDim.x * blockDim.x) {
    const int k = ref >> 1, s = ref & 1;
    const int c = w.c0 + k;
    const int g = s ? d.c_gb[c] : d.c_ga[c];
    const int b = lw_body(d, w, k, s);
    w.side[ref] = b >= 0 ? make_int4(g, w.hrank[ref], w.bh[b] - w.bn[b] + w.rank[ref], w.bn[b])
                         : make_int4(g, -1, 0, 0);
  }
}

__device__ __forceinline__ int lw_want(int4 e, int pass) { return pass == 0 ? e.y : e.z + pass * e.w; }

/* The ordered solve of one large world.  Rows are tickets in the skewed order
 * (lw_ticket); a lane holds one row: it waits for the row's first body i,
 * then runs the row's contacts in order with i's velocity in registers,
 * waiting before each for the second body's earlier updates, and finally
 * stores i's velocity and releases i's counter by the row's update count.
 * No lane blocks: each pass of a warp's loop polls every lane's next
 * dependency once, then all lanes whose dependency is met run their update
 * together (the FP64 pipe charges a warp instruction in full however few
 * lanes it carries, so lanes that spin and then solve alone pay for every
 * update separately).  A lane whose row is finished takes the next ticket on
 * the following pass (one atomic per warp).  The earliest unfinished ticket
 * finds its dependencies met on its warp's next poll, so the solve always
 * progresses; a lane that polls one dependency poll_limit times (default
 * kPollLimit, shapes_batch_set_wait_limit) raises the
 * timeout flag and every warp returns. */
constexpr int kOrderedThreads = 128;
constexpr long long kPollLimit = 1ll << 22; /* polls of one dependency before giving up */
constexpr int kOrderedBlocksPerSM = 2;

__global__ void __launch_bounds__(kOrderedThreads) k_lw_ordered(Dev d, LW w, int iterations, int warm_start,
                                                                  long long poll_limit) {
  if (d.counters[kCntOverflow]) return;
  lw_range(w);
  const unsigned kAll = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int n_rows = w.rowoff[w.nc];
  const int passes = warm_start ? iterations + 1 : iterations;
  const long long total = (long long)passes * n_rows;
  const int skew = max(1, min((int)w.ctl[3], n_rows));
  bool has = false, exhausted = total == 0, dyn_i = false;
  int stage = 0, pass = 0, k = 0, k1 = 0, m = 0, gi = 0, want_i = 0;
  int4 cur = make_int4(0, -1, 0, 0); /* side entry of contact k's second body */
  double vi[3] = {0.0, 0.0, 0.0}, ima = 0.0, ira = 0.0;
  long long polls = 0;
  int empty = 0;
  for (;;) {
    if (!exhausted) { /* lanes without a row take the next tickets, in order */
      const unsigned need = __ballot_sync(kAll, !has);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(&w.ctl[0], (unsigned long long)__popc(need));
        base = __shfl_sync(kAll, base, leader);
        const long long t = (long long)base + __popc(need & below);
        if (!has && t < total) {
          int pi, r;
          lw_ticket(t, passes, skew, n_rows, pi, r);
          pass = pi + (warm_start ? 0 : 1);
          const int k0 = w.row_start[r];
          k1 = r + 1 < n_rows ? w.row_start[r + 1] : w.nc;
          k = k0;
          m = k1 - k0;
          if (pass == 0) { /* the warm-start pass updates the cache hits only */
            while (k < k1 && !w.hitflag[k]) ++k;
            m = 0;
            for (int x = k; x < k1; ++x) m += w.hitflag[x];
          }
          if (m > 0) {
            has = true;
            stage = 0;
            polls = 0;
            const int4 e0 = w.side[k << 1];
            gi = e0.x;
            dyn_i = e0.y >= 0;
            want_i = lw_want(e0, pass);
            ima = __ldg(d.iml + gi);
            ira = __ldg(d.imr + gi);
            cur = w.side[(k << 1) | 1];
          }
        }
        if ((long long)base + __popc(need) >= total) exhausted = true;
      }
    }
    if (exhausted && !__any_sync(kAll, has)) break;
    /* poll each lane's next dependency once */
    bool ready = false;
    if (has && stage == 0 && (!dyn_i || ld_acquire_gpu(w.done + (gi - w.b0)) == want_i)) {
      vi[0] = __ldcg(d.vx + gi);
      vi[1] = __ldcg(d.vy + gi);
      vi[2] = __ldcg(d.w + gi);
      stage = 1;
      polls = 0;
    }
    const bool dyn_j = cur.y >= 0;
    if (has && stage == 1) ready = !dyn_j || ld_acquire_gpu(w.done + (cur.x - w.b0)) == lw_want(cur, pass);
    /* the ready lanes' updates, together */
    if (ready) {
      int kn = k + 1; /* the next contact's side entry, fetched beside the update */
      if (pass == 0)
        while (kn < k1 && !w.hitflag[kn]) ++kn;
      const int4 nxt = kn < k1 ? w.side[(kn << 1) | 1] : cur;
      const int c = w.c0 + k, gb = cur.x;
      double v[6] = {vi[0], vi[1], vi[2], __ldcg(d.vx + gb), __ldcg(d.vy + gb), __ldcg(d.w + gb)};
      const double imb = __ldg(d.iml + gb), irb = __ldg(d.imr + gb);
      const double mm[6] = {ima, ima, ira, imb, imb, irb};
      lw_contact_math(reinterpret_cast<const double2*>(d.con + c), v, mm, reinterpret_cast<double2*>(d.lam) + c,
                      pass == 0);
      if (dyn_i) {
        vi[0] = v[0];
        vi[1] = v[1];
        vi[2] = v[2];
      }
      if (dyn_j) {
        __stcg(d.vx + gb, v[3]);
        __stcg(d.vy + gb, v[4]);
        __stcg(d.w + gb, v[5]);
        red_release_gpu_add(w.done + (gb - w.b0), 1);
      }
      k = kn;
      cur = nxt;
      polls = 0;
      if (k >= k1) {
        if (dyn_i) {
          __stcg(d.vx + gi, vi[0]);
          __stcg(d.vy + gi, vi[1]);
          __stcg(d.w + gi, vi[2]);
          red_release_gpu_add(w.done + (gi - w.b0), m); /* release: the row's writes of i before the counter */
        }
        has = false;
      }
    } else if (has && ++polls > poll_limit) {
      atomicExch(&w.ctl[1], 1ull);
    }
    if (!__any_sync(kAll, ready)) {
      const unsigned long long flag = *reinterpret_cast<volatile unsigned long long*>(&w.ctl[1]);
      if (__shfl_sync(kAll, flag, 0)) break; /* an update timed out */
      if (++empty > 16) __nanosleep(64);
    } else {
      empty = 0;
    }
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
