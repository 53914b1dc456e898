/*
 * Device kernels of the GB300 world step.
 *
 * Arithmetic contract (shared with the CPU oracle): IEEE binary64, every sum a
 * left fold in the reference's source order, no contraction (-fmad=false), the
 * reference's comparison spellings.  Floating-point comparisons whose only job
 * is ordering (AABB overlap) are done on order-preserving 64-bit integer keys,
 * which give the same answers as the IEEE comparisons for every non-NaN value;
 * NaN operands take the IEEE path.  On GB300 the FP64 pipe retires about 0.05
 * warp-instructions per clock per SM and charges masked-off lanes in full, so
 * every kernel here keeps warps full across its FP64 work and moves what it
 * can to the integer pipes.
 */
#pragma once
#include <cstdint>

#include "fp64_ops.cuh"
#include "shapes_sincos.h"

namespace shapes {

constexpr int kMaxVerts = 64;
constexpr uint32_t kWarmBit = 0x80000000u;
constexpr uint8_t kFlagStatic = 1;
constexpr uint8_t kFlagBoxNaN = 2;
constexpr uint8_t kFlagInactive = 4; /* empty slot (World.delete): no pairs, no motion */
constexpr uint8_t kFlagCircle = 8;
/* per-contact info byte */
constexpr uint8_t kInfoHit = 1;
constexpr uint8_t kInfoDynA = 2;
constexpr uint8_t kInfoDynB = 4;

/* Per-contact constraint data, built once per step (constraintGen,
 * Constraints/Contact.hs:60-72) plus the step-invariant factors of the solver:
 * effective-mass denominators (effMassM2, Constraint.hs:173-179), pairMu
 * (Friction.hs:46-48) and min bounciness (Restitution.hs:51). */
struct __align__(16) Con {
  double jn[6];
  double jf[6];
  double bn, bn0; /* baumgarte term, and bn + 0.0 */
  double rax, ray, rbx, rby, rnx, rny;
  double mcn, mcf; /* effective-mass denominators */
  double mu;
  double e;
  double rcn, rcf; /* RN(1/mcn), RN(1/mcf) for div_rn, or 0 when out of its range */
  double fast;     /* 1 when both radii are below 2^500 and the normal below 2 (exact zero-bounce path) */
  double pad;
};

/* Device view of a batch; passed by value to every kernel. */
struct Dev {
  int32_t n_worlds, n_bodies, n_verts;
  int32_t pair_cap, contact_cap, item_cap;
  const int32_t* world_body_off; /* [W+1] */
  const int32_t* body_world;     /* [N] */
  const int32_t* vert_off;       /* [N+1] */
  const double* lx;
  const double* ly;
  int32_t* emin;
  int32_t* emax;
  double* vx;
  double* vy;
  double* w;
  double* px;
  double* py;
  double* th;
  const double* iml;
  const double* imr;
  const double* mu;
  const double* bounce;
  double* wx;
  double* wy;
  double* nx;
  double* ny;
  double* plo;      /* [V] per edge e: projection of vertex emin[e] on normal e (null: SAT computes it) */
  double* phi;      /* [V] per edge e: projection of vertex emax[e] on normal e */
  double* box;      /* [4N] x0 x1 y0 y1 */
  uint64_t* boxk;   /* [4N] ordered keys of box */
  uint8_t* flags;   /* [N] */
  /* grid broadphase (worlds with grid_T[w] > 0) */
  const int32_t* grid_T;    /* [W] bucket table size (power of two), 0 = brute force */
  const int32_t* grid_base; /* [W] first bucket of the world */
  double* grid_inv_s;       /* [W] 1 / cell size, 0 = no usable grid this step */
  double* grid_lim;         /* [W] (1 - 2^-20) * cell size: bodies below it in x and y use the grid */
  int32_t* bucket_cnt;      /* [n_buckets + 1] counts, then scanned offsets */
  int32_t* bucket_off;      /* [n_buckets + 1] */
  int32_t* grid_ids;        /* [N] body ids sorted by bucket */
  int32_t* cell_x;          /* [N] */
  int32_t* cell_y;          /* [N] */
  uint8_t* row_mode;        /* [N] 1 = row found through the grid */
  int32_t* large_cnt;       /* [W] bodies of the world off the grid */
  int32_t* large_ids;       /* [N] per-world region at world_body_off[w] */
  int32_t n_buckets;
  /* incremental grid pairs (fat boxes); null when off */
  uint64_t* fatk;        /* [4N] ordered keys of each grid body's fat box */
  int32_t* nbr;          /* [N * nbr_cap] bodies whose fat boxes overlap (either index); -1 = removed */
  int32_t* nbr_cnt;      /* [N] entries used in nbr */
  uint8_t* moved;        /* [N] kMoved* bits of this frame */
  int32_t* inc_state;    /* [W] 0 = rebuild the adjacency next frame, 1 = valid */
  int32_t* inc_rebuild;  /* [W] this frame rebuilds the world's adjacency */
  int32_t* inc_moved;    /* [W] bodies re-inserted this frame */
  int32_t* inc_frames;   /* [W] consecutive quiet frames of a FULL world */
  double* inc_margin;    /* [W] fat-box margin */
  int32_t nbr_cap;
  int32_t* row_cnt; /* [N] mirrored per-row pair counts */
  int32_t* row_off; /* [N+1] scanned */
  int32_t* pair_a;  /* [pair_cap] global body index, the larger */
  int32_t* pair_b;  /* [pair_cap] */
  int32_t* slot_cnt;   /* [pair_cap] contacts per pair (0..2) */
  int32_t* slot_off;   /* [pair_cap+1] scanned */
  int32_t* slot_feat;  /* [2*pair_cap] fa | fb<<12 | flip<<24 */
  int32_t* np_perm;    /* [pair_cap] pairs in processing order, grouped by vertex-count class */
  const int32_t* ext_chunk;     /* [2 * n_ext_chunks] body range [b0, b1) of each extent-reduction chunk */
  const int32_t* ext_chunk_off; /* [n_worlds + 1] each world's chunks */
  double* ext_part_sum;         /* [n_ext_chunks] chunk sums of box extents */
  int32_t* ext_part_cnt;        /* [n_ext_chunks] chunk counts */
  int32_t n_ext_chunks;
  const uint8_t* world_sap; /* [n_worlds] 1: the world's small bodies pair by sweep and prune (null: none) */
  const int32_t* sap_base;  /* [n_worlds] first of the world's kSapBuckets buckets */
  int32_t* sap_cnt;         /* [n_sap_buckets + 1] bucket counts */
  int32_t* sap_off;         /* [n_sap_buckets + 1] their exclusive scan: bucket starts, then ends */
  int32_t n_sap_buckets;
  int32_t* sap_ids;         /* [n_bodies] small bodies of sweep worlds, in bucket order */
  int32_t* sap_qs;          /* [n_bodies] their buckets, in the same order */
  int32_t* sap_cursor;      /* [n_bodies] per row (mirrored index): the next free slot of the row */
  uint64_t* sap_range;      /* [2 * n_worlds] min and max order key of the small bodies' lower x */
  int32_t* sap_end;         /* [n_worlds] end of the world's run in sap_ids */
  const int32_t* pose_order; /* [n_bodies] pose-kernel order: within chunks of 1024 bodies, grouped by vertex
                                count, so that a warp's vertex loops have one length (null: index order) */
  int32_t* np_cls;     /* [2 * kNpClasses + 1] class counts, then offsets and cursors */
  double* slot_val;    /* [2*pair_cap*5] nx ny px py depth */
  uint64_t* c_key;     /* [contact_cap] packed world-local key */
  int32_t* c_ga;       /* [contact_cap] */
  int32_t* c_slot;     /* [contact_cap] each contact's slot t = 2 pair + s (k_contact_slots), or null */
  int32_t* c_gb;       /* [contact_cap] */
  uint8_t* c_flip;     /* [contact_cap] */
  uint8_t* c_hit;      /* [contact_cap] kInfo* bits */
  double* c_val;       /* [contact_cap*5] */
  Con* con;            /* [contact_cap] */
  double* lam;         /* [2*contact_cap] this step's cache Lagrangians */
  const uint64_t* old_key; /* previous cache keys */
  const double* old_lam;   /* previous cache Lagrangians */
  const int32_t* old_cwo;  /* [W+1] previous cache world offsets */
  int32_t* world_pair_off;    /* [W+1] */
  int32_t* world_contact_off; /* [W+1] */
  int32_t* last;              /* [N] scheduler scratch */
  int32_t* last_hit;          /* [N] scheduler scratch: last cache-hit contact of each body */
  int4* c_pred;               /* [contact_cap] per contact: previous contact touching side a, side b; previous hit contact of a, b (-1: none) */
  int32_t* c_lvl;             /* [2 * contact_cap] levels of the current and the previous pass */
  uint32_t* items;            /* [item_cap] */
  int32_t* ilevel;            /* [item_cap] */
  uint32_t* isorted;          /* [item_cap] */
  int32_t* ihist;             /* [item_cap] (unused by the warp-group solver) */
  int4* gdesc;                /* [item_cap + W + 1] per-group updates sorted by level: {id, a, b, info | world << 8} */
  int4* idesc;                /* [item_cap] the same descriptors in sequential order, per world region */
  long long* phase_clock;     /* [G * 8] per-group phase clocks when profiling, else null */
  int32_t* ghist;             /* [item_cap + W + 1] per-group level ends */
  int32_t* world_levels;      /* [W] dependency levels of each small world's last solve */
  int32_t* group_depth;       /* [G] */
  const int32_t* group_world_off; /* [G+1] offsets into group_worlds */
  const int32_t* group_worlds;    /* [W] world ids, grouped */
  unsigned long long* counters;   /* [kCntSlots] see kCnt* */
  double* world_residual;         /* [W] */
  double* world_depth;            /* [W] */
  /* learned warm start (null / zero when off) */
  uint8_t* learned_mask;       /* [W] 1 = contacts without a cache entry start from the network */
  int32_t* miss_flag;          /* [contact_cap] 1 = contact gets a feature row */
  int32_t* miss_off;           /* [contact_cap + 1] scanned miss_flag */
  int32_t* miss_ids;           /* [contact_cap] contact of each row */
  int32_t* miss_n;             /* [1] rows this step */
  float* mfeat;                /* [contact_cap x 16] raw features */
  int32_t collect_all;         /* 1 = rows for every world's misses (sample collection) */
  const double* judge_res;     /* [W] residual limit of the judge */
  const double* judge_depth;   /* [W] depth limit of the judge */
  const uint8_t* active;       /* [N] 0 = empty slot (World.delete); null when every slot is filled */
  const double* radius;        /* [N] > 0: a circle (one local point, the centre); 0: a hull */
};

enum {
  kCntPairs = 0,
  kCntContacts = 1,
  kCntHits = 2,
  kCntItems = 3,
  kCntLevels = 4,
  kCntOverflow = 5,
  kCntBadInput = 6,
  kCntGroupAlloc = 7, /* bump allocator of the per-group regions (reset every step) */
  kCntPredicted = 8,  /* contacts started from the network (summed over the call) */
  kCntReverted = 9,   /* worlds the judge switched back to the plain start */
  kCntMlpErr = 10,    /* set when a tensor-core wait of the network gave up */
  kCntSlots = 16,
};

/* Narrowphase work classes: (min(nv_a, 9) - 3) * 7 + (min(nv_b, 9) - 3). */
constexpr int kNpHullClasses = 49;            /* hull pairs by vertex counts 3..9+ each */
constexpr int kNpClasses = kNpHullClasses + 15; /* then circle-circle, circle-hull, hull-circle */

/* Flags any non-finite value among n bodies' ten state arrays. */
__global__ void k_check_finite(const double* a0, const double* a1, const double* a2, const double* a3,
                               const double* a4, const double* a5, const double* a6, const double* a7,
                               const double* a8, const double* a9, int n, unsigned long long* flag) {
  const double* arr[10] = {a0, a1, a2, a3, a4, a5, a6, a7, a8, a9};
  bool bad = false;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < 10LL * n;
       t += (long long)gridDim.x * blockDim.x) {
    const double v = arr[t / n][t % n];
    bad |= !isfinite(v);
  }
  if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1ull);
}

/* Ten arrays of n doubles copied in one launch (blockIdx.y = array), with an
 * optional finiteness check of what passes through.  Either side may be
 * pinned host memory mapped into the device address space: on a Grace host
 * the loads and stores then cross NVLink-C2C from every SM at once instead of
 * through the copy engines. */
struct Ptr10 {
  const double* src[10];
  double* dst[10];
};

/* Ten arrays of n doubles, array blockIdx.y; non-finite values set *bad_flag.
 * When both ends are 16-byte aligned each thread keeps four 16-byte loads in
 * flight, so a copy over the host link needs few blocks (copy10_grid sizes
 * the grid for kCopy10PerThread doubles a thread) and leaves the SMs to the
 * steps of other handles. */
constexpr int kCopy10PerThread = 8;

__global__ void k_copy10(Ptr10 p, int n, unsigned long long* bad_flag) {
  const double* __restrict__ src = p.src[blockIdx.y];
  double* __restrict__ dst = p.dst[blockIdx.y];
  bool bad = false;
  const int stride = gridDim.x * blockDim.x;
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
    const double2* __restrict__ s2 = reinterpret_cast<const double2*>(src);
    double2* __restrict__ d2 = reinterpret_cast<double2*>(dst);
    const int n2 = n >> 1;
    for (; i + 3 * stride < n2; i += 4 * stride) {
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = s2[i + u * stride];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        bad |= !isfinite(v[u].x) || !isfinite(v[u].y);
        d2[i + u * stride] = v[u];
      }
    }
    for (; i < n2; i += stride) {
      const double2 v = s2[i];
      bad |= !isfinite(v.x) || !isfinite(v.y);
      d2[i] = v;
    }
    if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
      const double v = src[n - 1];
      bad |= !isfinite(v);
      dst[n - 1] = v;
    }
  } else {
    for (; i < n; i += stride) {
      const double v = src[i];
      bad |= !isfinite(v);
      dst[i] = v;
    }
  }
  if (bad_flag && __any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(bad_flag, 1ull);
}

/* Up to kMaxSegments device-to-device copies in one launch (the retry
 * snapshot of a step and its restore): blockIdx.y picks the segment; every
 * segment starts on an allocation base (8-byte aligned), so whole 8-byte
 * words are copied and the last bytes singly. */
constexpr int kMaxSegments = 12;
struct Segments {
  const void* src[kMaxSegments];
  void* dst[kMaxSegments];
  unsigned long long bytes[kMaxSegments];
};

__global__ void k_copy_segments(Segments s) {
  const int k = blockIdx.y;
  const unsigned long long nb = s.bytes[k], nw = nb >> 3;
  const uint64_t* __restrict__ sw = static_cast<const uint64_t*>(s.src[k]);
  uint64_t* __restrict__ dw = static_cast<uint64_t*>(s.dst[k]);
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  for (unsigned long long i = t; i < nw; i += stride) dw[i] = sw[i];
  if (t < (nb & 7ull)) {
    const unsigned long long b = (nw << 3) + t;
    static_cast<uint8_t*>(s.dst[k])[b] = static_cast<const uint8_t*>(s.src[k])[b];
  }
}

/* Contacts in the caller's layout (keys i, j, fa, fb, flip and values nx, ny,
 * px, py, depth, five each), written to device memory or to mapped pinned
 * host memory.  The key fields follow pack_key. */
__global__ void k_export_contacts(const uint64_t* key, const uint8_t* flip, const double* val, int n,
                                  int32_t* keys5, double* vals5) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const uint64_t k = key[c];
    int32_t* ko = keys5 + 5 * (size_t)c;
    ko[0] = (int32_t)(k >> 44);
    ko[1] = (int32_t)((k >> 24) & 0xfffff);
    ko[2] = (int32_t)((k >> 12) & 0xfff);
    ko[3] = (int32_t)(k & 0xfff);
    ko[4] = flip[c];
    const double* vi = val + 5 * (size_t)c;
    double* vo = vals5 + 5 * (size_t)c;
#pragma unroll
    for (int q = 0; q < 5; ++q) vo[q] = vi[q];
  }
}

/* Staged body state -> live arrays, one thread per body; changed[g] = 1 when
 * a field the pose depends on (position, rotation, inverse masses, which set
 * the static flag) differs bit for bit from the live value. */
__global__ void k_commit_bodies(Ptr10 p, int n, uint8_t* changed, const unsigned long long* bad = nullptr) {
  const bool skip = bad && *bad != 0; /* refused input: the live state stays */
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < n; g += gridDim.x * blockDim.x) {
    if (skip) {
      changed[g] = 0;
      continue;
    }
    bool c = false;
#pragma unroll
    for (int k = 0; k < 10; ++k) {
      const double v = p.src[k][g];
      if (k >= 3 && k <= 7) c |= __double_as_longlong(v) != __double_as_longlong(p.dst[k][g]);
      p.dst[k][g] = v;
    }
    changed[g] = c ? 1 : 0;
  }
}

/* ------------------------------------------------------------------------ */
/* helpers                                                                    */
/* ------------------------------------------------------------------------ */

__device__ __forceinline__ bool is_nan(double d) { return d != d; }



__device__ __forceinline__ uint64_t pack_key(int i, int j, int fa, int fb) {
  return ((uint64_t)i << 44) | ((uint64_t)j << 24) | ((uint64_t)fa << 12) | (uint64_t)fb;
}

/* ------------------------------------------------------------------------ */
/* A2 pose + A11 integrate                                                    */
/* ------------------------------------------------------------------------ */

/* listToHull extents (ConvexHull.hs:151-167): for each local edge, the first
 * strict min / max vertex along its local unit normal (extentAlong',
 * ConvexHull.hs:81-92).  One thread per edge. */
__global__ void k_init_extents(Dev d) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < d.n_verts; v += gridDim.x * blockDim.x) {
    /* find the owning body by binary search over vert_off */
    int lo = 0, hi = d.n_bodies - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (d.vert_off[mid] <= v) lo = mid; else hi = mid - 1;
    }
    const int b0 = d.vert_off[lo], nv = d.vert_off[lo + 1] - b0, e = v - b0;
    if (nv < 3) { /* a circle: no edges */
      d.emin[v] = 0;
      d.emax[v] = 0;
      continue;
    }
    const int n1 = e < nv - 1 ? e + 1 : 0;
    const double ddx = d.lx[b0 + n1] - d.lx[b0 + e], ddy = d.ly[b0 + n1] - d.ly[b0 + e];
    const double ex = ddy, ey = -ddx;
    const double len = sqrt(ex * ex + ey * ey);
    const double nx = ex / len, ny = ey / len;
    double lo_d = d.lx[b0] * nx + d.ly[b0] * ny, hi_d = lo_d;
    int imin = 0, imax = 0;
    for (int k = 1; k < nv; ++k) {
      const double t = d.lx[b0 + k] * nx + d.ly[b0 + k] * ny;
      if (t < lo_d) { lo_d = t; imin = k; }
      if (t > hi_d) { hi_d = t; imax = k; }
    }
    d.emin[v] = imin;
    d.emax[v] = imax;
  }
}

/* advanceObj (Constraint.hs:225-229) when `advance`, then moveShape
 * (World.hs:132-133): rotation matrix from shapes_sincos, the 3x3 product of
 * toTransform (Transform.hs:34-38, 73-77; MatrixTemplate.hs:47-67), afmul
 * (Linear.hs:217-220) per vertex, unitEdgeNormal (ConvexHull.hs:218-226) per
 * edge, then hullToAabb (Aabb.hs:81-84, 106-110) and its ordered keys.
 * One thread per body, bodies taken in pose_order: the FP64 pipe charges a
 * warp instruction in full whatever its active lanes, so a warp whose hulls
 * have 3..8 vertices would run 8 iterations for all of them; grouped by vertex
 * count, its loops have one length.  Each body still writes only its own
 * outputs, so the order changes no result. */
__global__ void k_integrate_pose(Dev d, double dt, int advance, const uint8_t* only = nullptr) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < d.n_bodies; t += gridDim.x * blockDim.x) {
    const int g = d.pose_order ? d.pose_order[t] : t;
    if (only && !only[g]) continue; /* re-pose: this body's pose inputs did not change */
    if (d.active && !d.active[g]) { /* empty slot: left as it was, out of the broadphase */
      d.flags[g] = kFlagInactive;
      continue;
    }
    double px = d.px[g], py = d.py[g], th = d.th[g];
    if (advance) {
      const double vx = d.vx[g], vy = d.vy[g], w = d.w[g];
      px = (vx * dt) + px;
      py = (vy * dt) + py;
      th = (dt * w) + th;
      d.px[g] = px;
      d.py[g] = py;
      d.th[g] = th;
    }
    double s, c;
    shapes_sincos(th, &s, &c);
    const double ms = -s;
    /* rows of translate(px,py) times columns of rotate(c,s), summed in the
     * reference's order (joinTransforms, Transform.hs:73-77) */
    double m00, m01, m02, m10, m11, m12;
    if (finite_bits(c) && finite_bits(s) && finite_bits(px) && finite_bits(py)) {
      /* every product by 1.0 or 0.0 is exact, so the sums reduce to
       * signed-zero rules on the integer pipe */
      const double zc = signed_zero(c), zs = signed_zero(s), zms = signed_zero(ms);
      const double zpx = signed_zero(px), zpy = signed_zero(py);
      m00 = add_zero(add_zero(c, zs), zpx);
      m01 = add_zero(add_zero(ms, zc), zpx);
      m02 = plus_zero(px);
      m10 = add_zero(add_zero(s, zc), zpy);
      m11 = add_zero(add_zero(c, zms), zpy);
      m12 = plus_zero(py);
    } else {
      m00 = (1.0 * c + 0.0 * s) + px * 0.0;
      m01 = (1.0 * ms + 0.0 * c) + px * 0.0;
      m02 = (1.0 * 0.0 + 0.0 * 0.0) + px * 1.0;
      m10 = (0.0 * c + 1.0 * s) + py * 0.0;
      m11 = (0.0 * ms + 1.0 * c) + py * 0.0;
      m12 = (0.0 * 0.0 + 1.0 * 0.0) + py * 1.0;
    }
    /* m02 * 1.0 == m02 and m12 * 1.0 == m12 unless NaN (then both are NaN) */
    const bool t_nan = nan_bits(m02) || nan_bits(m12);
    const int b0 = d.vert_off[g], nv = d.vert_off[g + 1] - b0;
    const double rad = d.radius ? d.radius[g] : 0.0;
    if (rad > 0.0) {
      /* setCircleTransform (Circle.hs:60-64): the transformed local origin;
       * circleToAabb (Aabb.hs:86-89): centre -+ radius */
      const double lx = d.lx[b0], ly = d.ly[b0];
      const double x = t_nan ? (m00 * lx + m01 * ly) + m02 * 1.0 : (mul_rn_int(m00, lx) + m01 * ly) + m02;
      const double y = t_nan ? (m10 * lx + m11 * ly) + m12 * 1.0 : (mul_rn_int(m10, lx) + m11 * ly) + m12;
      d.wx[b0] = x;
      d.wy[b0] = y;
      d.nx[b0] = 0.0;
      d.ny[b0] = 0.0;
      const double cb0 = x - rad, cb1 = x + rad, cb2 = y - rad, cb3 = y + rad;
      d.box[4 * g + 0] = cb0;
      d.box[4 * g + 1] = cb1;
      d.box[4 * g + 2] = cb2;
      d.box[4 * g + 3] = cb3;
      d.boxk[4 * g + 0] = okey(cb0);
      d.boxk[4 * g + 1] = okey(cb1);
      d.boxk[4 * g + 2] = okey(cb2);
      d.boxk[4 * g + 3] = okey(cb3);
      uint8_t f = kFlagCircle;
      if (d.iml[g] == 0.0 && d.imr[g] == 0.0) f |= kFlagStatic;
      if (nan_bits(cb0) || nan_bits(cb1) || nan_bits(cb2) || nan_bits(cb3)) f |= kFlagBoxNaN;
      d.flags[g] = f;
      continue;
    }
    double x0 = 0, y0 = 0, xp = 0, yp = 0;
    double bx0 = 0, bx1 = 0, by0 = 0, by1 = 0;
    for (int k = 0; k < nv; ++k) {
      const double lx = d.lx[b0 + k], ly = d.ly[b0 + k];
      /* one product per coordinate on the integer pipe (exact), as in SAT */
      const double x = t_nan ? (m00 * lx + m01 * ly) + m02 * 1.0 : (mul_rn_int(m00, lx) + m01 * ly) + m02;
      const double y = t_nan ? (m10 * lx + m11 * ly) + m12 * 1.0 : (mul_rn_int(m10, lx) + m11 * ly) + m12;
      d.wx[b0 + k] = x;
      d.wy[b0 + k] = y;
      if (k == 0) {
        x0 = x; y0 = y;
        bx0 = x; bx1 = x; by0 = y; by1 = y;
      } else {
        const double ddx = x - xp, ddy = y - yp;
        const double ex = ddy, ey = -ddx;
        const double len = sqrt(ex * ex + ey * ey);
        d.nx[b0 + k - 1] = ex / len;
        d.ny[b0 + k - 1] = ey / len;
        bx0 = f_lt(bx0, x) ? bx0 : x;
        bx1 = f_lt(x, bx1) ? bx1 : x;
        by0 = f_lt(by0, y) ? by0 : y;
        by1 = f_lt(y, by1) ? by1 : y;
      }
      xp = x;
      yp = y;
    }
    {
      const double ddx = x0 - xp, ddy = y0 - yp;
      const double ex = ddy, ey = -ddx;
      const double len = sqrt(ex * ex + ey * ey);
      d.nx[b0 + nv - 1] = ex / len;
      d.ny[b0 + nv - 1] = ey / len;
    }
    if (d.plo) { /* extentAlongSelf (ConvexHull.hs:107-118): the SAT's self extents, once per frame */
      for (int e = 0; e < nv; ++e) {
        const double dx = d.nx[b0 + e], dy = d.ny[b0 + e];
        const int mi = b0 + d.emin[b0 + e], ma = b0 + d.emax[b0 + e];
        d.plo[b0 + e] = d.wx[mi] * dx + d.wy[mi] * dy;
        d.phi[b0 + e] = d.wx[ma] * dx + d.wy[ma] * dy;
      }
    }
    d.box[4 * g + 0] = bx0;
    d.box[4 * g + 1] = bx1;
    d.box[4 * g + 2] = by0;
    d.box[4 * g + 3] = by1;
    d.boxk[4 * g + 0] = okey(bx0);
    d.boxk[4 * g + 1] = okey(bx1);
    d.boxk[4 * g + 2] = okey(by0);
    d.boxk[4 * g + 3] = okey(by1);
    uint8_t f = 0;
    if (d.iml[g] == 0.0 && d.imr[g] == 0.0) f |= kFlagStatic;
    if (nan_bits(bx0) || nan_bits(bx1) || nan_bits(by0) || nan_bits(by1)) f |= kFlagBoxNaN;
    d.flags[g] = f;
  }
}

/* ------------------------------------------------------------------------ */
/* A3 broadphase                                                              */
/* ------------------------------------------------------------------------ */

/* culledKeys (Aabb.hs:168-183): not both static, and boundsOverlap
 * (Aabb.hs:69-72) on x and y, i.e. not (c > b || d < a) with (a,b) = box i,
 * (c,d) = box j. */
__device__ __forceinline__ bool pair_overlaps(const Dev& d, int gi, int gj, uint8_t fi,
                                              const uint64_t ki[4]) {
  const uint8_t fj = d.flags[gj];
  if ((fi | fj) & kFlagInactive) return false;
  if ((fi & fj & kFlagStatic)) return false;
  if ((fi | fj) & kFlagBoxNaN) {
    const double* a = d.box + 4 * gi;
    const double* b = d.box + 4 * gj;
    return !(b[0] > a[1] || b[1] < a[0]) && !(b[2] > a[3] || b[3] < a[2]);
  }
  const ulonglong2 kj01 = *reinterpret_cast<const ulonglong2*>(d.boxk + 4 * gj);
  const ulonglong2 kj23 = *reinterpret_cast<const ulonglong2*>(d.boxk + 4 * gj + 2);
  return !(kj01.x > ki[1] || kj01.y < ki[0]) && !(kj23.x > ki[3] || kj23.y < ki[2]);
}

/* One warp per row i (the larger index of a pair): lanes test j = i-1, i-2, ...
 * 32 at a time, so ballot order is the reference's descending j order.
 * COUNT: writes the row's pair count at its mirrored position
 * q = off + (n_w - 1 - i), so that an exclusive scan over q lays rows out in
 * descending i within each world.  !COUNT: writes the pairs at row_off[q]. */
template <bool COUNT>
__global__ void k_broadphase(Dev d) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw_total = (gridDim.x * blockDim.x) >> 5;
  for (int g = wid; g < d.n_bodies; g += nw_total) {
    if (d.row_mode[g]) continue; /* this row comes from the grid */
    const int wld = d.body_world[g];
    const int off = d.world_body_off[wld];
    const int n = d.world_body_off[wld + 1] - off;
    const int i = g - off;
    const int q = off + (n - 1 - i);
    const uint8_t fi = d.flags[g];
    uint64_t ki[4];
    ki[0] = d.boxk[4 * g + 0];
    ki[1] = d.boxk[4 * g + 1];
    ki[2] = d.boxk[4 * g + 2];
    ki[3] = d.boxk[4 * g + 3];
    int count = 0;
    const int base_out = COUNT ? 0 : d.row_off[q];
    for (int base = 0; base < i; base += 32) {
      const int jl = i - 1 - base - lane;
      bool hit = false;
      if (jl >= 0) hit = pair_overlaps(d, g, off + jl, fi, ki);
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (!COUNT && hit) {
        const int pos = base_out + count + __popc(m & ((1u << lane) - 1u));
        if (pos < d.pair_cap) {
          d.pair_a[pos] = g;
          d.pair_b[pos] = off + jl;
        }
      }
      count += __popc(m);
    }
    if (COUNT && lane == 0) d.row_cnt[q] = count;
  }
}


/* Grid broadphase for larger worlds.  It finds exactly the pairs the
 * brute-force rows find, faster: the cell size s is twice the mean AABB extent
 * of the world; a body is "small" when its width and height are below
 * s (1 - 2^-20), its box is finite and its cell index fits 30 bits.  A small
 * body is binned by the cell of its box's min corner, floor(x0 / s) and
 * floor(y0 / s) (computed as x0 * (1/s): monotone in x0).  Two small bodies
 * whose closed boxes overlap have |x0_i - x0_j| < s (1 - 2^-20) and likewise in
 * y, so their cells differ by at most one in each axis: every such pair is
 * found by scanning the 3x3 cells around a body.  Cells are hashed into a
 * table of 2^k >= 2n buckets by their Morton code; a bucket may hold other
 * cells, so candidates are kept only when their exact cell matches.  Bodies
 * that are not small are listed per world and checked against everything:
 * their own rows take the brute-force path, and every grid row also checks
 * them.  Grid rows are written unordered and then sorted (descending j), so
 * the final list is the reference's descending (i, j) order. */

__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x &= 0xffffu;
  x = (x | (x << 8)) & 0x00ff00ffu;
  x = (x | (x << 4)) & 0x0f0f0f0fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

__device__ __forceinline__ uint32_t cell_bucket(int cx, int cy, int T) {
  return (spread16((uint32_t)cx) | (spread16((uint32_t)cy) << 1)) & (uint32_t)(T - 1);
}

/* One CTA per world: mean of max(width, height) over finite boxes -> 1/s. */
/* Mean box extent of each grid world, which sets its cell size (2x the mean).
 * The cell size only decides how fast the grid finds the pairs, never which
 * pairs it finds (any positive size gives the pairs of culledKeys), so the sum
 * may be split: one block per chunk of at most 4096 bodies of one world
 * (k_extent_parts), then one thread per world adds its chunks in order
 * (deterministic; a world of one chunk sums exactly as one block would).  A
 * single large world thus spreads over the GPU instead of one SM. */
__global__ void k_extent_parts(Dev d, int inc) {
  __shared__ double s_sum[32];
  __shared__ int s_cnt[32];
  const int k = blockIdx.x;
  if (k >= d.n_ext_chunks) return;
  const int b0 = d.ext_chunk[2 * k], b1 = d.ext_chunk[2 * k + 1];
  const int wld = d.body_world[b0];
  if (d.grid_T[wld] == 0 || (inc && d.inc_state[wld] != 0)) return;
  double sum = 0.0;
  int cnt = 0;
  for (int g = b0 + threadIdx.x; g < b1; g += blockDim.x) {
    const double w = d.box[4 * g + 1] - d.box[4 * g + 0];
    const double h = d.box[4 * g + 3] - d.box[4 * g + 2];
    const double e = w > h ? w : h;
    if (small_mag(e)) {
      sum += e;
      ++cnt;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_sum[threadIdx.x >> 5] = sum;
    s_cnt[threadIdx.x >> 5] = cnt;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    int c = 0;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      t += s_sum[q];
      c += s_cnt[q];
    }
    d.ext_part_sum[k] = t;
    d.ext_part_cnt[k] = c;
  }
}

/* Twice the mean extent over a world's chunks, added in chunk order. */
__device__ __forceinline__ double world_cell_size(const Dev& d, int wld) {
  double t = 0.0;
  int c = 0;
  for (int k = d.ext_chunk_off[wld]; k < d.ext_chunk_off[wld + 1]; ++k) {
    t += d.ext_part_sum[k];
    c += d.ext_part_cnt[k];
  }
  return c > 0 ? 2.0 * t / c : 0.0;
}

/* One thread per world: cell size, its reciprocal and the size limit of a
 * grid body. */
__global__ void k_grid_stats(Dev d) {
  const int wld = blockIdx.x * blockDim.x + threadIdx.x;
  if (wld >= d.n_worlds || d.grid_T[wld] == 0) return;
  const double s = world_cell_size(d, wld);
  const double inv = (s > 0.0 && small_mag(s) && small_mag(1.0 / s)) ? 1.0 / s : 0.0;
  d.grid_inv_s[wld] = inv;
  d.grid_lim[wld] = inv > 0.0 ? (1.0 - 0x1p-20) / inv : 0.0;
  d.large_cnt[wld] = 0;
  if (d.world_sap && d.world_sap[wld]) { /* the small bodies' range of lower x, gathered by k_grid_bin */
    d.sap_range[2 * wld] = ~0ull;
    d.sap_range[2 * wld + 1] = 0ull;
  }
}

/* One thread per body: grid bodies get a cell and a bucket count, the rest go
 * on their world's list of large bodies. */
__global__ void k_grid_bin(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    const int T = d.grid_T[wld];
    uint8_t mode = 0;
    if (T > 0) {
      const double inv_s = d.grid_inv_s[wld];
      bool small = false;
      int cx = 0, cy = 0;
      if (inv_s > 0.0 && !(d.flags[g] & kFlagBoxNaN)) {
        const double x0 = d.box[4 * g + 0], x1 = d.box[4 * g + 1];
        const double y0 = d.box[4 * g + 2], y1 = d.box[4 * g + 3];
        const double lim = d.grid_lim[wld];
        const double qx = x0 * inv_s, qy = y0 * inv_s;
        if (small_mag(x0) && small_mag(x1) && small_mag(y0) && small_mag(y1) && (x1 - x0) < lim &&
            (y1 - y0) < lim && fabs(qx) < 0x1p30 && fabs(qy) < 0x1p30) {
          small = true;
          cx = (int)floor(qx);
          cy = (int)floor(qy);
        }
      }
      if (small) {
        mode = 1;
        d.cell_x[g] = cx;
        d.cell_y[g] = cy;
        if (d.world_sap && d.world_sap[wld]) {
          const uint64_t k = okey(d.box[4 * g + 0]);
          atomicMin(reinterpret_cast<unsigned long long*>(&d.sap_range[2 * wld]), (unsigned long long)k);
          atomicMax(reinterpret_cast<unsigned long long*>(&d.sap_range[2 * wld + 1]), (unsigned long long)k);
        } else {
          atomicAdd(&d.bucket_cnt[d.grid_base[wld] + cell_bucket(cx, cy, T)], 1);
        }
      } else {
        const int k = atomicAdd(&d.large_cnt[wld], 1);
        d.large_ids[d.world_body_off[wld] + k] = g;
      }
    }
    d.row_mode[g] = mode;
  }
}

/* Places grid bodies into their buckets (bucket_off turns from starts into ends). */
__global__ void k_grid_scatter(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    if (!d.row_mode[g]) continue;
    const int wld = d.body_world[g];
    if (d.world_sap && d.world_sap[wld]) continue; /* swept, not binned */
    const int b = d.grid_base[wld] + cell_bucket(d.cell_x[g], d.cell_y[g], d.grid_T[wld]);
    const int pos = atomicAdd(&d.bucket_off[b], 1);
    d.grid_ids[pos] = g;
  }
}

/* One thread per grid row i: pairs (i, j), j < i, with the 3x3 cells' bodies
 * and with the world's large bodies.  COUNT writes the row count; otherwise
 * the row is written unordered at its offset.  Buckets are read between the
 * starts (the ends of the previous bucket) and the ends left by the scatter. */
template <bool COUNT>
__global__ void k_grid_rows(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    if (!d.row_mode[g]) continue;
    const int wld = d.body_world[g];
    const int off = d.world_body_off[wld];
    const int n = d.world_body_off[wld + 1] - off;
    const int q = off + (n - 1 - (g - off));
    const int T = d.grid_T[wld], base = d.grid_base[wld];
    const int cx = d.cell_x[g], cy = d.cell_y[g];
    const uint8_t fi = d.flags[g];
    uint64_t ki[4];
    ki[0] = d.boxk[4 * g + 0];
    ki[1] = d.boxk[4 * g + 1];
    ki[2] = d.boxk[4 * g + 2];
    ki[3] = d.boxk[4 * g + 3];
    int count = 0;
    const int out = COUNT ? 0 : d.row_off[q];
    const bool sap = d.world_sap && d.world_sap[wld]; /* the sweep adds the small-body pairs */
    for (int dy = sap ? 2 : -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        const int ncx = cx + dx, ncy = cy + dy;
        const int b = base + cell_bucket(ncx, ncy, T);
        const int k0 = b > 0 ? d.bucket_off[b - 1] : 0, k1 = d.bucket_off[b];
        for (int k = k0; k < k1; ++k) {
          const int j = d.grid_ids[k];
          if (j >= g || d.cell_x[j] != ncx || d.cell_y[j] != ncy) continue;
          if (pair_overlaps(d, g, j, fi, ki)) {
            if (!COUNT && out + count < d.pair_cap) {
              d.pair_a[out + count] = g;
              d.pair_b[out + count] = j;
            }
            ++count;
          }
        }
      }
    }
    const int nl = d.large_cnt[wld];
    for (int k = 0; k < nl; ++k) {
      const int j = d.large_ids[off + k];
      if (j < g && pair_overlaps(d, g, j, fi, ki)) {
        if (!COUNT && out + count < d.pair_cap) {
          d.pair_a[out + count] = g;
          d.pair_b[out + count] = j;
        }
        ++count;
      }
    }
    if (COUNT) {
      d.row_cnt[q] = count;
      if (sap) d.sap_cursor[q] = count; /* the sweep's pairs follow the large ones */
    }
  }
}

/* ---- sweep and prune ------------------------------------------------------
 * For large single worlds, the small bodies (the grid's classification: box
 * below the cell limit) can be paired by sweep and prune along x instead of
 * the 3x3 cell search.  The bodies are sorted by their box's lower x
 * quantised to kSapBuckets buckets over the world's range, q(x) =
 * floor((x - xmin) * (kSapBuckets - 1) / (xmax - xmin)) clamped to the last
 * bucket; q is non-decreasing in x (each operation is a monotone rounding),
 * so two small bodies whose closed boxes overlap, x0_j <= x1_i, have
 * q(x0_j) <= q(x1_i).  A counting sort (one 16-bit radix digit) orders them;
 * from each body the sweep walks forward while q(x0) <= q(x1) of the body
 * and tests every candidate with the exact test every path uses
 * (pair_overlaps).  Each overlapping pair is met once, from the body earlier
 * in the order (within a bucket the order is arbitrary: the walk from the
 * earlier one still reaches the later one).  It is added to the row of its
 * larger index with an atomic slot after that row's large-body pairs, and the
 * rows are then sorted descending like the grid's, so the pairs and their
 * order are exactly those of culledKeys. */
constexpr int kSapBuckets = 65536;

__device__ __forceinline__ double from_okey(uint64_t k) {
  const uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  return __longlong_as_double((long long)u);
}

__device__ __forceinline__ int sap_bucket(const Dev& d, int wld, double x) {
  const double lo = from_okey(d.sap_range[2 * wld]), hi = from_okey(d.sap_range[2 * wld + 1]);
  const double span = hi - lo;
  const double scale = span > 0.0 && small_mag(span) ? (double)(kSapBuckets - 1) / span : 0.0;
  const double t = (x - lo) * scale;
  if (!(t > 0.0)) return 0;
  return t >= (double)(kSapBuckets - 1) ? kSapBuckets - 1 : (int)t;
}

__global__ void k_sap_count(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    if (!d.row_mode[g]) continue;
    const int wld = d.body_world[g];
    if (!d.world_sap[wld]) continue;
    atomicAdd(&d.sap_cnt[d.sap_base[wld] + sap_bucket(d, wld, d.box[4 * g + 0])], 1);
  }
}

/* Places the swept bodies by bucket (sap_cnt turns from starts into ends);
 * records the end of each world's run. */
__global__ void k_sap_scatter(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    if (!d.row_mode[g]) continue;
    const int wld = d.body_world[g];
    if (!d.world_sap[wld]) continue;
    const int q = sap_bucket(d, wld, d.box[4 * g + 0]);
    const int pos = atomicAdd(&d.sap_off[d.sap_base[wld] + q], 1);
    d.sap_ids[pos] = g;
    d.sap_qs[pos] = q;
  }
}

__global__ void k_sap_ends(Dev d) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < d.n_worlds; w += gridDim.x * blockDim.x)
    if (d.world_sap[w]) d.sap_end[w] = d.sap_off[d.sap_base[w] + kSapBuckets - 1];
}

/* One thread per position of the sorted run: the forward sweep.  COUNT adds
 * to the rows' counts; otherwise writes the pairs at atomic slots. */
template <bool COUNT>
__global__ void k_sap_rows(Dev d) {
  const int n_swept = d.sap_off[d.n_sap_buckets - 1]; /* end of the last bucket */
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n_swept; p += gridDim.x * blockDim.x) {
    const int g = d.sap_ids[p];
    const int wld = d.body_world[g];
    const int off = d.world_body_off[wld];
    const int n = d.world_body_off[wld + 1] - off;
    const int end = d.sap_end[wld];
    const int q1 = sap_bucket(d, wld, d.box[4 * g + 1]);
    const uint8_t fi = d.flags[g];
    uint64_t ki[4];
    ki[0] = d.boxk[4 * g + 0];
    ki[1] = d.boxk[4 * g + 1];
    ki[2] = d.boxk[4 * g + 2];
    ki[3] = d.boxk[4 * g + 3];
    for (int t = p + 1; t < end && d.sap_qs[t] <= q1; ++t) {
      const int j = d.sap_ids[t];
      if (!pair_overlaps(d, g, j, fi, ki)) continue;
      const int hi = g > j ? g : j, lo = g > j ? j : g;
      const int q = off + (n - 1 - (hi - off));
      if (COUNT) {
        atomicAdd(&d.row_cnt[q], 1);
      } else {
        const int pos = d.row_off[q] + atomicAdd(&d.sap_cursor[q], 1);
        if (pos < d.pair_cap) {
          d.pair_a[pos] = hi;
          d.pair_b[pos] = lo;
        }
      }
    }
  }
}

/* Sorts each grid row's j descending (rows hold a handful of pairs). */
__global__ void k_grid_sort_rows(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    if (!d.row_mode[g]) continue;
    const int wld = d.body_world[g];
    const int off = d.world_body_off[wld];
    const int n = d.world_body_off[wld + 1] - off;
    const int q = off + (n - 1 - (g - off));
    const int r0 = d.row_off[q], r1 = min(d.row_off[q + 1], d.pair_cap);
    for (int a = r0 + 1; a < r1; ++a) {
      const int v = d.pair_b[a];
      int b = a - 1;
      while (b >= r0 && d.pair_b[b] < v) {
        d.pair_b[b + 1] = d.pair_b[b];
        --b;
      }
      d.pair_b[b + 1] = v;
    }
  }
}

/* ---- incremental grid pairs ------------------------------------------------
 * The grid rows above search the 3x3 cells of every body every frame.  Most
 * bodies move far less than a cell per frame, so the incremental variant keeps
 * for each grid body a fat box (its box grown by a margin of s/32, s the
 * world's cell size) and the list of bodies whose fat boxes overlap it (an
 * adjacency, symmetric: each overlap is listed at both bodies).  While a
 * body's box stays inside its fat box nothing about it is searched again:
 * boxes inside overlapping-or-not fat boxes overlap only if the fat boxes do,
 * so the exact pairs of a row are its adjacency entries j < i whose current
 * boxes overlap (pair_overlaps, the same test as every other path).  A body
 * whose box left its fat box (or that changed between grid and large) is
 * "moved": it is removed from its old neighbours' lists, gets a new fat box,
 * searches the 3x3 cells of the fat-box grid (binned only in worlds with
 * moved bodies) and is appended to each unmoved neighbour's list.
 * Each world picks one of three modes per frame: LIST (the above), BUILD
 * (every grid body searches and the lists are written afresh: a new world,
 * every world after a retry, and a world coming back from FULL) and FULL
 * (more than a quarter of the world moved: no lists; the rows search the
 * 3x3 cells of the fat-box grid directly, like the plain grid rows).  A FULL
 * world keeps counting the bodies that leave their fat boxes and returns
 * through BUILD once that share stays below an eighth for four frames.  Large bodies (fat box not small, or a non-finite
 * box) stay on the per-world large list as before.
 * Rows come out unordered and are sorted like grid rows, so the pair list is
 * exactly the brute-force rows' list.  A list that would exceed nbr_cap sets
 * overflow bit 4 and the host retries with a larger capacity. */

constexpr int kIncList = 0, kIncBuild = 1, kIncFull = 2; /* per-world mode of a frame */
constexpr int kIncStateNew = 0, kIncStateList = 1, kIncStateFull = 2;
constexpr uint8_t kMovedBit = 1;     /* re-inserted this frame */
constexpr uint8_t kMovedWasGrid = 2; /* was in the adjacency before this frame */
constexpr uint8_t kMovedNowGrid = 4; /* is in the adjacency after this frame */

/* Fat box of a body's current box, its cell, and whether it is small enough
 * for the grid (the same finiteness and size rules as k_grid_bin, on the fat
 * box). */
__device__ __forceinline__ bool fat_box(const Dev& d, int g, int wld, double fb[4], int* cx, int* cy) {
  const double inv_s = d.grid_inv_s[wld];
  if (!(inv_s > 0.0) || (d.flags[g] & kFlagBoxNaN)) return false;
  const double m = d.inc_margin[wld];
  fb[0] = d.box[4 * g + 0] - m;
  fb[1] = d.box[4 * g + 1] + m;
  fb[2] = d.box[4 * g + 2] - m;
  fb[3] = d.box[4 * g + 3] + m;
  const double lim = d.grid_lim[wld];
  const double qx = fb[0] * inv_s, qy = fb[2] * inv_s;
  if (!(small_mag(fb[0]) && small_mag(fb[1]) && small_mag(fb[2]) && small_mag(fb[3]) && (fb[1] - fb[0]) < lim &&
        (fb[3] - fb[2]) < lim && fabs(qx) < 0x1p30 && fabs(qy) < 0x1p30))
    return false;
  *cx = (int)floor(qx);
  *cy = (int)floor(qy);
  return true;
}

/* One CTA per grid world: in a world that rebuilds, the cell size from the
 * mean extent (as k_grid_stats) and the margin s/32; every world clears its
 * large list and moved count. */
__global__ void k_inc_stats(Dev d) {
  const int wld = blockIdx.x * blockDim.x + threadIdx.x;
  if (wld >= d.n_worlds || d.grid_T[wld] == 0) return;
  if (d.inc_state[wld] != 0) {
    d.large_cnt[wld] = 0;
    d.inc_moved[wld] = 0;
    return;
  }
  const double sz = world_cell_size(d, wld);
  const double inv = (sz > 0.0 && small_mag(sz) && small_mag(1.0 / sz)) ? 1.0 / sz : 0.0;
  d.grid_inv_s[wld] = inv;
  d.grid_lim[wld] = inv > 0.0 ? (1.0 - 0x1p-20) / inv : 0.0;
  d.inc_margin[wld] = inv > 0.0 ? 0.03125 / inv : 0.0;
  d.large_cnt[wld] = 0;
  d.inc_moved[wld] = 0;
}

/* One thread per body of a grid world: moved or not, and the large list. */
__global__ void k_inc_mark(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0) continue;
    const bool rebuild = d.inc_state[wld] == 0;
    const bool was = !rebuild && d.row_mode[g];
    bool inside = false;
    if (was) {
      const uint64_t* f = d.fatk + 4 * g;
      const ulonglong2 b01 = *reinterpret_cast<const ulonglong2*>(d.boxk + 4 * g);
      const ulonglong2 b23 = *reinterpret_cast<const ulonglong2*>(d.boxk + 4 * g + 2);
      inside = !(d.flags[g] & kFlagBoxNaN) && f[0] <= b01.x && b01.y <= f[1] && f[2] <= b23.x && b23.y <= f[3];
    }
    bool fits = false;
    if (!inside) { /* only a body that is not staying needs the fat-box verdict */
      double fb[4];
      int cx = 0, cy = 0;
      fits = fat_box(d, g, wld, fb, &cx, &cy);
      if (fits) { /* its new fat box (read by nothing before k_inc_scatter) */
        for (int k = 0; k < 4; ++k) d.fatk[4 * g + k] = okey(fb[k]);
        d.cell_x[g] = cx;
        d.cell_y[g] = cy;
      }
    }
    const bool moved = rebuild || (!inside && (was || fits));
    const bool now = inside || fits;
    d.moved[g] = (moved ? kMovedBit : 0) | (was ? kMovedWasGrid : 0) | (now ? kMovedNowGrid : 0);
    if (moved && !rebuild) atomicAdd(&d.inc_moved[wld], 1);
    if (!now) {
      const int k = atomicAdd(&d.large_cnt[wld], 1);
      d.large_ids[d.world_body_off[wld] + k] = g;
    }
  }
}

/* One thread per world: this frame's mode (inc_rebuild) and the next
 * frame's state (inc_state). */
__global__ void k_inc_decide(Dev d) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < d.n_worlds; w += gridDim.x * blockDim.x) {
    if (d.grid_T[w] == 0) continue;
    const int n = d.world_body_off[w + 1] - d.world_body_off[w];
    const int st = d.inc_state[w], moved = d.inc_moved[w];
    int mode;
    if (st == kIncStateNew) {
      mode = kIncBuild;
    } else if (st == kIncStateList) {
      mode = 4 * moved > n ? kIncFull : kIncList;
    } else { /* FULL: back through BUILD after 4 quiet-enough frames */
      const int quiet = 8 * moved < n ? d.inc_frames[w] + 1 : 0;
      d.inc_frames[w] = quiet;
      mode = quiet >= 4 ? kIncBuild : kIncFull;
    }
    if (mode == kIncFull && st != kIncStateFull) d.inc_frames[w] = 0;
    d.inc_rebuild[w] = mode;
    d.inc_state[w] = mode == kIncFull ? kIncStateFull : kIncStateList;
  }
}

/* One thread per moved body that was in the adjacency: its entry in each
 * unmoved neighbour's list becomes -1 (every entry is removed by the thread
 * of the body it names, so the stores never collide). */
__global__ void k_inc_remove(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0 || d.inc_rebuild[wld] != kIncList) continue;
    const uint8_t mg = d.moved[g];
    if (!(mg & kMovedBit) || !(mg & kMovedWasGrid)) continue;
    const int32_t* lst = d.nbr + (size_t)g * d.nbr_cap;
    const int n = min(d.nbr_cnt[g], d.nbr_cap);
    for (int k = 0; k < n; ++k) {
      const int j = lst[k];
      if (j < 0 || (d.moved[j] & kMovedBit)) continue;
      int32_t* lj = d.nbr + (size_t)j * d.nbr_cap;
      const int nj = min(d.nbr_cnt[j], d.nbr_cap);
      for (int t = 0; t < nj; ++t)
        if (lj[t] == g) {
          lj[t] = -1;
          break;
        }
    }
  }
}

/* One thread per body: a moved body's grid membership (its fat box and cell
 * were written by k_inc_mark; a staying body keeps the ones it has, which
 * still contain its box); counts grid bodies into the buckets of worlds that
 * search this frame. */
__global__ void k_inc_refat(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0) continue;
    const int mode = d.inc_rebuild[wld];
    const uint8_t mg = d.moved[g];
    const bool now = (mg & kMovedNowGrid) != 0;
    if (mg & kMovedBit) d.row_mode[g] = now ? 1 : 0;
    if (mode == kIncBuild) d.nbr_cnt[g] = 0;
    if (now && (mode != kIncList || d.inc_moved[wld] > 0))
      atomicAdd(&d.bucket_cnt[d.grid_base[wld] + cell_bucket(d.cell_x[g], d.cell_y[g], d.grid_T[wld])], 1);
  }
}

__global__ void k_inc_scatter(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0 || !d.row_mode[g] || !(d.inc_rebuild[wld] != kIncList || d.inc_moved[wld] > 0)) continue;
    const int b = d.grid_base[wld] + cell_bucket(d.cell_x[g], d.cell_y[g], d.grid_T[wld]);
    const int pos = atomicAdd(&d.bucket_off[b], 1);
    d.grid_ids[pos] = g;
  }
}

__device__ __forceinline__ bool fat_overlap(const uint64_t* a, const uint64_t* b) {
  return !(b[0] > a[1] || b[1] < a[0]) && !(b[2] > a[3] || b[3] < a[2]);
}

/* One thread per re-inserted grid body: its new list from the 3x3 cells of
 * the fat-box grid; in an incremental frame it is also appended to each
 * unmoved neighbour's list. */
__global__ void k_inc_query(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0 || !d.row_mode[g]) continue;
    const int mode = d.inc_rebuild[wld];
    const bool rebuild = mode == kIncBuild;
    if (mode == kIncFull || (!rebuild && !(d.moved[g] & kMovedBit))) continue;
    const int T = d.grid_T[wld], base = d.grid_base[wld];
    const int cx = d.cell_x[g], cy = d.cell_y[g];
    uint64_t fg[4];
    for (int k = 0; k < 4; ++k) fg[k] = d.fatk[4 * g + k];
    int32_t* lst = d.nbr + (size_t)g * d.nbr_cap;
    int cnt = 0;
    bool over = false;
    for (int dy = -1; dy <= 1; ++dy) {
      for (int dx = -1; dx <= 1; ++dx) {
        const int ncx = cx + dx, ncy = cy + dy;
        const int b = base + cell_bucket(ncx, ncy, T);
        const int k0 = b > 0 ? d.bucket_off[b - 1] : 0, k1 = d.bucket_off[b];
        for (int k = k0; k < k1; ++k) {
          const int j = d.grid_ids[k];
          if (j == g || d.cell_x[j] != ncx || d.cell_y[j] != ncy) continue;
          if (!fat_overlap(fg, d.fatk + 4 * j)) continue;
          if (cnt < d.nbr_cap) lst[cnt] = j; else over = true;
          ++cnt;
          if (!rebuild && !(d.moved[j] & kMovedBit)) {
            const int pos = atomicAdd(&d.nbr_cnt[j], 1);
            if (pos < d.nbr_cap) d.nbr[(size_t)j * d.nbr_cap + pos] = g; else over = true;
          }
        }
      }
    }
    d.nbr_cnt[g] = cnt;
    if (over) atomicOr(&d.counters[kCntOverflow], 4ull);
  }
}

/* One thread per grid row i: the entries j < i of its list whose current
 * boxes overlap, then the world's large bodies j < i.  COUNT also compacts
 * the list (drops removed entries). */
template <bool COUNT>
__global__ void k_inc_rows(Dev d) {
  for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < d.n_bodies; g += gridDim.x * blockDim.x) {
    const int wld = d.body_world[g];
    if (d.grid_T[wld] == 0 || !d.row_mode[g]) continue;
    const int off = d.world_body_off[wld];
    const int n = d.world_body_off[wld + 1] - off;
    const int q = off + (n - 1 - (g - off));
    const uint8_t fi = d.flags[g];
    uint64_t ki[4];
    ki[0] = d.boxk[4 * g + 0];
    ki[1] = d.boxk[4 * g + 1];
    ki[2] = d.boxk[4 * g + 2];
    ki[3] = d.boxk[4 * g + 3];
    int count = 0;
    const int out = COUNT ? 0 : d.row_off[q];
    if (d.inc_rebuild[wld] == kIncFull) { /* no lists: the 3x3 cells of the fat-box grid */
      const int T = d.grid_T[wld], base = d.grid_base[wld];
      const int cx = d.cell_x[g], cy = d.cell_y[g];
      for (int dy = -1; dy <= 1; ++dy) {
        for (int dx = -1; dx <= 1; ++dx) {
          const int ncx = cx + dx, ncy = cy + dy;
          const int b = base + cell_bucket(ncx, ncy, T);
          const int k0 = b > 0 ? d.bucket_off[b - 1] : 0, k1 = d.bucket_off[b];
          for (int k = k0; k < k1; ++k) {
            const int j = d.grid_ids[k];
            if (j >= g || d.cell_x[j] != ncx || d.cell_y[j] != ncy) continue;
            if (pair_overlaps(d, g, j, fi, ki)) {
              if (!COUNT && out + count < d.pair_cap) {
                d.pair_a[out + count] = g;
                d.pair_b[out + count] = j;
              }
              ++count;
            }
          }
        }
      }
    } else {
      int32_t* lst = d.nbr + (size_t)g * d.nbr_cap;
      int nl = min(d.nbr_cnt[g], d.nbr_cap);
      if (COUNT) {
        int w = 0;
        for (int k = 0; k < nl; ++k) {
          const int j = lst[k];
          if (j >= 0) lst[w++] = j;
        }
        if (d.nbr_cnt[g] <= d.nbr_cap) d.nbr_cnt[g] = w;
        nl = w;
      }
      for (int k = 0; k < nl; ++k) {
        const int j = lst[k];
        if (j >= 0 && j < g && pair_overlaps(d, g, j, fi, ki)) {
          if (!COUNT && out + count < d.pair_cap) {
            d.pair_a[out + count] = g;
            d.pair_b[out + count] = j;
          }
          ++count;
        }
      }
    }
    const int nlarge = d.large_cnt[wld];
    for (int k = 0; k < nlarge; ++k) {
      const int j = d.large_ids[off + k];
      if (j < g && pair_overlaps(d, g, j, fi, ki)) {
        if (!COUNT && out + count < d.pair_cap) {
          d.pair_a[out + count] = g;
          d.pair_b[out + count] = j;
        }
        ++count;
      }
    }
    if (COUNT) d.row_cnt[q] = count;
  }
}

/* world_pair_off[w] = row_off[world_body_off[w]] (first row of the world in
 * mirrored order); also records the pair total and overflow. */
__global__ void k_world_pair_offsets(Dev d) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w <= d.n_worlds; w += gridDim.x * blockDim.x) {
    const int p = d.row_off[d.world_body_off[w]];
    d.world_pair_off[w] = p;
    if (w == d.n_worlds) {
      d.counters[kCntPairs] = (unsigned long long)p;
      if (p > d.pair_cap) d.counters[kCntOverflow] |= 1ull;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* A5-A7 narrowphase                                                          */
/* ------------------------------------------------------------------------ */

struct HullView {
  const double* wx;
  const double* wy;
  const double* nx;
  const double* ny;
  const int32_t* emin;
  const int32_t* emax;
  const double* plo; /* null: computed per axis */
  const double* phi;
  int nv;
};

__device__ __forceinline__ HullView hull_view(const Dev& d, int g) {
  const int b0 = d.vert_off[g];
  HullView h;
  h.wx = d.wx + b0;
  h.wy = d.wy + b0;
  h.nx = d.nx + b0;
  h.ny = d.ny + b0;
  h.emin = d.emin + b0;
  h.emax = d.emax + b0;
  h.plo = d.plo ? d.plo + b0 : nullptr;
  h.phi = d.phi ? d.phi + b0 : nullptr;
  h.nv = d.vert_off[g + 1] - b0;
  return h;
}

/* overlap (SAT.hs:103-118): extentAlongSelf with the precomputed extent
 * indices (ConvexHull.hs:111-118), extentAlong over the penetrator
 * (ConvexHull.hs:81-100), overlapTest/overlapAmount (SAT.hs:74-95). */
/* The comparisons run on the integer pipe through order-preserving keys; a
 * NaN projection compares false exactly as in IEEE arithmetic (a NaN first
 * projection pins lo and hi, later NaNs never replace them). */
__device__ __forceinline__ bool sat_axis(const HullView& se, int e, const HullView& sp,
                                         double* depth, int* pen) {
  const double dx = se.nx[e], dy = se.ny[e];
  double sa, sb;
  if (se.plo) { /* the hull's extent along its own normal, computed once per frame by the pose */
    sa = se.plo[e];
    sb = se.phi[e];
  } else {
    const int mi = se.emin[e], ma = se.emax[e];
    sa = se.wx[mi] * dx + se.wy[mi] * dy;
    sb = se.wx[ma] * dx + se.wy[ma] * dy;
  }
  /* one product of each projection on the integer pipe (mul_rn_int, exact),
   * the other on the FP64 pipe: the kernel is bound by FP64 throughput at
   * high occupancy, so the two pipes share the work */
  const double t0 = mul_rn_int(sp.wx[0], dx) + sp.wy[0] * dy;
  double lo = t0, hi = t0;
  uint64_t klo = okey(t0), khi = klo;
  const bool pinned = nan_bits(t0);
  int pmin = 0;
  for (int k = 1; k < sp.nv; ++k) {
    const double t = mul_rn_int(sp.wx[k], dx) + sp.wy[k] * dy;
    if (pinned || nan_bits(t)) continue;
    const uint64_t kt = okey(t);
    if (kt < klo) { lo = t; klo = kt; pmin = k; }
    if (kt > khi) { hi = t; khi = kt; }
  }
  *pen = pmin;
  if (f_lt(sb, lo) || f_lt(hi, sa)) return false; /* Separated */
  *depth = sb - lo;
  return true;
}

/* minOverlap (SAT.hs:121-138): first Separated axis, else first strict
 * minimum depth.  Returns false when separated. */
__device__ __forceinline__ bool min_overlap(const HullView& se, const HullView& sp, int* edge,
                                            double* depth, int* pen) {
  double best = 0.0;
  int be = 0, bp = 0;
  for (int e = 0; e < se.nv; ++e) {
    double dep;
    int p;
    if (!sat_axis(se, e, sp, &dep, &p)) return false;
    if (e == 0 || f_lt(dep, best)) { best = dep; be = e; bp = p; }
  }
  *edge = be;
  *depth = best;
  *pen = bp;
  return true;
}

enum { kClipNone = 0, kClipLeft = 1, kClipRight = 2, kClipBoth = 3 };

/* clipSegment (Linear.hs:327-343), intersect2 (Linear.hs:244-251),
 * invM2x2 (Linear.hs:194-199). */
__device__ __forceinline__ int clip_segment(double bpx, double bpy, double bnx, double bny,
                                            double ipx, double ipy, double inx, double iny,
                                            double ax, double ay, double bx, double by,
                                            double* cx, double* cy) {
  const double b0 = bpx * bnx + bpy * bny;
  const double b1 = ipx * inx + ipy * iny;
  const double det = bnx * iny - bny * inx;
  const double inv = 1.0 / det;
  const double m00 = iny * inv, m01 = (-bny) * inv, m10 = (-inx) * inv, m11 = bnx * inv;
  const double x = m00 * b0 + m01 * b1;
  const double y = m10 * b0 + m11 * b1;
  *cx = x;
  *cy = y;
  const double a_ = ax * bnx + ay * bny;
  const double b_ = bx * bnx + by * bny;
  const double c_ = x * bnx + y * bny;
  if (f_lt(a_, c_)) return f_lt(b_, c_) ? kClipBoth : kClipLeft;
  if (f_lt(b_, c_)) return kClipRight;
  return kClipNone;
}

/* contact_ (SAT.hs:261-267): penetratingEdge (SAT.hs:152-166), clipEdge
 * (SAT.hs:190-218) and flattenContactPoints (SAT.hs:181-187).  Writes up to
 * two (index, x, y) points, descending index. */
__device__ __forceinline__ int manifold(const HullView& se, int e, const HullView& sp, int pen,
                                        int idx[2], double xs[2], double ys[2]) {
  const int ne = e < se.nv - 1 ? e + 1 : 0;
  const double ax = se.wx[e], ay = se.wy[e], bx = se.wx[ne], by = se.wy[ne];
  const double nx = se.nx[e], ny = se.ny[e];
  const int vb = pen, vc = pen < sp.nv - 1 ? pen + 1 : 0, va = pen > 0 ? pen - 1 : sp.nv - 1;
  const double abn = fabs((sp.wx[vb] - sp.wx[va]) * nx + (sp.wy[vb] - sp.wy[va]) * ny);
  const double bcn = fabs((sp.wx[vc] - sp.wx[vb]) * nx + (sp.wy[vc] - sp.wy[vb]) * ny);
  int ci, di;
  if (f_lt(bcn, abn)) { ci = vb; di = vc; } else { ci = va; di = vb; }
  double cx = sp.wx[ci], cy = sp.wy[ci], dx = sp.wx[di], dy = sp.wy[di];
  const double lpx = cx, lpy = cy;
  const double lnx = dy - cy, lny = -(dx - cx);
  double qx, qy;
  int k = clip_segment(ax, ay, bx - ax, by - ay, lpx, lpy, lnx, lny, cx, cy, dx, dy, &qx, &qy);
  if (k == kClipBoth) return 0;
  if (k == kClipLeft) { cx = qx; cy = qy; }
  if (k == kClipRight) { dx = qx; dy = qy; }
  k = clip_segment(bx, by, ax - bx, ay - by, lpx, lpy, lnx, lny, cx, cy, dx, dy, &qx, &qy);
  if (k == kClipBoth) return 0;
  if (k == kClipLeft) { cx = qx; cy = qy; }
  if (k == kClipRight) { dx = qx; dy = qy; }
  k = clip_segment(ax, ay, -nx, -ny, lpx, lpy, lnx, lny, cx, cy, dx, dy, &qx, &qy);
  if (k == kClipBoth) return 0;
  if (k == kClipLeft) { idx[0] = di; xs[0] = dx; ys[0] = dy; return 1; }
  if (k == kClipRight) { idx[0] = ci; xs[0] = cx; ys[0] = cy; return 1; }
  if (ci > di) {
    idx[0] = ci; xs[0] = cx; ys[0] = cy;
    idx[1] = di; xs[1] = dx; ys[1] = dy;
  } else {
    idx[0] = di; xs[0] = dx; ys[0] = dy;
    idx[1] = ci; xs[1] = cx; ys[1] = cy;
  }
  return 2;
}

/* ---- circles (Contact.hs:22-40, Contact/Circle.hs, CircleVsHull.hs, GJK.hs) */

__device__ __forceinline__ double dot2(double ax, double ay, double bx, double by) { return ax * bx + ay * by; }

/* crossV2V2 (Linear.hs:135-139): (a x b) x c. */
__device__ __forceinline__ void cross3(double ax, double ay, double bx, double by, double cx, double cy,
                                       double* x, double* y) {
  const double abz = ax * by - ay * bx;
  *x = -(abz * cy);
  *y = abz * cx;
}

/* sameDirection (GJK.hs:137-138): a . b > 0, compared on the integer pipe. */
__device__ __forceinline__ bool same_dir(double ax, double ay, double bx, double by) {
  return f_lt(0.0, dot2(ax, ay, bx, by));
}

/* support (ConvexHull.hs:124-128): the first vertex of largest projection. */
__device__ __forceinline__ int gjk_support(const HullView& h, double dx, double dy) {
  int best = 0;
  double bd = dot2(h.wx[0], h.wy[0], dx, dy);
  for (int k = 1; k < h.nv; ++k) {
    const double t = dot2(h.wx[k], h.wy[k], dx, dy);
    if (f_lt(bd, t)) { bd = t; best = k; }
  }
  return best;
}

/* GJK.closestSimplex (GJK.hs:52-135) from vertex 0 toward (ox, oy): returns
 * the simplex size (3 = encloses the point), s[0] the vertex added last.  The
 * reference loop is unbounded; this one gives up after 4 nv + 8 extensions
 * (a failed search), a bound an ordinary convex hull never reaches. */
__device__ int gjk_closest(const HullView& h, double ox, double oy, int s[3]) {
  int n = 1;
  s[0] = 0;
  double dx = ox - h.wx[0], dy = oy - h.wy[0];
  for (int it = 0; it < 4 * h.nv + 8; ++it) {
    const int a = gjk_support(h, dx, dy);
    if (n == 1) {
      if (a == s[0]) return 1;
      s[1] = s[0];
      s[0] = a;
      n = 2;
      const double abx = h.wx[s[1]] - h.wx[a], aby = h.wy[s[1]] - h.wy[a];
      const double aox = ox - h.wx[a], aoy = oy - h.wy[a];
      if (same_dir(abx, aby, aox, aoy)) {
        cross3(abx, aby, aox, aoy, abx, aby, &dx, &dy);
      } else {
        n = 1;
        dx = aox;
        dy = aoy;
      }
      continue;
    }
    if (a == s[0] || a == s[1]) return 2;
    const int b = s[0], c = s[1];
    const double ax = h.wx[a], ay = h.wy[a];
    const double abx = h.wx[b] - ax, aby = h.wy[b] - ay;
    const double acx = h.wx[c] - ax, acy = h.wy[c] - ay;
    const double aox = ox - ax, aoy = oy - ay;
    const double abc = abx * acy - aby * acx;
    const double abcacx = -(abc * acy), abcacy = abc * acx;
    const double ababcx = aby * abc, ababcy = -(abx * abc);
    int mode; /* 0 star, 1 (a, c), 2 enclosed */
    if (same_dir(abcacx, abcacy, aox, aoy)) mode = same_dir(acx, acy, aox, aoy) ? 1 : 0;
    else mode = same_dir(ababcx, ababcy, aox, aoy) ? 0 : 2;
    if (mode == 2) {
      s[0] = a; s[1] = b; s[2] = c;
      return 3;
    }
    if (mode == 1) {
      s[0] = a; s[1] = c; n = 2;
      cross3(acx, acy, aox, aoy, acx, acy, &dx, &dy);
    } else if (same_dir(abx, aby, aox, aoy)) {
      s[0] = a; s[1] = b; n = 2;
      cross3(abx, aby, aox, aoy, abx, aby, &dx, &dy);
    } else {
      s[0] = a; n = 1;
      dx = aox; dy = aoy;
    }
  }
  return n;
}

/* Circle.contact (Contact/Circle.hs:27-56): a is penetrated, b penetrates. */
__device__ bool circle_circle(double ax, double ay, double ra, double bx, double by, double rb, double* v) {
  const double abx = bx - ax, aby = by - ay;
  const double rab = ra + rb;
  const double ab_sq = abx * abx + aby * aby;
  if (!f_le(ab_sq, rab * rab)) return false;
  const double len = sqrt(ab_sq);
  const double ux = abx / len, uy = aby / len;
  const double a1x = ux * ra + ax, a1y = uy * ra + ay;
  const double b1x = ux * (-rb) + bx, b1y = uy * (-rb) + by;
  v[0] = ux;
  v[1] = uy;
  v[2] = (a1x + b1x) / 2.0;
  v[3] = (a1y + b1y) / 2.0;
  v[4] = ra + rb - len;
  return true;
}

/* CircleVsHull.generateContacts (CircleVsHull.hs:18-69): the circle
 * penetrates; one contact at the closest hull point, keyed by the vertex the
 * simplex ended on; none for a 3-point simplex. */
__device__ bool circle_hull(double ox, double oy, double r, const HullView& hull, int* feature, double* v) {
  int s[3];
  const int n = gjk_closest(hull, ox, oy, s);
  if (n == 3) return false;
  double qx, qy;
  if (n == 1) {
    qx = hull.wx[s[0]];
    qy = hull.wy[s[0]];
  } else { /* closestAlong (CircleVsHull.hs:61-69) */
    const double ax = hull.wx[s[0]], ay = hull.wy[s[0]];
    const double aox = ox - ax, aoy = oy - ay;
    const double abx = hull.wx[s[1]] - ax, aby = hull.wy[s[1]] - ay;
    const double l = sqrt(abx * abx + aby * aby);
    const double ux = abx / l, uy = aby / l;
    const double t = dot2(aox, aoy, ux, uy);
    qx = ux * t + ax;
    qy = uy * t + ay;
  }
  const double bx = ox - qx, by = oy - qy;
  const double ab_sq = bx * bx + by * by;
  if (f_lt(r * r, ab_sq)) return false; /* processSimplex_ (CircleVsHull.hs:44-59) */
  const double len = sqrt(ab_sq);
  *feature = s[0];
  v[0] = -(bx / len);
  v[1] = -(by / len);
  v[2] = qx;
  v[3] = qy;
  v[4] = r - len;
  return true;
}

/* Pairs are processed grouped by the vertex counts of their two hulls, so
 * that the lanes of a warp run SAT loops of the same trip counts (one thread
 * per pair, the warp pays for its longest loop), and pairs with a circle
 * (circle-circle, or GJK against a hull of a given vertex count) apart from
 * them, so that no warp runs both the SAT and the circle code.  The grouping
 * is a permutation of the processing order only: every pair still writes its
 * own slots, so the results do not depend on it. */
__device__ __forceinline__ int np_class(const Dev& d, int p) {
  const int ga = d.pair_a[p], gb = d.pair_b[p];
  const int na = max(3, min(d.vert_off[ga + 1] - d.vert_off[ga], 9));
  const int nb = max(3, min(d.vert_off[gb + 1] - d.vert_off[gb], 9));
  const bool ca = d.radius && d.radius[ga] > 0.0, cb = d.radius && d.radius[gb] > 0.0;
  if (ca && cb) return kNpHullClasses;
  if (ca) return kNpHullClasses + 1 + (nb - 3);
  if (cb) return kNpHullClasses + 8 + (na - 3);
  return (na - 3) * 7 + (nb - 3);
}

__global__ void k_np_count(Dev d) {
  __shared__ int32_t h[kNpClasses];
  for (int k = threadIdx.x; k < kNpClasses; k += blockDim.x) h[k] = 0;
  __syncthreads();
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x)
    atomicAdd(&h[np_class(d, p)], 1);
  __syncthreads();
  for (int k = threadIdx.x; k < kNpClasses; k += blockDim.x)
    if (h[k]) atomicAdd(&d.np_cls[k], h[k]);
}

/* counts -> offsets (np_cls[kNpClasses + k]) and cursors (np_cls[k]). */
__global__ void k_np_offsets(Dev d) {
  if (threadIdx.x == 0) {
    int run = 0;
    for (int k = 0; k < kNpClasses; ++k) {
      const int c = d.np_cls[k];
      d.np_cls[kNpClasses + k] = run;
      d.np_cls[k] = run;
      run += c;
    }
    d.np_cls[2 * kNpClasses] = run;
  }
}

__global__ void k_np_scatter(Dev d) {
  __shared__ int32_t h[kNpClasses];
  __shared__ int32_t base[kNpClasses];
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  const int stride = gridDim.x * blockDim.x;
  for (int p0 = blockIdx.x * blockDim.x; p0 < P; p0 += stride) {
    for (int k = threadIdx.x; k < kNpClasses; k += blockDim.x) h[k] = 0;
    __syncthreads();
    const int p = p0 + threadIdx.x;
    int cls = -1, rank = 0;
    if (p < P) {
      cls = np_class(d, p);
      rank = atomicAdd(&h[cls], 1);
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kNpClasses; k += blockDim.x)
      base[k] = h[k] ? atomicAdd(&d.np_cls[k], h[k]) : 0;
    __syncthreads();
    if (cls >= 0) d.np_perm[base[cls] + rank] = p;
    __syncthreads();
  }
}

/* HullVsHull.generateContacts (HullVsHull.hs:54-90) over SAT.contact
 * (SAT.hs:238-258) for every broadphase pair.  One thread per pair (taken
 * in class order); results go to two fixed slots per pair and are compacted
 * after a scan. */
__global__ void k_narrowphase(Dev d) {
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < P; i += gridDim.x * blockDim.x) {
    const int p = d.np_perm ? d.np_perm[i] : i;
    const int ga = d.pair_a[p], gb = d.pair_b[p];
    const HullView a = hull_view(d, ga), b = hull_view(d, gb);
    const double ra = d.radius ? d.radius[ga] : 0.0, rb = d.radius ? d.radius[gb] : 0.0;
    if (ra > 0.0 || rb > 0.0) { /* Contact.generateContacts (Contact.hs:22-40) */
      double v[5];
      int f = 0, fa = 0, fb = 0, flip = 0;
      bool hit;
      if (ra > 0.0 && rb > 0.0) {
        hit = circle_circle(a.wx[0], a.wy[0], ra, b.wx[0], b.wy[0], rb, v);
      } else if (ra > 0.0) {
        hit = circle_hull(a.wx[0], a.wy[0], ra, b, &f, v);
        fb = f;
      } else {
        hit = circle_hull(b.wx[0], b.wy[0], rb, a, &f, v);
        fa = f;
        flip = 1;
      }
      if (hit) {
        d.slot_feat[2 * p] = fa | (fb << 12) | (flip << 24);
        double* o = d.slot_val + 5 * (2 * (size_t)p);
        for (int k = 0; k < 5; ++k) o[k] = v[k];
      }
      d.slot_cnt[p] = hit ? 1 : 0;
      continue;
    }
    int cnt = 0;
    int e_ab, pen_ab, e_ba, pen_ba;
    double dep_ab, dep_ba;
    if (min_overlap(a, b, &e_ab, &dep_ab, &pen_ab) && min_overlap(b, a, &e_ba, &dep_ba, &pen_ba)) {
      const bool flip = !f_lt(dep_ab, dep_ba);
      const HullView& se = flip ? b : a;
      const HullView& sp = flip ? a : b;
      const int e = flip ? e_ba : e_ab;
      const int pen = flip ? pen_ba : pen_ab;
      int idx[2];
      double xs[2], ys[2];
      cnt = manifold(se, e, sp, pen, idx, xs, ys);
      const double nx = se.nx[e], ny = se.ny[e];
      const double vdot = se.wx[e] * nx + se.wy[e] * ny;
      for (int q = 0; q < cnt; ++q) {
        const int fa = flip ? idx[q] : e;
        const int fb = flip ? e : idx[q];
        d.slot_feat[2 * p + q] = fa | (fb << 12) | ((flip ? 1 : 0) << 24);
        double* v = d.slot_val + 5 * (2 * (size_t)p + q);
        v[0] = nx;
        v[1] = ny;
        v[2] = xs[q];
        v[3] = ys[q];
        v[4] = vdot - (xs[q] * nx + ys[q] * ny);
      }
    }
    d.slot_cnt[p] = cnt;
  }
}

/* ---- L lanes per pair: the axis search spread over lanes, shuffle-reduced ----
 * The same contacts as k_narrowphase, with each pair's separating-axis search
 * split over L lanes of a warp (L = 32: one warp per pair; 32 / L pairs per
 * warp).  Lane e of a pair's lanes tests axes e, e + L, ... of both hulls
 * (sat_axis, unchanged); the lanes then agree, by shuffles, on whether any
 * axis separates and on each direction's minimum, taken exactly as
 * min_overlap's fold takes it: the first axis of the least depth, except that
 * a NaN depth on axis 0 keeps axis 0 and a NaN on any other axis is never
 * chosen.  The manifold, circles and the writes run on the pair's first
 * lane.  Selected by shapes_batch_set_narrowphase_lanes. */
struct AxisBest {
  uint64_t key; /* okey of the depth; ~0 when the lane holds no eligible axis */
  int e;        /* axis (kNoAxis when none) */
  int pen;
  double dep;
};
constexpr int kNoAxis = 0x7fffffff;

__device__ __forceinline__ void axis_take(AxisBest& b, int e, double dep, int pen) {
  if (nan_bits(dep)) return; /* never the fold's choice except on axis 0 (handled apart) */
  const uint64_t k = okey(dep);
  if (k < b.key || (k == b.key && e < b.e)) {
    b.key = k;
    b.e = e;
    b.pen = pen;
    b.dep = dep;
  }
}

template <int L>
__device__ __forceinline__ void axis_reduce(AxisBest& b) {
#pragma unroll
  for (int o = L / 2; o; o >>= 1) {
    const uint64_t k = __shfl_xor_sync(0xffffffffu, b.key, o, L);
    const int e = __shfl_xor_sync(0xffffffffu, b.e, o, L);
    const int pen = __shfl_xor_sync(0xffffffffu, b.pen, o, L);
    const double dep = __shfl_xor_sync(0xffffffffu, b.dep, o, L);
    if (k < b.key || (k == b.key && e < b.e)) {
      b.key = k;
      b.e = e;
      b.pen = pen;
      b.dep = dep;
    }
  }
}

/* One direction of minOverlap over this lane's axes: sep is set when one of
 * them separates; axis 0's depth and penetrator (on lane 0 of the pair) are
 * kept in d0 and p0. */
template <int L>
__device__ __forceinline__ void axes_lane(const HullView& se, const HullView& sp, int sub, AxisBest& best, bool* sep,
                                          double* d0, int* p0) {
  for (int e = sub; e < se.nv; e += L) {
    double dep;
    int pen;
    if (!sat_axis(se, e, sp, &dep, &pen)) {
      *sep = true;
      continue;
    }
    if (e == 0) {
      *d0 = dep;
      *p0 = pen;
    }
    axis_take(best, e, dep, pen);
  }
}

template <int L>
__global__ void k_narrowphase_lanes(Dev d) {
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  constexpr int G = 32 / L; /* pairs per warp */
  const int lane = threadIdx.x & 31, sub = lane & (L - 1);
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long n_warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long base = warp * G; base < P; base += n_warps * G) { /* warp-uniform */
    const int i = (int)base + lane / L;
    const bool live = i < P;
    const int p = live ? (d.np_perm ? d.np_perm[i] : i) : 0;
    const int ga = live ? d.pair_a[p] : 0, gb = live ? d.pair_b[p] : 0;
    HullView a{}, b{};
    double ra = 0.0, rb = 0.0;
    if (live) {
      a = hull_view(d, ga);
      b = hull_view(d, gb);
      ra = d.radius ? d.radius[ga] : 0.0;
      rb = d.radius ? d.radius[gb] : 0.0;
    }
    const bool circ = ra > 0.0 || rb > 0.0;
    AxisBest ab{~0ull, kNoAxis, 0, 0.0}, ba{~0ull, kNoAxis, 0, 0.0};
    bool sep = false;
    double d0_ab = 0.0, d0_ba = 0.0;
    int p0_ab = 0, p0_ba = 0;
    if (live && !circ) {
      axes_lane<L>(a, b, sub, ab, &sep, &d0_ab, &p0_ab);
      axes_lane<L>(b, a, sub, ba, &sep, &d0_ba, &p0_ba);
    }
    axis_reduce<L>(ab);
    axis_reduce<L>(ba);
    const unsigned group_mask = (L == 32 ? 0xffffffffu : ((1u << L) - 1u)) << (lane & ~(L - 1));
    sep = (__ballot_sync(0xffffffffu, sep) & group_mask) != 0;
    if (!live || sub != 0) continue;
    if (circ) { /* Contact.generateContacts (Contact.hs:22-40), as k_narrowphase */
      double v[5];
      int f = 0, fa = 0, fb = 0, flip = 0;
      bool hit;
      if (ra > 0.0 && rb > 0.0) {
        hit = circle_circle(a.wx[0], a.wy[0], ra, b.wx[0], b.wy[0], rb, v);
      } else if (ra > 0.0) {
        hit = circle_hull(a.wx[0], a.wy[0], ra, b, &f, v);
        fb = f;
      } else {
        hit = circle_hull(b.wx[0], b.wy[0], rb, a, &f, v);
        fa = f;
        flip = 1;
      }
      if (hit) {
        d.slot_feat[2 * p] = fa | (fb << 12) | (flip << 24);
        double* o = d.slot_val + 5 * (2 * (size_t)p);
        for (int k = 0; k < 5; ++k) o[k] = v[k];
      }
      d.slot_cnt[p] = hit ? 1 : 0;
      continue;
    }
    int cnt = 0;
    if (!sep) {
      /* axis 0 with a NaN depth stays the fold's choice */
      const int e_ab = nan_bits(d0_ab) ? 0 : ab.e, pen_ab = nan_bits(d0_ab) ? p0_ab : ab.pen;
      const double dep_ab = nan_bits(d0_ab) ? d0_ab : ab.dep;
      const int e_ba = nan_bits(d0_ba) ? 0 : ba.e, pen_ba = nan_bits(d0_ba) ? p0_ba : ba.pen;
      const double dep_ba = nan_bits(d0_ba) ? d0_ba : ba.dep;
      const bool flip = !f_lt(dep_ab, dep_ba);
      const HullView& se = flip ? b : a;
      const HullView& sp = flip ? a : b;
      const int e = flip ? e_ba : e_ab;
      const int pen = flip ? pen_ba : pen_ab;
      int idx[2];
      double xs[2], ys[2];
      cnt = manifold(se, e, sp, pen, idx, xs, ys);
      const double nx = se.nx[e], ny = se.ny[e];
      const double vdot = se.wx[e] * nx + se.wy[e] * ny;
      for (int q = 0; q < cnt; ++q) {
        const int fa = flip ? idx[q] : e;
        const int fb = flip ? e : idx[q];
        d.slot_feat[2 * p + q] = fa | (fb << 12) | ((flip ? 1 : 0) << 24);
        double* v = d.slot_val + 5 * (2 * (size_t)p + q);
        v[0] = nx;
        v[1] = ny;
        v[2] = xs[q];
        v[3] = ys[q];
        v[4] = vdot - (xs[q] * nx + ys[q] * ny);
      }
    }
    d.slot_cnt[p] = cnt;
  }
}

/* ------------------------------------------------------------------------ */
/* A8-A9 constraint build + warm-start lookup                                 */
/* ------------------------------------------------------------------------ */

__device__ __forceinline__ double cross2(double ax, double ay, double bx, double by) {
  return ax * by - ay * bx;
}

/* world_contact_off[w] = slot_off[world_pair_off[w]]; totals + overflow. */
__global__ void k_world_contact_offsets(Dev d) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w <= d.n_worlds; w += gridDim.x * blockDim.x) {
    const int p = min(d.world_pair_off[w], d.pair_cap);
    const int c = d.slot_off[p];
    d.world_contact_off[w] = c;
    if (w == d.n_worlds) {
      d.counters[kCntContacts] = (unsigned long long)c;
      if (c > d.contact_cap) d.counters[kCntOverflow] |= 2ull;
    }
  }
}

/* One thread per contact slot.  Compacts the contact, builds its
 * ContactConstraint (NonPenetration.hs:16-56, Friction.hs:18-44,
 * Restitution.hs:21-31, flip handling Utils.hs:175-215 / Constraint.hs:96-98),
 * the step-invariant solver factors, and looks the key up in the previous
 * cache: descZipVector (Utils/Descending.hs:47-71) over two strictly
 * descending key lists pairs each new key with an equal old key exactly when
 * one exists, which a binary search over the world's old entries finds.
 * `build_solver` = 0 compacts contacts only (collide). */
/* The slot of every contact, so that k_build's threads take contacts rather
 * than slots: about half the slots of a settled pile are empty (separated
 * pairs, pairs with one contact), and an idle lane still costs its warp's FP64
 * instructions. */
__global__ void k_contact_slots(Dev d) {
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  const int C = (int)d.counters[kCntContacts];
  if (C > d.contact_cap) return;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < 2 * P; t += gridDim.x * blockDim.x) {
    const int p = t >> 1, s = t & 1;
    if (s < d.slot_cnt[p]) d.c_slot[d.slot_off[p] + s] = t;
  }
}

__global__ void k_build(Dev d, double dt, double beta, double slop, int warm_start, int build_solver) {
  const int P = min((int)d.counters[kCntPairs], d.pair_cap);
  const int C = (int)d.counters[kCntContacts];
  if (C > d.contact_cap) return;
  const int n = d.c_slot ? C : 2 * P; /* contacts (k_contact_slots ran), else slots */
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int t = i, c = i;
    if (d.c_slot) {
      t = d.c_slot[i];
    } else {
      if ((t & 1) >= d.slot_cnt[t >> 1]) continue;
      c = d.slot_off[t >> 1] + (t & 1);
    }
    const int p = t >> 1;
    const int ga = d.pair_a[p], gb = d.pair_b[p];
    const int wld = d.body_world[ga];
    const int off = d.world_body_off[wld];
    const int feat = d.slot_feat[t];
    const int fa = feat & 0xfff, fb = (feat >> 12) & 0xfff, flip = (feat >> 24) & 1;
    const double* v = d.slot_val + 5 * (size_t)t;
    const double nx = v[0], ny = v[1], px = v[2], py = v[3], depth = v[4];
    const uint64_t key = pack_key(ga - off, gb - off, fa, fb);
    d.c_key[c] = key;
    d.c_ga[c] = ga;
    d.c_gb[c] = gb;
    d.c_flip[c] = (uint8_t)flip;
    double* cv = d.c_val + 5 * (size_t)c;
    cv[0] = nx;
    cv[1] = ny;
    cv[2] = px;
    cv[3] = py;
    cv[4] = depth;
    if (!build_solver) continue;
    /* constraintGen: positions of (a, b) = (i, j); a Flip contact is built
     * with the bodies swapped, then its Jacobian halves are swapped back. */
    const double xi = d.px[ga], yi = d.py[ga], xj = d.px[gb], yj = d.py[gb];
    const double xa = flip ? xj : xi, ya = flip ? yj : yi;
    const double xb = flip ? xi : xj, yb = flip ? yi : yj;
    double jn[6], jf[6];
    jn[0] = -nx;
    jn[1] = -ny;
    jn[2] = cross2(xa - px, ya - py, nx, ny);
    jn[3] = nx;
    jn[4] = ny;
    jn[5] = cross2(px - xb, py - yb, nx, ny);
    const double tbx = ny, tby = -nx;
    const double tax = -tbx, tay = -tby;
    jf[0] = tax;
    jf[1] = tay;
    jf[2] = cross2(px - xa, py - ya, tax, tay);
    jf[3] = tbx;
    jf[4] = tby;
    jf[5] = cross2(px - xb, py - yb, tbx, tby);
    Con cc;
    for (int k = 0; k < 3; ++k) {
      cc.jn[k] = flip ? jn[k + 3] : jn[k];
      cc.jn[k + 3] = flip ? jn[k] : jn[k + 3];
      cc.jf[k] = flip ? jf[k + 3] : jf[k];
      cc.jf[k + 3] = flip ? jf[k] : jf[k + 3];
    }
    cc.bn = depth > slop ? (beta / dt) * (slop - depth) : 0.0;
    cc.bn0 = cc.bn + 0.0;
    cc.rax = px - xi;
    cc.ray = py - yi;
    cc.rbx = px - xj;
    cc.rby = py - yj;
    cc.rnx = flip ? -nx : nx;
    cc.rny = flip ? -ny : ny;
    const double ima = d.iml[ga], ira = d.imr[ga], imb = d.iml[gb], irb = d.imr[gb];
    const double m[6] = {ima, ima, ira, imb, imb, irb};
    double mcn = (cc.jn[0] * m[0]) * cc.jn[0];
    double mcf = (cc.jf[0] * m[0]) * cc.jf[0];
    for (int k = 1; k < 6; ++k) {
      mcn = mcn + (cc.jn[k] * m[k]) * cc.jn[k];
      mcf = mcf + (cc.jf[k] * m[k]) * cc.jf[k];
    }
    cc.mcn = mcn;
    cc.mcf = mcf;
    cc.rcn = recip_ok(mcn) ? 1.0 / mcn : 0.0;
    cc.rcf = recip_ok(mcf) ? 1.0 / mcf : 0.0;
    cc.mu = (d.mu[ga] + d.mu[gb]) / 2.0;
    const double ea = d.bounce[ga], eb = d.bounce[gb];
    cc.e = ea <= eb ? ea : eb;
    cc.fast = (small_mag(cc.rax) && small_mag(cc.ray) && small_mag(cc.rbx) && small_mag(cc.rby) &&
               below_two(cc.rnx) && below_two(cc.rny)) ? 1.0 : 0.0;
    cc.pad = 0.0;
    d.con[c] = cc;
    /* warm-start lookup */
    double l0 = 0.0, l1 = 0.0;
    uint8_t hit = 0;
    if (warm_start) {
      int lo = d.old_cwo[wld], hi = d.old_cwo[wld + 1] - 1;
      while (lo <= hi) { /* keys strictly descending */
        const int mid = (lo + hi) >> 1;
        const uint64_t k = d.old_key[mid];
        if (k == key) {
          hit = 1;
          l0 = d.old_lam[2 * mid];
          l1 = d.old_lam[2 * mid + 1];
          break;
        }
        if (k > key) lo = mid + 1; else hi = mid - 1;
      }
    }
    if (d.miss_flag)
      d.miss_flag[c] = (warm_start && !hit && (d.collect_all || d.learned_mask[wld])) ? 1 : 0;
    uint8_t info = hit ? kInfoHit : 0;
    if (!(d.flags[ga] & kFlagStatic)) info |= kInfoDynA;
    if (!(d.flags[gb] & kFlagStatic)) info |= kInfoDynB;
    d.c_hit[c] = info;
    d.lam[2 * c] = l0;
    d.lam[2 * c + 1] = l1;
  }
}

/* ------------------------------------------------------------------------ */
/* A9-A10 dependency-level schedule                                           */
/* ------------------------------------------------------------------------ */

/* Block-wide exclusive scan of in-place int array a[0..n), returns total. */
__device__ int block_exclusive_scan(int32_t* a, int n, int32_t* smem /* >= 32 */) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int lane = tid & 31, wid = tid >> 5, nwarp = (nt + 31) >> 5;
  int carry = 0;
  for (int base = 0; base < n; base += nt) {
    const int idx = base + tid;
    const int x = idx < n ? a[idx] : 0;
    int incl = x;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (lane == 31) smem[wid] = incl;
    __syncthreads();
    if (wid == 0) {
      int ws = lane < nwarp ? smem[lane] : 0;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, ws, o);
        if (lane >= o) ws += y;
      }
      if (lane < nwarp) smem[lane] = ws; /* inclusive warp sums */
    }
    __syncthreads();
    const int wprefix = wid > 0 ? smem[wid - 1] : 0;
    const int chunk_total = smem[nwarp - 1];
    if (idx < n) a[idx] = carry + wprefix + incl - x;
    carry += chunk_total;
    __syncthreads();
  }
  return carry;
}

/* applyLagrangian2 (Constraint.hs:197-204): v += (J * lambda) * invMass.
 * Every contact Jacobian built by k_build has J[0] = -J[3] and J[1] = -J[4]
 * (the normal and the tangent enter the two bodies with opposite signs, and
 * a Flip only swaps the halves), and (-x) * l is exactly -(x * l) in IEEE
 * arithmetic, so those two products are computed once. */
__device__ __forceinline__ void apply_impulse(const double j[6], double l, double v[6],
                                              const double m[6]) {
  const double p3 = j[3] * l, p4 = j[4] * l;
  v[0] = v[0] + (-p3) * m[0];
  v[1] = v[1] + (-p4) * m[1];
  v[2] = v[2] + (j[2] * l) * m[2];
  v[3] = v[3] + p3 * m[3];
  v[4] = v[4] + p4 * m[4];
  v[5] = v[5] + (j[5] * l) * m[5];
}

/* J . v as a left fold (Shapes/Linear/Template.hs:108-110). */
__device__ __forceinline__ double dot6(const double j[6], const double v[6]) {
  double s = j[0] * v[0];
#pragma unroll
  for (int k = 1; k < 6; ++k) s = s + j[k] * v[k];
  return s;
}

/* Where a solver group keeps its bodies' velocities during the solve: in the
 * warp's shared-memory slice (slot = global body index + delta of its world)
 * when the group fits, else in global memory. */
struct VelStore {
  double* s;   /* shared: 3 doubles per slot */
  const Dev* d;
  __device__ __forceinline__ void load(int g, int delta, double& x, double& y, double& w) const {
    if (s) {
      const double* p = s + 3 * (g + delta);
      x = p[0]; y = p[1]; w = p[2];
    } else {
      x = d->vx[g]; y = d->vy[g]; w = d->w[g];
    }
  }
  __device__ __forceinline__ void store(int g, int delta, double x, double y, double w) const {
    if (s) {
      double* p = s + 3 * (g + delta);
      p[0] = x; p[1] = y; p[2] = w;
    } else {
      d->vx[g] = x; d->vy[g] = y; d->w[g] = w;
    }
  }
};

/* Pulls a constraint record's cache lines into L1 ahead of its level. */
__device__ __forceinline__ void prefetch_con(const Con* c) {
  const char* p = reinterpret_cast<const char*>(c);
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p + 128));
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p + sizeof(Con) - 8));
}

/* One update.  Warm: applySln of the cached Lagrangians
 * (Solvers/Contact.hs:105-113).  Otherwise improveContactSln
 * (Solvers/Contact.hs:124-143): both new Lagrangians from the same velocities
 * (contactLagrangian, Constraints/Contact.hs:86-95; bounceB,
 * Restitution.hs:34-51; lagrangian2, Constraint.hs:164-169), then positive /
 * clampAbs (SolutionProcessors.hs:33-53) and applySln (non-penetration first).
 * bounceB is min 0 (e * (v_closing . n)); when e = 0 and every velocity and
 * radius is below 2^500 the product is a signed zero and the result is +0, so
 * b + bounceB equals the precomputed b + 0.0 bit for bit. */
__device__ __forceinline__ void solve_item(const Dev& d, uint32_t item, int ga, int gb, uint8_t info,
                                           const VelStore& vs, int delta) {
  const int c = (int)(item & ~kWarmBit);
  const double2* cp = reinterpret_cast<const double2*>(d.con + c);
  double j_n[6], j_f[6];
  {
    const double2 a0 = cp[0], a1 = cp[1], a2 = cp[2], a3 = cp[3], a4 = cp[4], a5 = cp[5];
    j_n[0] = a0.x; j_n[1] = a0.y; j_n[2] = a1.x; j_n[3] = a1.y; j_n[4] = a2.x; j_n[5] = a2.y;
    j_f[0] = a3.x; j_f[1] = a3.y; j_f[2] = a4.x; j_f[3] = a4.y; j_f[4] = a5.x; j_f[5] = a5.y;
  }
  double v[6];
  vs.load(ga, delta, v[0], v[1], v[2]);
  vs.load(gb, delta, v[3], v[4], v[5]);
  const double ima = __ldg(d.iml + ga), ira = __ldg(d.imr + ga), imb = __ldg(d.iml + gb), irb = __ldg(d.imr + gb);
  const double m[6] = {ima, ima, ira, imb, imb, irb};
  double ln_apply, lf_apply;
  double2* lam2 = reinterpret_cast<double2*>(d.lam) + c;
  const double2 cached = *lam2;
  if (item & kWarmBit) {
    ln_apply = cached.x;
    lf_apply = cached.y;
  } else {
    const double2 b6 = cp[6];   /* bn, bn0 */
    const double2 b9 = cp[9];   /* rnx, rny */
    const double2 b10 = cp[10]; /* mcn, mcf */
    const double2 b11 = cp[11]; /* mu, e */
    const double2 b12 = cp[12]; /* RN(1/mcn), RN(1/mcf) */
    const double cn = cached.x, cf = cached.y;
    const uint64_t ebits = (uint64_t)__double_as_longlong(b11.y) & 0x7fffffffffffffffull;
    const bool fastflag = __double_as_longlong(cp[13].x) != 0;
    double bias;
    if (ebits == 0 && fastflag && small_mag(v[0]) && small_mag(v[1]) && small_mag(v[2]) &&
        small_mag(v[3]) && small_mag(v[4]) && small_mag(v[5])) {
      bias = b6.y;
    } else {
      const double2 b7 = cp[7]; /* rax, ray */
      const double2 b8 = cp[8]; /* rbx, rby */
      /* closing velocity ((-va + (-wa) z× ra) + vb) + wb z× rb */
      const double nwa = -v[2];
      const double cvx = ((-v[0] + (-(nwa * b7.y))) + v[3]) + (-(v[5] * b8.y));
      const double cvy = ((-v[1] + nwa * b7.x) + v[4]) + v[5] * b8.x;
      const double tb = b11.y * (cvx * b9.x + cvy * b9.y);
      const double bounce = f_le(0.0, tb) ? 0.0 : tb;
      bias = b6.x + bounce;
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
    *lam2 = make_double2(ln_cache, acc2);
  }
  apply_impulse(j_n, ln_apply, v, m);
  apply_impulse(j_f, lf_apply, v, m);
  if (info & kInfoDynA) vs.store(ga, delta, v[0], v[1], v[2]);
  if (info & kInfoDynB) vs.store(gb, delta, v[3], v[4], v[5]);
}

/* The reference applies warm starts then `iterations` sweeps strictly in
 * contact order (Solvers/Contact.hs:74-157).  Each update reads and writes only
 * its two bodies' velocities and its own Lagrangians, so running update u after
 * every earlier update that shares a non-static body with it reproduces the
 * sequential result bit for bit; static bodies are never written in the step.
 * level(u) = 1 + max(level of the last earlier update on each of its dynamic
 * bodies), and updates of one level touch disjoint bodies.  The levels pipeline
 * the sweeps: sweep s+1 starts on a body as soon as sweep s is done with it, so
 * a world offers about iterations+1 independent updates per level.
 *
 * Each warp owns one solver group: up to 32 worlds of similar size (the host
 * sorts worlds by size and packs them so that a level fills about one warp).
 * A warp never waits for another warp:
 *   1. applyExternal (World.hs:156-158, constantAccel External.hs:23-28) on the
 *      group's bodies;
 *   2. lane l scans world l's updates in sequential order, keeping each body's
 *      last level in the warp's slice of shared memory when it fits;
 *   3. the warp counting-sorts each world's updates by level in place;
 *   4. the warp runs the levels in order, lanes taking the level's updates of
 *      all its worlds, with __syncwarp between levels.
 * Steps 2-3 are latency-bound integer work that overlaps the FP64-bound step 4
 * of the other warps on the SM. */
constexpr int kMaxGroupWorlds = 32;

constexpr int kScanBlock = 8;

__global__ void k_schedule_solve(Dev d, int iterations, int warm_start, int external, double ax, double ay,
                                 double dt, int n_groups, int smem_last_per_warp) {
  extern __shared__ __align__(16) int32_t s_dyn[];
  __shared__ int32_t s_delta[8][kMaxGroupWorlds];
  if (d.counters[kCntOverflow]) return; /* buffers incomplete: the host retries */
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int grp = blockIdx.x * (blockDim.x >> 5) + wib;
  if (grp >= n_groups) return;
  const int o0 = d.group_world_off[grp], o1 = d.group_world_off[grp + 1];
  const int nw = o1 - o0;
  const int stride = iterations + 1;
  int32_t* s_last = s_dyn + wib * smem_last_per_warp;
  if (d.phase_clock && lane == 0) d.phase_clock[8 * grp + 0] = clock64();
  /* 1. gravity, 2a. reset last levels (lane-parallel over each world) */
  int group_bodies = 0;
  for (int k = 0; k < nw; ++k) {
    const int wld = d.group_worlds[o0 + k];
    group_bodies += d.world_body_off[wld + 1] - d.world_body_off[wld];
  }
  const bool smem_last = group_bodies <= smem_last_per_warp;
  {
    int base = 0;
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + lane; g < b1; g += 32) {
        if (external && !(0.0 == d.iml[g]) && !(d.flags[g] & kFlagInactive)) {
          d.vx[g] = d.vx[g] + ax * dt;
          d.vy[g] = d.vy[g] + ay * dt;
        }
        if (smem_last) s_last[base + g - b0] = 0;
        else d.last[g] = 0;
      }
      base += b1 - b0;
    }
  }
  __syncwarp();
  /* 2b. lane l scans world l */
  int my_depth = 0, my_items = 0, my_hits = 0;
  size_t my_region = 0;
  int c0 = 0, c1 = 0;
  int32_t* last = d.last;
  if (lane < nw) {
    const int wld = d.group_worlds[o0 + lane];
    int base = 0;
    for (int k = 0; k < lane; ++k) {
      const int w2 = d.group_worlds[o0 + k];
      base += d.world_body_off[w2 + 1] - d.world_body_off[w2];
    }
    const int b0 = d.world_body_off[wld];
    last = smem_last ? s_last + base - b0 : d.last;
    c0 = d.world_contact_off[wld];
    c1 = d.world_contact_off[wld + 1];
    my_region = (size_t)stride * c0;
  }
  /* Sequential scan of this lane's world, pass by pass.  The only
   * loop-carried dependency is through last[]; contacts are read in blocks of
   * kScanBlock and the next block is loaded while the current one is
   * processed, so the global-load latency hides behind kScanBlock updates of
   * shared-memory work (loads past the world's end are clamped to its last
   * contact and never used). */
  if (lane < nw && c0 < c1) {
    for (int pass = warm_start ? 0 : 1; pass <= iterations; ++pass) {
      uint8_t inf[kScanBlock];
      int ia[kScanBlock], ib[kScanBlock];
#pragma unroll
      for (int k = 0; k < kScanBlock; ++k) {
        const int cc = min(c0 + k, c1 - 1);
        inf[k] = d.c_hit[cc];
        ia[k] = d.c_ga[cc];
        ib[k] = d.c_gb[cc];
      }
      for (int cb = c0; cb < c1; cb += kScanBlock) {
        uint8_t inf2[kScanBlock];
        int ia2[kScanBlock], ib2[kScanBlock];
#pragma unroll
        for (int k = 0; k < kScanBlock; ++k) {
          const int cc = min(cb + kScanBlock + k, c1 - 1);
          inf2[k] = d.c_hit[cc];
          ia2[k] = d.c_ga[cc];
          ib2[k] = d.c_gb[cc];
        }
#pragma unroll
        for (int k = 0; k < kScanBlock; ++k) {
          const int cur_c = cb + k;
          const uint8_t info = inf[k];
          if (cur_c < c1 && !(pass == 0 && !(info & kInfoHit))) {
            const int ga = ia[k], gb = ib[k];
            const bool da = info & kInfoDynA, db = info & kInfoDynB;
            const int la = da ? last[ga] : 0, lb = db ? last[gb] : 0;
            const int lvl = (la > lb ? la : lb) + 1;
            if (da) last[ga] = lvl;
            if (db) last[gb] = lvl;
            d.idesc[my_region + my_items] =
                make_int4((int)((uint32_t)cur_c | (pass == 0 ? kWarmBit : 0u)), ga, gb, (int)info | (lane << 8));
            d.ilevel[my_region + my_items] = lvl;
            ++my_items;
            my_depth = lvl > my_depth ? lvl : my_depth;
            my_hits += pass == 0;
          }
          inf[k] = inf2[k];
          ia[k] = ia2[k];
          ib[k] = ib2[k];
        }
      }
    }
  }
  if (lane < nw) d.world_levels[d.group_worlds[o0 + lane]] = my_depth;
  if (d.phase_clock && lane == 0) d.phase_clock[8 * grp + 1] = clock64();
  /* 3. the group's updates counting-sorted by level into a region of gdesc /
   *    ghist taken from a bump allocator, as packed descriptors, so that a
   *    level is one contiguous run */
  int max_depth = my_depth, tot_items = my_items, tot_hits = my_hits;
  for (int o = 16; o > 0; o >>= 1) {
    max_depth = max(max_depth, __shfl_xor_sync(0xffffffffu, max_depth, o));
    tot_items += __shfl_xor_sync(0xffffffffu, tot_items, o);
    tot_hits += __shfl_xor_sync(0xffffffffu, tot_hits, o);
  }
  int gbase = 0;
  if (lane == 0) {
    atomicAdd(&d.counters[kCntLevels], (unsigned long long)max_depth);
    atomicAdd(&d.counters[kCntHits], (unsigned long long)tot_hits);
    atomicAdd(&d.counters[kCntItems], (unsigned long long)tot_items);
    gbase = (int)atomicAdd(&d.counters[kCntGroupAlloc], (unsigned long long)(tot_items + 1));
  }
  gbase = __shfl_sync(0xffffffffu, gbase, 0);
  int32_t* gh = d.ghist + gbase;
  int4* gdesc = d.gdesc + gbase;
  /* the histogram lives in the warp's shared slice when the depth fits (the
   * last levels are dead by now), else in gh */
  int32_t* hist = max_depth <= smem_last_per_warp ? s_last : gh;
  for (int t = lane; t < max_depth; t += 32) hist[t] = 0;
  __syncwarp();
  for (int k = 0; k < nw; ++k) {
    const int n_items = __shfl_sync(0xffffffffu, my_items, k);
    const size_t region = (size_t)__shfl_sync(0xffffffffu, (unsigned long long)my_region, k);
#pragma unroll 8
    for (int t = lane; t < n_items; t += 32) atomicAdd(&hist[d.ilevel[region + t] - 1], 1);
  }
  __syncwarp();
  {
    int carry = 0;
    for (int t0 = 0; t0 < max_depth; t0 += 32) {
      const int t = t0 + lane;
      const int x = t < max_depth ? hist[t] : 0;
      int incl = x;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (t < max_depth) hist[t] = carry + incl - x;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncwarp();
  for (int k = 0; k < nw; ++k) {
    const int n_items = __shfl_sync(0xffffffffu, my_items, k);
    const size_t region = (size_t)__shfl_sync(0xffffffffu, (unsigned long long)my_region, k);
#pragma unroll 8
    for (int t = lane; t < n_items; t += 32) {
      const int4 u = d.idesc[region + t];
      gdesc[atomicAdd(&hist[d.ilevel[region + t] - 1], 1)] = u;
    }
  }
  __syncwarp();
  if (hist != gh)
    for (int t = lane; t < max_depth; t += 32) gh[t] = hist[t];
  __syncwarp();
  if (d.phase_clock && lane == 0) d.phase_clock[8 * grp + 2] = clock64();
  /* 4. levels.  gh[L] is now the end of level L (0-based) in gdesc.  The
   *    group's velocities move to the warp's shared slice when they fit (3
   *    doubles per body), so the only dependent access per level is a
   *    shared-memory load.  A two-deep software pipeline keeps everything else
   *    off that path: while level L runs, the descriptors of level L+1 are in
   *    registers with their constraint lines being pulled into L1, and the
   *    descriptors and end offset of level L+2 are loading. */
  const bool smem_vel = 6 * group_bodies <= smem_last_per_warp;
  int32_t* dl = s_delta[wib];
  if (lane < nw) {
    const int wld = d.group_worlds[o0 + lane];
    int base = 0;
    for (int k = 0; k < lane; ++k) {
      const int w2 = d.group_worlds[o0 + k];
      base += d.world_body_off[w2 + 1] - d.world_body_off[w2];
    }
    dl[lane] = base - d.world_body_off[wld];
  }
  __syncwarp();
  VelStore vs;
  vs.d = &d;
  vs.s = smem_vel ? reinterpret_cast<double*>(s_last) : nullptr;
  if (smem_vel) {
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + lane; g < b1; g += 32) {
        double* p = vs.s + 3 * (g + dl[k]);
        p[0] = d.vx[g];
        p[1] = d.vy[g];
        p[2] = d.w[g];
      }
    }
  }
  __syncwarp();
  const int4 none = make_int4(0, 0, 0, 0);
  /* e_prev = start of level L, e_cur = end of level L, e_next = end of L+1 */
  int e_prev = 0;
  int e_cur = max_depth > 0 ? gh[0] : 0;
  int e_next = max_depth > 1 ? gh[1] : e_cur;
  int4 cur = lane < e_cur ? gdesc[lane] : none;
  int4 nxt = e_cur + lane < e_next ? gdesc[e_cur + lane] : none;
  if (lane < e_cur) prefetch_con(d.con + (cur.x & ~kWarmBit));
  for (int L = 0; L < max_depth; ++L) {
    /* issue level L+2's loads; they are consumed one iteration later */
    const int e_next2 = L + 2 < max_depth ? gh[L + 2] : e_next;
    const int4 nxt2 = e_next + lane < tot_items ? gdesc[e_next + lane] : none;
    if (e_cur + lane < e_next) prefetch_con(d.con + (nxt.x & ~kWarmBit));
    const int count = e_cur - e_prev;
    if (lane < count)
      solve_item(d, (uint32_t)cur.x, cur.y, cur.z, (uint8_t)(cur.w & 0xff), vs, dl[cur.w >> 8]);
    for (int t = lane + 32; t < count; t += 32) { /* levels wider than a warp */
      const int4 u = gdesc[e_prev + t];
      solve_item(d, (uint32_t)u.x, u.y, u.z, (uint8_t)(u.w & 0xff), vs, dl[u.w >> 8]);
    }
    __syncwarp();
    cur = nxt;
    nxt = nxt2;
    e_prev = e_cur;
    e_cur = e_next;
    e_next = e_next2;
  }
  if (smem_vel) {
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + lane; g < b1; g += 32) {
        const double* p = vs.s + 3 * (g + dl[k]);
        d.vx[g] = p[0];
        d.vy[g] = p[1];
        d.w[g] = p[2];
      }
    }
  }
  if (d.phase_clock && lane == 0) {
    d.phase_clock[8 * grp + 3] = clock64();
    d.phase_clock[8 * grp + 4] = max_depth;
    d.phase_clock[8 * grp + 5] = tot_items;
    d.phase_clock[8 * grp + 6] = group_bodies;
    d.phase_clock[8 * grp + 7] = nw;
  }
}

/* The same schedule and solve with P warps per group (one group per CTA of
 * 32 P threads).  A group's worlds are scanned by P warps at once (world k by
 * lane k / P of warp k % P), the counting sort and the level loop use all
 * 32 P threads, and __syncthreads separates the levels.  Updates of one level
 * touch disjoint dynamic bodies, so splitting a level over more threads
 * changes nothing in the results; it lets the host pack more worlds into a
 * group (fuller FP64 instructions: one warp instruction serves 32 updates)
 * without lengthening each warp's share of a level. */
template <int P, bool PAR>
__global__ void __launch_bounds__(32 * P) k_group_solve(Dev d, int iterations, int warm_start, int external,
                                                        double ax, double ay, double dt, int n_groups,
                                                        int smem_ints, int heavy_first) {
  constexpr int NT = 32 * P;
  extern __shared__ __align__(16) int32_t s_dyn[];
  __shared__ int32_t s_delta[kMaxGroupWorlds];
  __shared__ int32_t s_coff[kMaxGroupWorlds + 1]; /* PAR: prefix of the worlds' contact counts */
  __shared__ int32_t s_c0[kMaxGroupWorlds];       /* PAR: first contact of each world */
  __shared__ int32_t s_wdepth[kMaxGroupWorlds];   /* PAR: levels of each world */
  __shared__ int32_t s_nitems[kMaxGroupWorlds];
  __shared__ unsigned long long s_region[kMaxGroupWorlds];
  __shared__ int32_t s_red[3][P];
  __shared__ int32_t s_gbase;
  if (d.counters[kCntOverflow]) return; /* buffers incomplete: the host retries */
  const int tid = threadIdx.x, lane = tid & 31, wib = tid >> 5;
  /* Groups come sorted heaviest first.  With heavy_first = h > 0 the first h
   * CTAs (one wave over the SMs) take the h heaviest groups and the rest take
   * the others lightest first, so that a heavy group starts beside light ones
   * instead of beside the next heaviest. */
  const int hf = min(heavy_first, n_groups);
  const int grp = (int)blockIdx.x < hf ? (int)blockIdx.x : n_groups - 1 - ((int)blockIdx.x - hf);
  if (grp >= n_groups) return;
  const int o0 = d.group_world_off[grp], o1 = d.group_world_off[grp + 1];
  const int nw = o1 - o0;
  const int stride = iterations + 1;
  int32_t* s_last = s_dyn;
  if (d.phase_clock && tid == 0) d.phase_clock[8 * grp + 0] = clock64();
  /* 1. gravity, 2a. reset last levels */
  int group_bodies = 0;
  for (int k = 0; k < nw; ++k) {
    const int wld = d.group_worlds[o0 + k];
    group_bodies += d.world_body_off[wld + 1] - d.world_body_off[wld];
  }
  /* PAR keeps two per-body entries (last contact, last cache-hit contact) */
  const bool smem_last = (PAR ? 2 : 1) * group_bodies <= smem_ints;
  {
    int base = 0;
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + tid; g < b1; g += NT) {
        if (external && !(0.0 == d.iml[g]) && !(d.flags[g] & kFlagInactive)) {
          d.vx[g] = d.vx[g] + ax * dt;
          d.vy[g] = d.vy[g] + ay * dt;
        }
        if (PAR) {
          if (smem_last) {
            s_last[base + g - b0] = -1;
            s_last[group_bodies + base + g - b0] = -1;
          } else {
            d.last[g] = -1;
            d.last_hit[g] = -1;
          }
        } else {
          if (smem_last) s_last[base + g - b0] = 0;
          else d.last[g] = 0;
        }
      }
      if (tid == 0) s_delta[k] = base - b0;
      base += b1 - b0;
    }
  }
  __syncthreads();
  if constexpr (PAR) {
    if (tid == 0) {
      int acc = 0;
      for (int k = 0; k < nw; ++k) {
        const int wld = d.group_worlds[o0 + k];
        s_coff[k] = acc;
        s_c0[k] = d.world_contact_off[wld];
        s_wdepth[k] = 0;
        acc += d.world_contact_off[wld + 1] - d.world_contact_off[wld];
      }
      s_coff[nw] = acc;
    }
    __syncthreads();
  }
  int my_depth = 0, my_items = 0, my_hits = 0;
  if constexpr (!PAR) {
  /* 2b. world k is scanned by lane k / P of warp k % P */
  const int my_k = lane * P + wib;
  size_t my_region = 0;
  int c0 = 0, c1 = 0;
  int32_t* last = d.last;
  if (my_k < nw) {
    const int wld = d.group_worlds[o0 + my_k];
    last = smem_last ? s_last + s_delta[my_k] : d.last;
    c0 = d.world_contact_off[wld];
    c1 = d.world_contact_off[wld + 1];
    my_region = (size_t)stride * c0;
  }
  if (my_k < nw && c0 < c1) {
    for (int pass = warm_start ? 0 : 1; pass <= iterations; ++pass) {
      uint8_t inf[kScanBlock];
      int ia[kScanBlock], ib[kScanBlock];
#pragma unroll
      for (int k = 0; k < kScanBlock; ++k) {
        const int cc = min(c0 + k, c1 - 1);
        inf[k] = d.c_hit[cc];
        ia[k] = d.c_ga[cc];
        ib[k] = d.c_gb[cc];
      }
      for (int cb = c0; cb < c1; cb += kScanBlock) {
        uint8_t inf2[kScanBlock];
        int ia2[kScanBlock], ib2[kScanBlock];
#pragma unroll
        for (int k = 0; k < kScanBlock; ++k) {
          const int cc = min(cb + kScanBlock + k, c1 - 1);
          inf2[k] = d.c_hit[cc];
          ia2[k] = d.c_ga[cc];
          ib2[k] = d.c_gb[cc];
        }
#pragma unroll
        for (int k = 0; k < kScanBlock; ++k) {
          const int cur_c = cb + k;
          const uint8_t info = inf[k];
          if (cur_c < c1 && !(pass == 0 && !(info & kInfoHit))) {
            const int ga = ia[k], gb = ib[k];
            const bool da = info & kInfoDynA, db = info & kInfoDynB;
            const int la = da ? last[ga] : 0, lb = db ? last[gb] : 0;
            const int lvl = (la > lb ? la : lb) + 1;
            if (da) last[ga] = lvl;
            if (db) last[gb] = lvl;
            d.idesc[my_region + my_items] =
                make_int4((int)((uint32_t)cur_c | (pass == 0 ? kWarmBit : 0u)), ga, gb, (int)info | (my_k << 8));
            d.ilevel[my_region + my_items] = lvl;
            ++my_items;
            my_depth = lvl > my_depth ? lvl : my_depth;
            my_hits += pass == 0;
          }
          inf[k] = inf2[k];
          ia[k] = ia2[k];
          ib[k] = ib2[k];
        }
      }
    }
  }
  if (my_k < nw) {
    s_nitems[my_k] = my_items;
    s_region[my_k] = (unsigned long long)my_region;
    d.world_levels[d.group_worlds[o0 + my_k]] = my_depth;
  }
  } else {
    /* 2b. Dependency levels without a walk over every update.  Phase A: the
     * lane of world k walks the world's contacts once and records, for each
     * dynamic side, the previous contact of the world on that body and the
     * previous cache-hit contact (c_pred); the per-body arrays end holding
     * each body's last contact and last hit contact. */
    int32_t* lastc = smem_last ? s_last : d.last;
    int32_t* lasth = smem_last ? s_last + group_bodies : d.last_hit;
    const int my_k = lane * P + wib;
    if (my_k < nw) {
      const int dl = smem_last ? s_delta[my_k] : 0;
      const int c0 = s_c0[my_k], c1 = c0 + (s_coff[my_k + 1] - s_coff[my_k]);
      if (c0 < c1) {
        uint8_t inf[kScanBlock];
        int ia[kScanBlock], ib[kScanBlock];
#pragma unroll
        for (int k = 0; k < kScanBlock; ++k) {
          const int cc = min(c0 + k, c1 - 1);
          inf[k] = d.c_hit[cc];
          ia[k] = d.c_ga[cc];
          ib[k] = d.c_gb[cc];
        }
        for (int cb = c0; cb < c1; cb += kScanBlock) {
          uint8_t inf2[kScanBlock];
          int ia2[kScanBlock], ib2[kScanBlock];
#pragma unroll
          for (int k = 0; k < kScanBlock; ++k) {
            const int cc = min(cb + kScanBlock + k, c1 - 1);
            inf2[k] = d.c_hit[cc];
            ia2[k] = d.c_ga[cc];
            ib2[k] = d.c_gb[cc];
          }
#pragma unroll
          for (int k = 0; k < kScanBlock; ++k) {
            const int c = cb + k;
            if (c < c1) {
              const uint8_t info = inf[k];
              const bool hit = info & kInfoHit;
              int4 pr = make_int4(-1, -1, -1, -1);
              if (info & kInfoDynA) {
                const int sa = ia[k] + dl;
                pr.x = lastc[sa];
                pr.z = lasth[sa];
                lastc[sa] = c;
                if (hit) lasth[sa] = c;
              }
              if (info & kInfoDynB) {
                const int sb = ib[k] + dl;
                pr.y = lastc[sb];
                pr.w = lasth[sb];
                lastc[sb] = c;
                if (hit) lasth[sb] = c;
              }
              d.c_pred[c] = pr;
            }
            inf[k] = inf2[k];
            ia[k] = ia2[k];
            ib[k] = ib2[k];
          }
        }
      }
    }
    __syncthreads();
    /* Phase B: the passes in order over the group's contacts in chunks of the
     * CTA's threads.  An update's level is one more than its predecessors'
     * on each dynamic body: the previous contact of the same pass touching
     * it, else the body's last contact of the previous pass (only cache hits
     * are updates of the warm-start pass).  Within a chunk the levels are
     * raised to a fixed point (they only grow and stay at or below the final
     * values), which gives every update the level a walk over the updates in
     * order gives it.  Update (pass p, contact c) of world k takes slot
     * (p - p0) n_k + (c - c0_k) of the world's region; a slot without an
     * update (the warm-start pass of a contact without a cache hit) keeps
     * level 0. */
    const int NC = s_coff[nw];
    const int p0 = warm_start ? 0 : 1;
    for (int p = p0; p <= iterations; ++p) {
      int32_t* Lc = d.c_lvl + (size_t)(p & 1) * d.contact_cap;
      const int32_t* Lp = d.c_lvl + (size_t)((p + 1) & 1) * d.contact_cap;
      for (int s0 = 0; s0 < NC; s0 += NT) {
        const int gc = s0 + tid;
        int k = 0, c = -1, ga = 0, gb = 0;
        uint8_t info = 0;
        int4 pr = make_int4(-1, -1, -1, -1);
        if (gc < NC) {
          while (k + 1 < nw && s_coff[k + 1] <= gc) ++k;
          c = s_c0[k] + (gc - s_coff[k]);
          info = d.c_hit[c];
          ga = d.c_ga[c];
          gb = d.c_gb[c];
          pr = d.c_pred[c];
        }
        const bool live = c >= 0 && !(p == 0 && !(info & kInfoHit));
        const int dl = smem_last ? s_delta[k] : 0;
        int a_same = -1, b_same = -1, base = 0;
        if (live && (info & kInfoDynA)) {
          a_same = p == 0 ? pr.z : pr.x;
          if (a_same < 0 && p > p0) {
            const int q = p - 1 == 0 ? lasth[ga + dl] : lastc[ga + dl];
            if (q >= 0) base = max(base, Lp[q]);
          }
        }
        if (live && (info & kInfoDynB)) {
          b_same = p == 0 ? pr.w : pr.y;
          if (b_same < 0 && p > p0) {
            const int q = p - 1 == 0 ? lasth[gb + dl] : lastc[gb + dl];
            if (q >= 0) base = max(base, Lp[q]);
          }
        }
        if (live) Lc[c] = 0;
        __syncthreads();
        int L = 0;
        for (;;) {
          int v = base;
          if (a_same >= 0) v = max(v, Lc[a_same]);
          if (b_same >= 0) v = max(v, Lc[b_same]);
          const int nl = live ? v + 1 : 0;
          const bool changed = nl != L;
          L = nl;
          __syncthreads(); /* every read of this round before any write */
          if (changed) Lc[c] = L;
          if (!__syncthreads_or(changed)) break;
        }
        if (c >= 0) {
          const size_t slot = (size_t)stride * s_c0[k] + (size_t)(p - p0) * (s_coff[k + 1] - s_coff[k]) +
                              (size_t)(gc - s_coff[k]);
          if (live) {
            d.idesc[slot] = make_int4((int)((uint32_t)c | (p == 0 ? kWarmBit : 0u)), ga, gb, (int)info | (k << 8));
            ++my_items;
            my_depth = L > my_depth ? L : my_depth;
            my_hits += p == 0;
            atomicMax(&s_wdepth[k], L);
          }
          d.ilevel[slot] = L; /* 0: no update in this slot */
        }
      }
      __syncthreads();
    }
    if (tid < nw) {
      const int n_k = s_coff[tid + 1] - s_coff[tid];
      s_nitems[tid] = (iterations + 1 - p0) * n_k;
      s_region[tid] = (unsigned long long)stride * (unsigned long long)s_c0[tid];
      d.world_levels[d.group_worlds[o0 + tid]] = s_wdepth[tid];
    }
    __syncthreads();
  }
  if (d.phase_clock && tid == 0) d.phase_clock[8 * grp + 1] = clock64();
  /* 3. counting sort by level into a region of gdesc / ghist */
  int max_depth = my_depth, tot_items = my_items, tot_hits = my_hits;
  for (int o = 16; o > 0; o >>= 1) {
    max_depth = max(max_depth, __shfl_xor_sync(0xffffffffu, max_depth, o));
    tot_items += __shfl_xor_sync(0xffffffffu, tot_items, o);
    tot_hits += __shfl_xor_sync(0xffffffffu, tot_hits, o);
  }
  if (lane == 0) {
    s_red[0][wib] = max_depth;
    s_red[1][wib] = tot_items;
    s_red[2][wib] = tot_hits;
  }
  __syncthreads();
  max_depth = 0;
  tot_items = 0;
  tot_hits = 0;
#pragma unroll
  for (int w = 0; w < P; ++w) {
    max_depth = max(max_depth, s_red[0][w]);
    tot_items += s_red[1][w];
    tot_hits += s_red[2][w];
  }
  if (tid == 0) {
    atomicAdd(&d.counters[kCntLevels], (unsigned long long)max_depth);
    atomicAdd(&d.counters[kCntHits], (unsigned long long)tot_hits);
    atomicAdd(&d.counters[kCntItems], (unsigned long long)tot_items);
    s_gbase = (int)atomicAdd(&d.counters[kCntGroupAlloc], (unsigned long long)(tot_items + 1));
  }
  __syncthreads();
  const int gbase = s_gbase;
  int32_t* gh = d.ghist + gbase;
  int4* gdesc = d.gdesc + gbase;
  int32_t* hist = max_depth <= smem_ints ? s_last : gh; /* the last levels are dead by now */
  for (int t = tid; t < max_depth; t += NT) hist[t] = 0;
  __syncthreads();
  for (int k = 0; k < nw; ++k) {
    const int n_items = s_nitems[k];
    const size_t region = (size_t)s_region[k];
#pragma unroll 4
    for (int t = tid; t < n_items; t += NT) {
      const int lvl = d.ilevel[region + t];
      if (!PAR || lvl > 0) atomicAdd(&hist[lvl - 1], 1);
    }
  }
  __syncthreads();
  if (wib == 0) { /* exclusive scan of the level counts by warp 0 */
    int carry = 0;
    for (int t0 = 0; t0 < max_depth; t0 += 32) {
      const int t = t0 + lane;
      const int x = t < max_depth ? hist[t] : 0;
      int incl = x;
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
      }
      if (t < max_depth) hist[t] = carry + incl - x;
      carry += __shfl_sync(0xffffffffu, incl, 31);
    }
  }
  __syncthreads();
  for (int k = 0; k < nw; ++k) {
    const int n_items = s_nitems[k];
    const size_t region = (size_t)s_region[k];
#pragma unroll 4
    for (int t = tid; t < n_items; t += NT) {
      const int lvl = d.ilevel[region + t];
      if (PAR && lvl <= 0) continue;
      const int4 u = d.idesc[region + t];
      gdesc[atomicAdd(&hist[lvl - 1], 1)] = u;
    }
  }
  __syncthreads();
  if (hist != gh)
    for (int t = tid; t < max_depth; t += NT) gh[t] = hist[t];
  __syncthreads();
  if (d.phase_clock && tid == 0) d.phase_clock[8 * grp + 2] = clock64();
  /* 4. levels, velocities in shared memory when they fit */
  const bool smem_vel = 6 * group_bodies <= smem_ints;
  VelStore vs;
  vs.d = &d;
  vs.s = smem_vel ? reinterpret_cast<double*>(s_last) : nullptr;
  if (smem_vel) {
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + tid; g < b1; g += NT) {
        double* p = vs.s + 3 * (g + s_delta[k]);
        p[0] = d.vx[g];
        p[1] = d.vy[g];
        p[2] = d.w[g];
      }
    }
  }
  __syncthreads();
  const int4 none = make_int4(0, 0, 0, 0);
  int e_prev = 0;
  int e_cur = max_depth > 0 ? gh[0] : 0;
  int e_next = max_depth > 1 ? gh[1] : e_cur;
  int4 cur = tid < e_cur ? gdesc[tid] : none;
  int4 nxt = e_cur + tid < e_next ? gdesc[e_cur + tid] : none;
  if (tid < e_cur) prefetch_con(d.con + (cur.x & ~kWarmBit));
  for (int L = 0; L < max_depth; ++L) {
    const int e_next2 = L + 2 < max_depth ? gh[L + 2] : e_next;
    const int4 nxt2 = e_next + tid < tot_items ? gdesc[e_next + tid] : none;
    if (e_cur + tid < e_next) prefetch_con(d.con + (nxt.x & ~kWarmBit));
    const int count = e_cur - e_prev;
    if (tid < count)
      solve_item(d, (uint32_t)cur.x, cur.y, cur.z, (uint8_t)(cur.w & 0xff), vs, s_delta[cur.w >> 8]);
    for (int t = tid + NT; t < count; t += NT) { /* levels wider than the CTA */
      const int4 u = gdesc[e_prev + t];
      solve_item(d, (uint32_t)u.x, u.y, u.z, (uint8_t)(u.w & 0xff), vs, s_delta[u.w >> 8]);
    }
    __syncthreads();
    cur = nxt;
    nxt = nxt2;
    e_prev = e_cur;
    e_cur = e_next;
    e_next = e_next2;
  }
  if (smem_vel) {
    for (int k = 0; k < nw; ++k) {
      const int wld = d.group_worlds[o0 + k];
      const int b0 = d.world_body_off[wld], b1 = d.world_body_off[wld + 1];
      for (int g = b0 + tid; g < b1; g += NT) {
        const double* p = vs.s + 3 * (g + s_delta[k]);
        d.vx[g] = p[0];
        d.vy[g] = p[1];
        d.w[g] = p[2];
      }
    }
  }
  if (d.phase_clock && tid == 0) {
    d.phase_clock[8 * grp + 3] = clock64();
    d.phase_clock[8 * grp + 4] = max_depth;
    d.phase_clock[8 * grp + 5] = tot_items;
    d.phase_clock[8 * grp + 6] = group_bodies;
    d.phase_clock[8 * grp + 7] = nw;
  }
}

/* Per-world solver residual after the last sweep: one more improveContactSln
 * pass over the world's contacts that applies nothing (every contact sees the
 * final velocities), reporting sqrt(mean over contacts of the normal and
 * friction amounts it would apply, squared).  The squared amounts of one
 * contact: */
__device__ __forceinline__ double residual_term(const Dev& d, int c) {
  const int ga = d.c_ga[c], gb = d.c_gb[c];
  const double2* cp = reinterpret_cast<const double2*>(d.con + c);
  double j_n[6], j_f[6];
  const double2 a0 = cp[0], a1 = cp[1], a2 = cp[2], a3 = cp[3], a4 = cp[4], a5 = cp[5];
  j_n[0] = a0.x; j_n[1] = a0.y; j_n[2] = a1.x; j_n[3] = a1.y; j_n[4] = a2.x; j_n[5] = a2.y;
  j_f[0] = a3.x; j_f[1] = a3.y; j_f[2] = a4.x; j_f[3] = a4.y; j_f[4] = a5.x; j_f[5] = a5.y;
  const double v[6] = {d.vx[ga], d.vy[ga], d.w[ga], d.vx[gb], d.vy[gb], d.w[gb]};
  const double2 b6 = cp[6], b7 = cp[7], b8 = cp[8], b9 = cp[9], b10 = cp[10], b11 = cp[11], b12 = cp[12];
  const double2 cached = reinterpret_cast<const double2*>(d.lam)[c];
  const double nwa = -v[2];
  const double cvx = ((-v[0] + (-(nwa * b7.y))) + v[3]) + (-(v[5] * b8.y));
  const double cvy = ((-v[1] + nwa * b7.x) + v[4]) + v[5] * b8.x;
  const double tb = b11.y * (cvx * b9.x + cvy * b9.y);
  const double bias = b6.x + (f_le(0.0, tb) ? 0.0 : tb);
  const double ln_new = div_rn(-(dot6(j_n, v) + bias), b10.x, b12.x);
  const double lf_new = div_rn(-plus_zero(dot6(j_f, v)), b10.y, b12.y);
  const double ln_apply = f_le(ln_new, -cached.x) ? -cached.x : ln_new;
  const double thr = (cached.x + ln_apply) * b11.x;
  const double acc = cached.y + lf_new;
  const double acc2 = f_lt(thr, acc) ? thr : (f_lt(acc, -thr) ? -thr : acc);
  const double lf_apply = acc2 - cached.y;
  return ln_apply * ln_apply + lf_apply * lf_apply;
}

/* One warp per world (fixed summation order); worlds of `split_from` bodies
 * or more are left to k_residual_part / k_metric_final. */
__global__ void k_residual(Dev d, int split_from) {
  const int lane = threadIdx.x & 31;
  const int wld = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wld >= d.n_worlds) return;
  if (d.world_body_off[wld + 1] - d.world_body_off[wld] >= split_from) return;
  const int c0 = d.world_contact_off[wld], c1 = d.world_contact_off[wld + 1];
  double sum = 0.0;
  for (int c = c0 + lane; c < c1; c += 32) sum += residual_term(d, c);
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if (lane == 0) d.world_residual[wld] = c1 > c0 ? sqrt(sum / (2.0 * (c1 - c0))) : 0.0;
}

/* Per-world maximum penetration depth over the contacts of the last collide.
 * One warp per world; worlds of `split_from` bodies or more are left to
 * k_depth_part / k_metric_final. */
__global__ void k_world_depth(Dev d, int split_from) {
  const int lane = threadIdx.x & 31;
  const int wld = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wld >= d.n_worlds) return;
  if (d.world_body_off[wld + 1] - d.world_body_off[wld] >= split_from) return;
  const int c0 = d.world_contact_off[wld], c1 = d.world_contact_off[wld + 1];
  double m = 0.0;
  for (int c = c0 + lane; c < c1; c += 32) m = fmax(m, d.c_val[5 * (size_t)c + 4]);
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if (lane == 0) d.world_depth[wld] = m;
}

/* The same metrics for one large world over kMetricParts warps: warp k takes
 * the k-th contiguous chunk of the world's contacts, and k_metric_final
 * combines the parts in order (a fixed summation order for the residual). */
constexpr int kMetricParts = 256;

template <bool RESIDUAL>
__global__ void k_metric_part(Dev d, int wld, double* part) {
  const int lane = threadIdx.x & 31;
  const int k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (k >= kMetricParts) return;
  const int c0 = d.world_contact_off[wld], c1 = d.world_contact_off[wld + 1];
  const int chunk = (c1 - c0 + kMetricParts - 1) / kMetricParts;
  const int a = c0 + k * chunk, b = min(c1, a + chunk);
  double acc = 0.0;
  for (int c = a + lane; c < b; c += 32) acc = RESIDUAL ? acc + residual_term(d, c) : fmax(acc, d.c_val[5 * (size_t)c + 4]);
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_xor_sync(0xffffffffu, acc, o);
    acc = RESIDUAL ? acc + t : fmax(acc, t);
  }
  if (lane == 0) part[k] = acc;
}

template <bool RESIDUAL>
__global__ void k_metric_final(Dev d, int wld, const double* part) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double acc = 0.0;
  for (int k = 0; k < kMetricParts; ++k) acc = RESIDUAL ? acc + part[k] : fmax(acc, part[k]);
  const int n = d.world_contact_off[wld + 1] - d.world_contact_off[wld];
  if (RESIDUAL)
    d.world_residual[wld] = n > 0 ? sqrt(acc / (2.0 * n)) : 0.0;
  else
    d.world_depth[wld] = acc;
}

/* ------------------------------------------------------------------------ */
/* scans                                                                      */
/* ------------------------------------------------------------------------ */

constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;

/* Tile sums of in[0..n) (n read from *n_dev when non-null, capped at n_cap). */
__global__ void k_scan_tiles(const int32_t* in, int n_cap, const unsigned long long* n_dev,
                             int32_t* tile_sums) {
  __shared__ int32_t s[32];
  const int n = n_dev ? (int)min((unsigned long long)n_cap, *n_dev) : n_cap;
  const int base = blockIdx.x * kScanTile;
  int sum = 0;
  for (int k = 0; k < kScanPerThread; ++k) {
    const int idx = base + k * kScanThreads + threadIdx.x;
    if (idx < n) sum += in[idx];
  }
  for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = sum;
  __syncthreads();
  if (threadIdx.x == 0) {
    int t = 0;
    for (int k = 0; k < kScanThreads / 32; ++k) t += s[k];
    tile_sums[blockIdx.x] = t;
  }
}

/* Exclusive scan of the tile sums (one block). */
__global__ void k_scan_tile_sums(int32_t* tile_sums, int n_tiles) {
  __shared__ int32_t s[32];
  block_exclusive_scan(tile_sums, n_tiles, s);
}

/* out[k] = exclusive prefix of in; out[n] = total. */
__global__ void k_scan_apply(const int32_t* in, int n_cap, const unsigned long long* n_dev,
                             const int32_t* tile_sums, int32_t* out) {
  __shared__ int32_t s_vals[kScanTile];
  __shared__ int32_t s_scan[32];
  const int n = n_dev ? (int)min((unsigned long long)n_cap, *n_dev) : n_cap;
  const int base = blockIdx.x * kScanTile;
  for (int k = threadIdx.x; k < kScanTile; k += kScanThreads) {
    const int idx = base + k;
    s_vals[k] = idx < n ? in[idx] : 0;
  }
  __syncthreads();
  /* per-thread serial over a contiguous run, then block scan of run totals */
  const int r0 = threadIdx.x * kScanPerThread;
  int run = 0;
  for (int k = 0; k < kScanPerThread; ++k) run += s_vals[r0 + k];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int incl = run;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) s_scan[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int ws = lane < kScanThreads / 32 ? s_scan[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, ws, o);
      if (lane >= o) ws += y;
    }
    if (lane < kScanThreads / 32) s_scan[lane] = ws;
  }
  __syncthreads();
  int prefix = tile_sums[blockIdx.x] + (wid > 0 ? s_scan[wid - 1] : 0) + incl - run;
  for (int k = 0; k < kScanPerThread; ++k) {
    const int idx = base + r0 + k;
    if (idx <= n) out[idx] = prefix;
    prefix += s_vals[r0 + k];
  }
}

}  // namespace shapes
