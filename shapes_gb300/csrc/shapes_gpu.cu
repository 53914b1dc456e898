/*
 * Host runtime behind include/shapes_gpu.h: one handle = a batch of
 * independent worlds resident on the device as structure-of-arrays, stepped by
 * the kernels of step_kernels.cuh on the handle's own CUDA stream.
 *
 * Buffers whose size depends on the step (pairs, contacts, solver updates) are
 * sized generously up front.  Kernels never write past a capacity: they raise a
 * sticky overflow flag instead, and the host then restores the state saved at
 * the start of the call, doubles the capacities and runs the call again, so a
 * call either completes exactly or returns an error with the state untouched.
 */
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <vector>

#include "../../include/shapes_gpu.h"
#include "step_kernels.cuh"
#include "large_world.cuh"
#include "learned.cuh"
#include "mlp.h"

using shapes::Con;
using shapes::Dev;

/* Text of the last CUDA error on this thread (shared with the MLP unit). */
thread_local std::string g_last_error;

namespace {

struct CudaError {
  cudaError_t err;
};

inline void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    throw CudaError{e};
  }
}

constexpr int kSMs = 152;

template <typename T>
T* dalloc(size_t n, const char* what) {
  void* p = nullptr;
  ck(cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)), what);
  return static_cast<T*>(p);
}

inline void dfree(void* p) {
  if (p) cudaFree(p);
}

inline int grid_for(long long n, int threads) {
  long long blocks = (n + threads - 1) / threads;
  long long cap = (long long)kSMs * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  return (int)blocks;
}

}  // namespace

struct shapes_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  int32_t W = 0, N = 0, V = 0;
  std::vector<int32_t> h_world_body_off;
  std::vector<int32_t> h_body_world;

  /* topology */
  int32_t* world_body_off = nullptr;
  int32_t* body_world = nullptr;
  int32_t* vert_off = nullptr;
  double* lx = nullptr;
  double* ly = nullptr;
  double* radius = nullptr; /* [N] circle radii (0 for hulls); null when there is no circle */
  int32_t* emin = nullptr;
  int32_t* emax = nullptr;
  /* state */
  double* body[10] = {nullptr};
  double* body_stage[10] = {nullptr}; /* set_bodies uploads here, validated, then swapped in */
  double* wx = nullptr;
  double* wy = nullptr;
  double* nx = nullptr;
  double* ny = nullptr;
  double* plo = nullptr; /* [V] self extents of each edge (SAT) */
  double* phi = nullptr;
  double* box = nullptr;
  uint64_t* boxk = nullptr;
  uint8_t* flags = nullptr;
  uint8_t* body_changed = nullptr; /* [N] scratch of set_bodies: pose inputs changed */
  int32_t* export_keys = nullptr;  /* staging of get_contacts for pageable caller arrays */
  double* export_vals = nullptr;
  int64_t export_cap = 0;
  /* broadphase / narrowphase */
  int32_t pair_cap = 0, contact_cap = 0;
  int64_t item_cap = 0;
  int32_t* row_cnt = nullptr;
  int32_t* row_off = nullptr;
  /* grid broadphase */
  int32_t grid_min_bodies = 64;
  bool any_grid = false;
  int32_t n_buckets = 0;
  int32_t* grid_T = nullptr;
  int32_t* grid_base = nullptr;
  double* grid_inv_s = nullptr;
  double* grid_lim = nullptr;
  int32_t* bucket_cnt = nullptr;
  int32_t* bucket_off = nullptr;
  int32_t* grid_ids = nullptr;
  int32_t* cell_x = nullptr;
  int32_t* cell_y = nullptr;
  uint8_t* row_mode = nullptr;
  int32_t* large_cnt = nullptr;
  int32_t* large_ids = nullptr;
  double* metric_part = nullptr; /* [kMetricParts] partial metrics of one large world */
  /* incremental grid pairs (fat boxes and adjacency lists) */
  bool incremental = true;
  int32_t nbr_cap = 24;
  uint64_t* fatk = nullptr;
  int32_t* nbr = nullptr;
  int32_t* nbr_cnt = nullptr;
  uint8_t* moved = nullptr;
  int32_t* inc_state = nullptr;
  int32_t* inc_rebuild = nullptr;
  int32_t* inc_moved = nullptr;
  int32_t* inc_frames = nullptr;
  double* inc_margin = nullptr;
  int32_t* pair_a = nullptr;
  int32_t* pair_b = nullptr;
  int32_t* slot_cnt = nullptr;
  int32_t* slot_off = nullptr;
  int32_t* slot_feat = nullptr;
  double* slot_val = nullptr;
  int32_t* np_perm = nullptr;
  int32_t* pose_order = nullptr; /* [N] bodies grouped by vertex count within chunks of 1024 */
  int32_t* ext_chunk = nullptr;      /* extent reduction: chunk body ranges, per-world chunk offsets, partials */
  int32_t* ext_chunk_off = nullptr;
  double* ext_part_sum = nullptr;
  int32_t* ext_part_cnt = nullptr;
  int32_t n_ext_chunks = 0;
  /* sweep and prune for the small bodies of large grid worlds (incremental pairs off) */
  int32_t sap_min_bodies = 0; /* 0: off */
  int32_t np_lanes = 1;       /* lanes per pair in the narrowphase (1: k_narrowphase) */
  long long lw_poll_limit = shapes::kPollLimit; /* ordered large-world solve: polls of one dependency */
  bool any_sap = false;
  int32_t n_sap_buckets = 0;
  uint8_t* world_sap = nullptr;
  int32_t *sap_base = nullptr, *sap_cnt = nullptr, *sap_off = nullptr, *sap_ids = nullptr, *sap_qs = nullptr;
  int32_t *sap_cursor = nullptr, *sap_end = nullptr;
  uint64_t* sap_range = nullptr;

  /* Tile sums every scan of a step needs: the longest scanned array is the
   * bodies, the contact slots, the grid buckets or the sweep buckets. */
  int32_t scan_tiles_needed() const {
    const int64_t scan_n =
        std::max<int64_t>(std::max<int64_t>(std::max<int64_t>(N, contact_cap), n_buckets), n_sap_buckets) + 1;
    return (int32_t)((scan_n + shapes::kScanTile - 1) / shapes::kScanTile) + 1;
  }

  void free_sap() {
    dfree(world_sap); dfree(sap_base); dfree(sap_cnt); dfree(sap_off); dfree(sap_ids); dfree(sap_qs);
    dfree(sap_cursor); dfree(sap_end); dfree(sap_range);
    world_sap = nullptr;
    sap_base = sap_cnt = sap_off = sap_ids = sap_qs = sap_cursor = sap_end = nullptr;
    sap_range = nullptr;
    any_sap = false;
    n_sap_buckets = 0;
  }

  /* Marks the grid worlds of at least sap_min_bodies bodies and sizes their
   * buckets (kSapBuckets per world). */
  void setup_sap() {
    free_sap();
    if (sap_min_bodies <= 0) return;
    std::vector<uint8_t> flag(W, 0);
    std::vector<int32_t> base(W, 0);
    int64_t nb = 0;
    for (int w = 0; w < W; ++w) {
      const int32_t n = h_world_body_off[w + 1] - h_world_body_off[w];
      if (n >= grid_min_bodies && n >= sap_min_bodies) {
        flag[w] = 1;
        base[w] = (int32_t)nb;
        nb += shapes::kSapBuckets;
      }
    }
    if (nb == 0) return;
    if (nb > INT32_MAX / 2) throw CudaError{cudaErrorMemoryAllocation};
    any_sap = true;
    n_sap_buckets = (int32_t)nb;
    world_sap = dalloc<uint8_t>(W, "cudaMalloc sweep");
    sap_base = dalloc<int32_t>(W, "cudaMalloc sweep");
    sap_cnt = dalloc<int32_t>((size_t)nb + 1, "cudaMalloc sweep");
    sap_off = dalloc<int32_t>((size_t)nb + 1, "cudaMalloc sweep");
    sap_ids = dalloc<int32_t>(std::max<int32_t>(N, 1), "cudaMalloc sweep");
    sap_qs = dalloc<int32_t>(std::max<int32_t>(N, 1), "cudaMalloc sweep");
    sap_cursor = dalloc<int32_t>(std::max<int32_t>(N, 1), "cudaMalloc sweep");
    sap_end = dalloc<int32_t>(W, "cudaMalloc sweep");
    sap_range = dalloc<uint64_t>(2 * (size_t)W, "cudaMalloc sweep");
    ck(cudaMemcpy(world_sap, flag.data(), W, cudaMemcpyHostToDevice), "upload sweep");
    ck(cudaMemcpy(sap_base, base.data(), sizeof(int32_t) * W, cudaMemcpyHostToDevice), "upload sweep");
    if (tile_sums && tile_cap < scan_tiles_needed()) { /* the sweep buckets' scan is the longest */
      dfree(tile_sums);
      tile_cap = scan_tiles_needed();
      tile_sums = dalloc<int32_t>(tile_cap, "cudaMalloc scan");
    }
  }
  int32_t* np_cls = nullptr; /* [2 * kNpClasses + 1] */
  int32_t* world_pair_off = nullptr;
  /* contacts: ping-pong between two buffers, the cache of step s is the
   * contact keys + Lagrangians of step s */
  uint64_t* c_key[2] = {nullptr, nullptr};
  double* lam[2] = {nullptr, nullptr};
  int32_t* cwo[2] = {nullptr, nullptr};
  int cache_buf = 0;   /* buffer holding the current cache */
  int results_buf = 0; /* buffer holding the last pairs/contacts results */
  bool have_results = false;
  int32_t* c_ga = nullptr;
  int32_t* c_slot = nullptr; /* [contact_cap] slot of each contact */
  int32_t* c_gb = nullptr;
  uint8_t* c_flip = nullptr;
  uint8_t* c_hit = nullptr;
  double* c_val = nullptr;
  Con* con = nullptr;
  /* scheduler */
  int32_t* last = nullptr;
  int32_t* last_hit = nullptr; /* [N] scheduler scratch: last cache-hit contact of a body */
  int4* c_pred = nullptr;      /* [contact_cap] previous contacts of each side (any / hit) */
  int32_t* c_lvl = nullptr;    /* [2 * contact_cap] dependency levels of two consecutive passes */
  uint32_t* items = nullptr;
  int32_t* ilevel = nullptr;
  uint32_t* isorted = nullptr;
  int32_t* ihist = nullptr;
  int4* gdesc = nullptr;
  int4* idesc = nullptr;
  int32_t* ghist = nullptr;
  long long* phase_clock = nullptr; /* [8 * G], allocated while profiling */
  int32_t phase_clock_groups = 0;
  int32_t* world_levels = nullptr;
  int32_t* group_depth = nullptr;
  int32_t* group_world_off = nullptr;
  int32_t* group_worlds = nullptr;
  std::vector<int32_t> h_group_world_off;
  std::vector<int32_t> h_group_worlds;
  int32_t grouped_iterations = -1;
  /* worlds solved by the large-world paths (not packed into warp groups) */
  int32_t large_world_bodies = SHAPES_LARGE_WORLD_BODIES;
  std::vector<int32_t> large_worlds;
  int32_t lw_nb_max = 0;
  int32_t* lw_bcnt = nullptr;
  int32_t* lw_bstart = nullptr;
  int32_t* lw_bh = nullptr;
  int32_t* lw_bn = nullptr;
  int32_t* lw_done = nullptr;
  int32_t* lw_refs = nullptr;
  int32_t* lw_rank = nullptr;
  int32_t* lw_hrank = nullptr;
  int32_t* lw_hitflag = nullptr;
  int32_t* lw_hitoff = nullptr;
  int32_t* lw_rowflag = nullptr; /* ordered path by rows: row starts (flag, scanned, list) */
  int32_t* lw_rowoff = nullptr;
  int32_t* lw_row_start = nullptr;
  int4* lw_side = nullptr;
  int32_t* lw_color = nullptr;
  int32_t* lw_color_cnt = nullptr;
  int32_t* lw_color_list = nullptr;
  int32_t* lw_seqflag = nullptr;
  int32_t* lw_seqoff = nullptr;
  int32_t* lw_seq_list = nullptr;
  unsigned long long* lw_ctl = nullptr; /* 8 per large world */
  int32_t worlds_per_group_override = 0;
  int32_t target_group_bodies = 0;
  int32_t solve_threads = 32;
  int32_t group_warps = 1; /* > 1: that many warps cooperate on each group (k_group_solve) */
  bool parallel_levels = true; /* cooperative groups: dependency levels by chunked fixed point */
  bool spread_heavy = false;   /* cooperative groups: heaviest groups first, one per SM, then lightest first */
  int num_sms() {
    if (sm_count <= 0) {
      int dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, dev);
      if (sm_count <= 0) sm_count = 1;
    }
    return sm_count;
  }
  int sm_count = 0;
  std::vector<int32_t> world_order; /* packing order of the worlds; empty = by body count */
  /* scans */
  int32_t* tile_sums = nullptr;
  int32_t tile_cap = 0;
  unsigned long long* counters = nullptr;
  double* world_residual = nullptr;
  double* world_depth = nullptr;
  bool residual_valid = false;
  /* world mutation: filled slots (device copy allocated on the first delete)
   * and each world's stack of empty slots (world-local slot ids) */
  uint8_t* active = nullptr;
  std::vector<uint8_t> h_active;
  std::vector<int32_t> h_vert_off;
  std::vector<double> h_radius; /* [N] circle radii, 0 for hulls */
  std::vector<std::vector<int32_t>> h_empties;
  /* learned warm start */
  const shapes_mlp* mlp_model = nullptr;
  uint8_t* learned_mask = nullptr; /* [W] */
  double* judge_res = nullptr;     /* [W] */
  double* judge_depth = nullptr;   /* [W] */
  bool judge_set = false;
  int32_t miss_cap = 0;            /* contact capacity the row buffers were sized for */
  int32_t* miss_flag = nullptr;
  int32_t* miss_off = nullptr;
  int32_t* miss_ids = nullptr;
  int32_t* miss_n = nullptr;
  float* mfeat = nullptr;
  /* training samples */
  float* ds_feat = nullptr;
  float* ds_tgt = nullptr;
  int64_t ds_cap = 0;
  unsigned long long* ds_count = nullptr;
  unsigned long long* snap_ds_count = nullptr;
  uint8_t* snap_mask = nullptr;
  /* snapshot for retries */
  double* snap_body[6] = {nullptr};
  uint64_t* snap_key = nullptr;
  double* snap_lam = nullptr;
  int32_t* snap_cwo = nullptr;
  int32_t snap_cap = 0;

  shapes_stats stats{};

  /* CUDA graphs: one captured step per write buffer, replayed while the
   * configuration and every buffer the step touches stay the same.  Anything
   * that reallocates a buffer, regroups the solver or changes which kernels a
   * step launches bumps graph_epoch. */
  bool graphs_enabled = true;
  uint64_t graph_epoch = 1;
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t epoch = 0;
    shapes_config cfg{};
  };
  StepGraph graph[2];
  int64_t graph_captures = 0;

  void invalidate_graphs() { ++graph_epoch; }

  void drop_graphs() {
    for (auto& g : graph) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
    }
  }

  /* One solver step writing buffer wb: replayed from its graph, captured on
   * first use (or after an invalidation).  Profiling records events between
   * stages, so profiled steps are launched directly. */
  void launch_step(const shapes_config& cfg, int wb) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (graphs_enabled && !profiling && stream != cudaStreamLegacy && stream != cudaStreamPerThread)
      ck(cudaStreamIsCapturing(stream, &cap), "cudaStreamIsCapturing");
    if (!graphs_enabled || profiling || stream == cudaStreamLegacy || stream == cudaStreamPerThread ||
        cap != cudaStreamCaptureStatusNone) { /* a caller's own capture takes the kernels as they are */
      enqueue_step(cfg, true, wb);
      return;
    }
    StepGraph& g = graph[wb];
    if (!g.exec || g.epoch != graph_epoch || std::memcmp(&g.cfg, &cfg, sizeof cfg) != 0) {
      if (g.exec) cudaGraphExecDestroy(g.exec);
      g.exec = nullptr;
      cudaGraph_t gr = nullptr;
      ck(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
      try {
        enqueue_step(cfg, true, wb);
      } catch (...) {
        cudaStreamEndCapture(stream, &gr);
        if (gr) cudaGraphDestroy(gr);
        throw;
      }
      ck(cudaStreamEndCapture(stream, &gr), "cudaStreamEndCapture");
      const cudaError_t e = cudaGraphInstantiate(&g.exec, gr, 0);
      cudaGraphDestroy(gr);
      ck(e, "cudaGraphInstantiate");
      g.epoch = graph_epoch;
      g.cfg = cfg;
      ++graph_captures;
    }
    ck(cudaGraphLaunch(g.exec, stream), "cudaGraphLaunch");
  }

  /* caller stream + per-stage profiling */
  cudaStream_t own_stream = nullptr;
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<int> ev_stage; /* stage of each recorded (start, end) pair */
  size_t ev_used = 0;
  double prof_ms[SHAPES_STAGE_COUNT] = {0};
  int64_t prof_launches[SHAPES_STAGE_COUNT] = {0};

  cudaEvent_t next_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e;
      ck(cudaEventCreate(&e), "cudaEventCreate");
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }

  /* Brackets `launches` kernel launches of stage `st` issued by f(). */
  template <typename F>
  void stage(int st, int launches, F&& f) {
    if (!profiling) {
      f();
      return;
    }
    ck(cudaEventRecord(next_event(), stream), "cudaEventRecord");
    f();
    ck(cudaEventRecord(next_event(), stream), "cudaEventRecord");
    ev_stage.push_back(st);
    prof_launches[st] += launches;
  }

  /* Accumulates the recorded stage times (stream already synchronized). */
  void collect_profile() {
    for (size_t k = 0; k < ev_stage.size(); ++k) {
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, ev_pool[2 * k], ev_pool[2 * k + 1]), "cudaEventElapsedTime");
      prof_ms[ev_stage[k]] += ms;
    }
    ev_stage.clear();
    ev_used = 0;
  }

  Dev view(int write_buf) const {
    Dev d{};
    d.n_worlds = W;
    d.n_bodies = N;
    d.n_verts = V;
    d.pair_cap = pair_cap;
    d.contact_cap = contact_cap;
    d.item_cap = (int32_t)std::min<int64_t>(item_cap, INT32_MAX);
    d.world_body_off = world_body_off;
    d.body_world = body_world;
    d.vert_off = vert_off;
    d.pose_order = pose_order;
    d.ext_chunk = ext_chunk;
    d.ext_chunk_off = ext_chunk_off;
    d.ext_part_sum = ext_part_sum;
    d.ext_part_cnt = ext_part_cnt;
    d.n_ext_chunks = n_ext_chunks;
    if (any_sap) {
      d.world_sap = world_sap;
      d.sap_base = sap_base;
      d.sap_cnt = sap_cnt;
      d.sap_off = sap_off;
      d.n_sap_buckets = n_sap_buckets;
      d.sap_ids = sap_ids;
      d.sap_qs = sap_qs;
      d.sap_cursor = sap_cursor;
      d.sap_range = sap_range;
      d.sap_end = sap_end;
    }
    d.lx = lx;
    d.ly = ly;
    d.radius = radius;
    d.emin = emin;
    d.emax = emax;
    d.vx = body[0];
    d.vy = body[1];
    d.w = body[2];
    d.px = body[3];
    d.py = body[4];
    d.th = body[5];
    d.iml = body[6];
    d.imr = body[7];
    d.mu = body[8];
    d.bounce = body[9];
    d.wx = wx;
    d.wy = wy;
    d.nx = nx;
    d.ny = ny;
    d.plo = plo;
    d.phi = phi;
    d.box = box;
    d.boxk = boxk;
    d.flags = flags;
    d.grid_T = grid_T;
    d.grid_base = grid_base;
    d.grid_inv_s = grid_inv_s;
    d.grid_lim = grid_lim;
    d.bucket_cnt = bucket_cnt;
    d.bucket_off = bucket_off;
    d.grid_ids = grid_ids;
    d.cell_x = cell_x;
    d.cell_y = cell_y;
    d.row_mode = row_mode;
    d.large_cnt = large_cnt;
    d.large_ids = large_ids;
    d.n_buckets = n_buckets;
    if (incremental && nbr) {
      d.fatk = fatk;
      d.nbr = nbr;
      d.nbr_cnt = nbr_cnt;
      d.moved = moved;
      d.inc_state = inc_state;
      d.inc_rebuild = inc_rebuild;
      d.inc_moved = inc_moved;
      d.inc_frames = inc_frames;
      d.inc_margin = inc_margin;
      d.nbr_cap = nbr_cap;
    }
    d.row_cnt = row_cnt;
    d.row_off = row_off;
    d.pair_a = pair_a;
    d.pair_b = pair_b;
    d.slot_cnt = slot_cnt;
    d.slot_off = slot_off;
    d.slot_feat = slot_feat;
    d.np_perm = np_perm;
    d.np_cls = np_cls;
    d.slot_val = slot_val;
    d.c_key = c_key[write_buf];
    d.c_ga = c_ga;
    d.c_slot = c_slot;
    d.c_gb = c_gb;
    d.c_flip = c_flip;
    d.c_hit = c_hit;
    d.c_val = c_val;
    d.con = con;
    d.lam = lam[write_buf];
    d.old_key = c_key[1 - write_buf];
    d.old_lam = lam[1 - write_buf];
    d.old_cwo = cwo[1 - write_buf];
    d.world_pair_off = world_pair_off;
    d.world_contact_off = cwo[write_buf];
    d.last = last;
    d.last_hit = last_hit;
    d.c_pred = c_pred;
    d.c_lvl = c_lvl;
    d.items = items;
    d.ilevel = ilevel;
    d.isorted = isorted;
    d.ihist = ihist;
    d.gdesc = gdesc;
    d.idesc = idesc;
    d.phase_clock = profiling ? phase_clock : nullptr;
    d.ghist = ghist;
    d.world_levels = world_levels;
    d.group_depth = group_depth;
    d.group_world_off = group_world_off;
    d.group_worlds = group_worlds;
    d.counters = counters;
    d.world_residual = world_residual;
    d.world_depth = world_depth;
    d.active = active;
    return d;
  }

  void free_row_buffers() {
    dfree(miss_flag); dfree(miss_off); dfree(miss_ids); dfree(miss_n); dfree(mfeat);
    miss_flag = miss_off = miss_ids = miss_n = nullptr;
    mfeat = nullptr;
    miss_cap = 0;
  }

  /* Feature-row buffers for the learned start / sample collection, sized by
   * the contact capacity (allocated on first use). */
  void ensure_row_buffers() {
    if (miss_cap == contact_cap && miss_flag) return;
    if (stream) ck(cudaStreamSynchronize(stream), "sync");
    invalidate_graphs();
    free_row_buffers();
    miss_flag = dalloc<int32_t>(contact_cap, "cudaMalloc rows");
    miss_off = dalloc<int32_t>((size_t)contact_cap + 1, "cudaMalloc rows");
    miss_ids = dalloc<int32_t>(contact_cap, "cudaMalloc rows");
    miss_n = dalloc<int32_t>(1, "cudaMalloc rows");
    mfeat = dalloc<float>((size_t)contact_cap * mlp::kIn, "cudaMalloc rows");
    miss_cap = contact_cap;
  }

  bool learned_on(const shapes_config& cfg) const {
    return (cfg.flags & SHAPES_FLAG_LEARNED) && mlp_model && cfg.warm_start && ds_cap == 0;
  }
  bool collect_on(const shapes_config& cfg) const { return ds_cap > 0 && cfg.warm_start; }

  void free_step_buffers() {
    dfree(pair_a); dfree(pair_b); dfree(slot_cnt); dfree(slot_off); dfree(slot_feat); dfree(slot_val);
    dfree(np_perm);
    np_perm = nullptr;
    for (int k = 0; k < 2; ++k) { dfree(c_key[k]); dfree(lam[k]); }
    dfree(c_ga); dfree(c_gb); dfree(c_slot); dfree(c_flip); dfree(c_hit); dfree(c_val); dfree(con);
    dfree(c_pred); dfree(c_lvl);
    c_pred = nullptr;
    c_lvl = nullptr;
    dfree(items); dfree(ilevel); dfree(isorted); dfree(ihist); dfree(gdesc); dfree(ghist); dfree(idesc);
    idesc = nullptr;
    dfree(tile_sums);
    dfree(snap_key); dfree(snap_lam);
    free_row_buffers();
    dfree(lw_refs); dfree(lw_rank); dfree(lw_hrank); dfree(lw_hitflag); dfree(lw_hitoff);
    dfree(lw_rowflag); dfree(lw_rowoff); dfree(lw_row_start); dfree(lw_side);
    lw_rowflag = lw_rowoff = lw_row_start = nullptr;
    lw_side = nullptr;
    dfree(lw_color); dfree(lw_color_list); dfree(lw_seqflag); dfree(lw_seqoff); dfree(lw_seq_list);
    lw_refs = lw_rank = lw_hrank = lw_hitflag = lw_hitoff = lw_color = lw_color_list = nullptr;
    lw_seqflag = lw_seqoff = lw_seq_list = nullptr;
    pair_a = pair_b = slot_cnt = slot_off = slot_feat = nullptr;
    slot_val = nullptr;
    c_key[0] = c_key[1] = nullptr;
    lam[0] = lam[1] = nullptr;
    c_ga = c_gb = c_slot = nullptr;
    c_flip = c_hit = nullptr;
    c_val = nullptr;
    con = nullptr;
    items = isorted = nullptr;
    ilevel = ihist = nullptr;
    gdesc = nullptr;
    ghist = nullptr;
    tile_sums = nullptr;
    snap_key = nullptr;
    snap_lam = nullptr;
  }

  /* (Re)allocates every buffer sized by pairs/contacts/updates.  Cache
   * contents in c_key/lam[cache_buf] are preserved across a regrowth. */
  void alloc_step_buffers(int32_t new_pair_cap, int32_t new_contact_cap, int iterations) {
    if (stream) ck(cudaStreamSynchronize(stream), "sync");
    invalidate_graphs();
    const int32_t old_cap = contact_cap;
    uint64_t* keep_key = nullptr;
    double* keep_lam = nullptr;
    if (c_key[cache_buf] && old_cap > 0) {
      keep_key = dalloc<uint64_t>(old_cap, "cudaMalloc keep");
      keep_lam = dalloc<double>(2 * (size_t)old_cap, "cudaMalloc keep");
      ck(cudaMemcpyAsync(keep_key, c_key[cache_buf], sizeof(uint64_t) * old_cap, cudaMemcpyDeviceToDevice, stream), "copy");
      ck(cudaMemcpyAsync(keep_lam, lam[cache_buf], sizeof(double) * 2 * old_cap, cudaMemcpyDeviceToDevice, stream), "copy");
      ck(cudaStreamSynchronize(stream), "sync");
    }
    free_step_buffers();
    pair_cap = new_pair_cap;
    contact_cap = new_contact_cap;
    item_cap = (int64_t)(iterations + 1) * contact_cap;
    pair_a = dalloc<int32_t>(pair_cap, "cudaMalloc pairs");
    pair_b = dalloc<int32_t>(pair_cap, "cudaMalloc pairs");
    slot_cnt = dalloc<int32_t>(pair_cap, "cudaMalloc slots");
    slot_off = dalloc<int32_t>((size_t)pair_cap + 1, "cudaMalloc slots");
    slot_feat = dalloc<int32_t>(2 * (size_t)pair_cap, "cudaMalloc slots");
    slot_val = dalloc<double>(10 * (size_t)pair_cap, "cudaMalloc slots");
    np_perm = dalloc<int32_t>(pair_cap, "cudaMalloc slots");
    for (int k = 0; k < 2; ++k) {
      c_key[k] = dalloc<uint64_t>(contact_cap, "cudaMalloc contacts");
      lam[k] = dalloc<double>(2 * (size_t)contact_cap, "cudaMalloc contacts");
    }
    c_ga = dalloc<int32_t>(contact_cap, "cudaMalloc contacts");
    c_slot = dalloc<int32_t>(contact_cap, "cudaMalloc contacts");
    c_gb = dalloc<int32_t>(contact_cap, "cudaMalloc contacts");
    c_flip = dalloc<uint8_t>(contact_cap, "cudaMalloc contacts");
    c_hit = dalloc<uint8_t>(contact_cap, "cudaMalloc contacts");
    c_val = dalloc<double>(5 * (size_t)contact_cap, "cudaMalloc contacts");
    con = dalloc<Con>(contact_cap, "cudaMalloc constraints");
    c_pred = dalloc<int4>(contact_cap, "cudaMalloc constraints");
    c_lvl = dalloc<int32_t>(2 * (size_t)contact_cap, "cudaMalloc constraints");
    items = dalloc<uint32_t>(1, "cudaMalloc items");
    ilevel = dalloc<int32_t>(item_cap, "cudaMalloc items");
    isorted = dalloc<uint32_t>(1, "cudaMalloc items");
    ihist = dalloc<int32_t>(1, "cudaMalloc items");
    gdesc = dalloc<int4>(item_cap + W + 1, "cudaMalloc items");
    ghist = dalloc<int32_t>(item_cap + W + 1, "cudaMalloc items");
    idesc = dalloc<int4>(item_cap, "cudaMalloc items");
    tile_cap = scan_tiles_needed();
    tile_sums = dalloc<int32_t>(tile_cap, "cudaMalloc scan");
    if (!large_worlds.empty()) {
      lw_refs = dalloc<int32_t>(2 * (size_t)contact_cap, "cudaMalloc large world");
      lw_rank = dalloc<int32_t>(2 * (size_t)contact_cap, "cudaMalloc large world");
      lw_hrank = dalloc<int32_t>(2 * (size_t)contact_cap, "cudaMalloc large world");
      lw_hitflag = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_hitoff = dalloc<int32_t>((size_t)contact_cap + 1, "cudaMalloc large world");
      lw_rowflag = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_rowoff = dalloc<int32_t>((size_t)contact_cap + 1, "cudaMalloc large world");
      lw_row_start = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_side = dalloc<int4>(2 * (size_t)contact_cap, "cudaMalloc large world");
      lw_color = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_color_list = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_seqflag = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
      lw_seqoff = dalloc<int32_t>((size_t)contact_cap + 1, "cudaMalloc large world");
      lw_seq_list = dalloc<int32_t>(contact_cap, "cudaMalloc large world");
    }
    snap_cap = contact_cap;
    snap_key = dalloc<uint64_t>(snap_cap, "cudaMalloc snapshot");
    snap_lam = dalloc<double>(2 * (size_t)snap_cap, "cudaMalloc snapshot");
    if (keep_key) {
      ck(cudaMemcpyAsync(c_key[cache_buf], keep_key, sizeof(uint64_t) * old_cap, cudaMemcpyDeviceToDevice, stream), "copy");
      ck(cudaMemcpyAsync(lam[cache_buf], keep_lam, sizeof(double) * 2 * old_cap, cudaMemcpyDeviceToDevice, stream), "copy");
      ck(cudaStreamSynchronize(stream), "sync");
      dfree(keep_key);
      dfree(keep_lam);
    }
  }

  int32_t cached_iterations = -1;

  void ensure_items(int iterations) {
    if ((int64_t)(iterations + 1) * contact_cap <= item_cap) return;
    ck(cudaStreamSynchronize(stream), "sync");
    invalidate_graphs();
    dfree(items); dfree(ilevel); dfree(isorted); dfree(ihist); dfree(gdesc); dfree(ghist); dfree(idesc);
    item_cap = (int64_t)(iterations + 1) * contact_cap;
    items = dalloc<uint32_t>(item_cap, "cudaMalloc items");
    ilevel = dalloc<int32_t>(item_cap, "cudaMalloc items");
    isorted = dalloc<uint32_t>(1, "cudaMalloc items");
    ihist = dalloc<int32_t>(1, "cudaMalloc items");
    gdesc = dalloc<int4>(item_cap + W + 1, "cudaMalloc items");
    ghist = dalloc<int32_t>(item_cap + W + 1, "cudaMalloc items");
    idesc = dalloc<int4>(item_cap, "cudaMalloc items");
  }

  /* Solver groups: worlds sorted by body count (largest first, so the longest
   * dependency chains start first) and packed `per_group` at a time, so that a
   * level of a group offers about one warp of updates (a world yields about
   * iterations+1 updates per level).  target_group_bodies > 0 overrides the
   * count with "worlds until this many bodies". */
  void make_groups(int iterations) {
    if (stream) ck(cudaStreamSynchronize(stream), "sync"); /* no kernel may still read the old groups */
    invalidate_graphs();
    std::vector<int32_t> order;
    const bool given = (int)world_order.size() == W;
    for (int k = 0; k < W; ++k) {
      const int w = given ? world_order[k] : k;
      if (h_world_body_off[w + 1] - h_world_body_off[w] < large_world_bodies) order.push_back(w);
    }
    const int n_small = (int)order.size();
    if (!given)
      std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (h_world_body_off[a + 1] - h_world_body_off[a]) > (h_world_body_off[b + 1] - h_world_body_off[b]);
      });
    int per_group = std::max(1, std::min(shapes::kMaxGroupWorlds, 32 / (iterations + 1)));
    if (worlds_per_group_override > 0) per_group = std::min(shapes::kMaxGroupWorlds, worlds_per_group_override);
    h_group_world_off.assign(1, 0);
    int32_t max_bodies = 0, bodies = 0, in_group = 0;
    for (int k = 0; k < n_small; ++k) {
      const int w = order[k];
      bodies += h_world_body_off[w + 1] - h_world_body_off[w];
      ++in_group;
      const bool close = target_group_bodies > 0 ? (bodies >= target_group_bodies || in_group == shapes::kMaxGroupWorlds)
                                                 : in_group == per_group;
      if (close || k == n_small - 1) {
        h_group_world_off.push_back(k + 1);
        max_bodies = std::max(max_bodies, bodies);
        bodies = 0;
        in_group = 0;
      }
    }
    h_group_worlds = order;
    dfree(group_world_off);
    dfree(group_worlds);
    dfree(group_depth);
    const size_t G = h_group_world_off.size() - 1;
    /* shared slice per warp (int32 units): last levels (1 per body) during the
     * scan, then velocities (3 doubles = 6 per body) during the solve */
    smem_last_cap = std::min<int32_t>(6 * max_bodies, 10240);
    group_world_off = dalloc<int32_t>(G + 1, "cudaMalloc groups");
    group_worlds = dalloc<int32_t>(std::max(n_small, 1), "cudaMalloc groups");
    group_depth = dalloc<int32_t>(std::max<size_t>(G, 1), "cudaMalloc groups");
    ck(cudaMemcpy(group_world_off, h_group_world_off.data(), sizeof(int32_t) * (G + 1), cudaMemcpyHostToDevice),
       "upload groups");
    if (n_small > 0)
      ck(cudaMemcpy(group_worlds, h_group_worlds.data(), sizeof(int32_t) * n_small, cudaMemcpyHostToDevice),
         "upload groups");
    grouped_iterations = iterations;
    dfree(phase_clock);
    phase_clock = dalloc<long long>(8 * std::max<size_t>(G, 1), "cudaMalloc groups");
    phase_clock_groups = (int32_t)G;
  }

  int num_groups() const { return (int)h_group_world_off.size() - 1; }

  /* Worlds with at least large_world_bodies bodies are solved by the
   * large-world paths; their per-body scratch is sized for the largest. */
  void setup_large_worlds() {
    dfree(lw_bcnt); dfree(lw_bstart); dfree(lw_bh); dfree(lw_bn); dfree(lw_done); dfree(lw_color_cnt); dfree(lw_ctl);
    lw_bcnt = lw_bstart = lw_bh = lw_bn = lw_done = lw_color_cnt = nullptr;
    lw_ctl = nullptr;
    large_worlds.clear();
    lw_nb_max = 0;
    for (int w = 0; w < W; ++w) {
      const int32_t n = h_world_body_off[w + 1] - h_world_body_off[w];
      if (n >= large_world_bodies) {
        large_worlds.push_back(w);
        lw_nb_max = std::max(lw_nb_max, n);
      }
    }
    if (large_worlds.empty()) return;
    lw_bcnt = dalloc<int32_t>((size_t)lw_nb_max + 1, "cudaMalloc large world");
    lw_bstart = dalloc<int32_t>((size_t)lw_nb_max + 1, "cudaMalloc large world");
    lw_bh = dalloc<int32_t>(lw_nb_max, "cudaMalloc large world");
    lw_bn = dalloc<int32_t>(lw_nb_max, "cudaMalloc large world");
    lw_done = dalloc<int32_t>(lw_nb_max, "cudaMalloc large world");
    lw_color_cnt = dalloc<int32_t>(shapes::kMaxColors + 1, "cudaMalloc large world");
    lw_ctl = dalloc<unsigned long long>(8 * large_worlds.size(), "cudaMalloc large world");
    ck(cudaMemset(lw_ctl, 0, sizeof(unsigned long long) * 8 * large_worlds.size()), "memset");
    if (!metric_part) metric_part = dalloc<double>(shapes::kMetricParts, "cudaMalloc large world");
  }

  shapes::LW lw_view(size_t k) const {
    shapes::LW w{};
    w.wld = large_worlds[k];
    w.b0 = h_world_body_off[w.wld];
    w.nb = h_world_body_off[w.wld + 1] - w.b0;
    w.bcnt = lw_bcnt;
    w.bstart = lw_bstart;
    w.refs = lw_refs;
    w.rank = lw_rank;
    w.hrank = lw_hrank;
    w.bh = lw_bh;
    w.bn = lw_bn;
    w.done = lw_done;
    w.hitflag = lw_hitflag;
    w.hitoff = lw_hitoff;
    w.rowflag = lw_rowflag;
    w.rowoff = lw_rowoff;
    w.row_start = lw_row_start;
    w.side = lw_side;
    w.color = lw_color;
    w.color_cnt = lw_color_cnt;
    w.color_list = lw_color_list;
    w.seqflag = lw_seqflag;
    w.seqoff = lw_seqoff;
    w.seq_list = lw_seq_list;
    w.ctl = lw_ctl + 8 * k;
    return w;
  }

  /* Solve one large world: ranks of every contact on its bodies, then the
   * ordered dataflow kernel, or the coloured sweep. */
  /* Per-world residual (or largest depth): one warp per world, and for each
   * large world kMetricParts warps plus an ordered combine. */
  void world_metric_kernels(const Dev& d, bool residual) {
    const int split = large_worlds.empty() ? INT32_MAX : large_world_bodies;
    if (residual)
      shapes::k_residual<<<(W * 32 + 127) / 128, 128, 0, stream>>>(d, split);
    else
      shapes::k_world_depth<<<(W * 32 + 127) / 128, 128, 0, stream>>>(d, split);
    for (int wld : large_worlds) {
      if (residual) {
        shapes::k_metric_part<true><<<shapes::kMetricParts / 4, 128, 0, stream>>>(d, wld, metric_part);
        shapes::k_metric_final<true><<<1, 32, 0, stream>>>(d, wld, metric_part);
      } else {
        shapes::k_metric_part<false><<<shapes::kMetricParts / 4, 128, 0, stream>>>(d, wld, metric_part);
        shapes::k_metric_final<false><<<1, 32, 0, stream>>>(d, wld, metric_part);
      }
    }
  }

  void solve_large_world(const Dev& d, size_t k, const shapes_config& cfg) {
    shapes::LW w = lw_view(k);
    const int cap = contact_cap;
    const bool ordered = !(cfg.flags & SHAPES_FLAG_COLOURED);
    stage(3, ordered ? 18 : 11, [&]() {
      shapes::k_lw_setup<<<grid_for(w.nb + 1, 256), 256, 0, stream>>>(d, w);
      shapes::k_lw_count<<<grid_for(cap, 256), 256, 0, stream>>>(d, w);
      scan_raw(w.bcnt, w.nb, nullptr, w.bstart);
      shapes::k_lw_scatter<<<grid_for(cap, 256), 256, 0, stream>>>(d, w);
      shapes::k_lw_rank<<<grid_for(w.nb, 128), 128, 0, stream>>>(d, w);
      scan_raw(w.hitflag, cap, w.ctl + 4, w.hitoff);
      shapes::k_lw_item_counts<<<1, 1, 0, stream>>>(w, counters + shapes::kCntHits, counters + shapes::kCntItems,
                                                    cfg.iterations);
      if (ordered) { /* the sequence's rows (runs of contacts with one first body), pass skew, side entries */
        shapes::k_lw_rowflag<<<grid_for(cap, 256), 256, 0, stream>>>(d, w);
        scan_raw(w.rowflag, cap, w.ctl + 4, w.rowoff);
        shapes::k_lw_row_list<<<grid_for(cap, 256), 256, 0, stream>>>(w);
        shapes::k_lw_skew<<<grid_for(cap, 256), 256, 0, stream>>>(d, w);
        shapes::k_lw_side<<<grid_for(2 * cap, 256), 256, 0, stream>>>(d, w);
      }
    });
    const int passes = cfg.iterations + (cfg.warm_start ? 1 : 0);
    const int colour_launches = 1 + 128 + 1 + 3 + 1 + 3 + 1 + passes * (shapes::kSeqColor + 1);
    stage(4, (ordered ? 1 : colour_launches) + (cfg.external ? 1 : 0), [&]() {
      if (cfg.external)
        shapes::k_lw_gravity<<<grid_for(w.nb, 256), 256, 0, stream>>>(d, w, cfg.accel_x, cfg.accel_y, cfg.dt);
      if (ordered) {
        shapes::k_lw_ordered<<<kSMs * shapes::kOrderedBlocksPerSM, shapes::kOrderedThreads, 0, stream>>>(
            d, w, cfg.iterations, cfg.warm_start, lw_poll_limit);
        return;
      }
      shapes::k_lw_color_init<<<grid_for(cap, 256), 256, 0, stream>>>(w);
      /* Jones-Plassmann rounds until every contact has a colour (rounds after
       * that return at once; whatever is left after the last goes to the
       * sequential colour) */
      for (int r = 0; r < 128; ++r) shapes::k_lw_color_round<<<grid_for(cap, 256), 256, 0, stream>>>(d, w, r);
      shapes::k_lw_color_count<<<grid_for(cap, 256), 256, 0, stream>>>(w);
      scan_raw(w.color_cnt, shapes::kMaxColors, nullptr, w.color_cnt);
      shapes::k_lw_color_scatter<<<grid_for(cap, 256), 256, 0, stream>>>(w);
      scan_raw(w.seqflag, cap, w.ctl + 4, w.seqoff);
      shapes::k_lw_seq_list<<<grid_for(cap, 256), 256, 0, stream>>>(w);
      for (int pass = cfg.warm_start ? 0 : 1; pass <= cfg.iterations; ++pass) {
        for (int col = 0; col < shapes::kSeqColor; ++col)
          shapes::k_lw_color_pass<<<grid_for(cap / 8 + 1, 128), 128, 0, stream>>>(d, w, col, pass == 0);
        shapes::k_lw_color_seq<<<1, 32, 0, stream>>>(d, w, pass == 0);
      }
    });
  }

  void free_incremental() {
    dfree(fatk); dfree(nbr); dfree(nbr_cnt); dfree(moved); dfree(inc_state); dfree(inc_rebuild); dfree(inc_moved);
    dfree(inc_frames); dfree(inc_margin);
    fatk = nullptr;
    nbr = nullptr;
    nbr_cnt = nullptr;
    moved = nullptr;
    inc_state = inc_rebuild = inc_moved = inc_frames = nullptr;
    inc_margin = nullptr;
  }

  /* Adjacency lists of nbr_cap entries per body; every world rebuilds next frame. */
  void setup_incremental() {
    free_incremental();
    if (!any_grid) return;
    fatk = dalloc<uint64_t>(4 * (size_t)N, "cudaMalloc grid");
    nbr = dalloc<int32_t>((size_t)N * nbr_cap, "cudaMalloc grid");
    nbr_cnt = dalloc<int32_t>(N, "cudaMalloc grid");
    moved = dalloc<uint8_t>(N, "cudaMalloc grid");
    inc_state = dalloc<int32_t>(W, "cudaMalloc grid");
    inc_rebuild = dalloc<int32_t>(W, "cudaMalloc grid");
    inc_moved = dalloc<int32_t>(W, "cudaMalloc grid");
    inc_frames = dalloc<int32_t>(W, "cudaMalloc grid");
    inc_margin = dalloc<double>(W, "cudaMalloc grid");
    reset_incremental();
  }

  void reset_incremental() {
    if (inc_state) ck(cudaMemsetAsync(inc_state, 0, sizeof(int32_t) * W, stream), "memset");
  }

  /* Worlds with at least grid_min_bodies bodies use the grid broadphase. */
  void setup_grid() {
    dfree(grid_T); dfree(grid_base); dfree(grid_inv_s); dfree(grid_lim); dfree(bucket_cnt); dfree(bucket_off);
    dfree(grid_ids); dfree(cell_x); dfree(cell_y); dfree(row_mode); dfree(large_cnt); dfree(large_ids);
    std::vector<int32_t> T(W), base(W);
    int64_t nb = 0;
    any_grid = false;
    for (int w = 0; w < W; ++w) {
      const int32_t n = h_world_body_off[w + 1] - h_world_body_off[w];
      int32_t t = 0;
      if (n >= grid_min_bodies) {
        t = 1;
        while (t < 2 * n) t <<= 1;
        any_grid = true;
      }
      T[w] = t;
      base[w] = (int32_t)nb;
      nb += t;
    }
    if (nb > INT32_MAX / 2) throw CudaError{cudaErrorMemoryAllocation};
    n_buckets = (int32_t)nb;
    grid_T = dalloc<int32_t>(W, "cudaMalloc grid");
    grid_base = dalloc<int32_t>(W, "cudaMalloc grid");
    grid_inv_s = dalloc<double>(W, "cudaMalloc grid");
    grid_lim = dalloc<double>(W, "cudaMalloc grid");
    bucket_cnt = dalloc<int32_t>((size_t)n_buckets + 1, "cudaMalloc grid");
    bucket_off = dalloc<int32_t>((size_t)n_buckets + 1, "cudaMalloc grid");
    grid_ids = dalloc<int32_t>(N, "cudaMalloc grid");
    cell_x = dalloc<int32_t>(N, "cudaMalloc grid");
    cell_y = dalloc<int32_t>(N, "cudaMalloc grid");
    row_mode = dalloc<uint8_t>(N, "cudaMalloc grid");
    large_cnt = dalloc<int32_t>(W, "cudaMalloc grid");
    large_ids = dalloc<int32_t>(N, "cudaMalloc grid");
    ck(cudaMemcpy(grid_T, T.data(), sizeof(int32_t) * W, cudaMemcpyHostToDevice), "upload grid");
    ck(cudaMemcpy(grid_base, base.data(), sizeof(int32_t) * W, cudaMemcpyHostToDevice), "upload grid");
    ck(cudaMemset(row_mode, 0, N), "memset");
    {
      /* chunks of at most 4096 bodies, never crossing a world (empty worlds have none) */
      dfree(ext_chunk); dfree(ext_chunk_off); dfree(ext_part_sum); dfree(ext_part_cnt);
      std::vector<int32_t> ranges, choff(W + 1, 0);
      for (int w = 0; w < W; ++w) {
        choff[w] = (int32_t)(ranges.size() / 2);
        for (int32_t b = h_world_body_off[w]; b < h_world_body_off[w + 1]; b += 4096) {
          ranges.push_back(b);
          ranges.push_back(std::min<int32_t>(b + 4096, h_world_body_off[w + 1]));
        }
      }
      n_ext_chunks = (int32_t)(ranges.size() / 2);
      choff[W] = n_ext_chunks;
      ext_chunk = dalloc<int32_t>(std::max<size_t>(ranges.size(), 1), "cudaMalloc grid");
      ext_chunk_off = dalloc<int32_t>((size_t)W + 1, "cudaMalloc grid");
      ext_part_sum = dalloc<double>(std::max<int32_t>(n_ext_chunks, 1), "cudaMalloc grid");
      ext_part_cnt = dalloc<int32_t>(std::max<int32_t>(n_ext_chunks, 1), "cudaMalloc grid");
      if (n_ext_chunks)
        ck(cudaMemcpy(ext_chunk, ranges.data(), sizeof(int32_t) * ranges.size(), cudaMemcpyHostToDevice),
           "upload grid");
      ck(cudaMemcpy(ext_chunk_off, choff.data(), sizeof(int32_t) * (W + 1), cudaMemcpyHostToDevice), "upload grid");
    }
    setup_incremental();
    setup_sap();
  }
  int32_t smem_last_cap = 0; /* bodies whose last level fits the solver's shared memory */

  void scan(const int32_t* in, int n_cap, const unsigned long long* n_dev, int32_t* out) {
    stage(6, 3, [&]() { scan_raw(in, n_cap, n_dev, out); });
  }

  void scan_raw(const int32_t* in, int n_cap, const unsigned long long* n_dev, int32_t* out) {
    const int tiles = (n_cap + 1 + shapes::kScanTile - 1) / shapes::kScanTile;
    shapes::k_scan_tiles<<<tiles, shapes::kScanThreads, 0, stream>>>(in, n_cap, n_dev, tile_sums);
    shapes::k_scan_tile_sums<<<1, 1024, 0, stream>>>(tile_sums, tiles);
    shapes::k_scan_apply<<<tiles, shapes::kScanThreads, 0, stream>>>(in, n_cap, n_dev, tile_sums, out);
  }

  void pose(int advance, double dt) {
    Dev d = view(0);
    shapes::k_integrate_pose<<<grid_for(N, 128), 128, 0, stream>>>(d, dt, advance);
  }

  /* Broadphase + narrowphase into buffer `wb`; with `solve`, also constraint
   * build, warm start, sweeps, integration. */
  void enqueue_step(const shapes_config& cfg, bool solve, int wb) {
    Dev d = view(wb);
    const bool learn = solve && learned_on(cfg), collect = solve && collect_on(cfg);
    if (learn || collect) { /* row buffers were sized by run() before this view */
      d.learned_mask = learned_mask;
      d.miss_flag = miss_flag;
      d.miss_off = miss_off;
      d.miss_ids = miss_ids;
      d.miss_n = miss_n;
      d.mfeat = mfeat;
      d.collect_all = collect ? 1 : 0;
      d.judge_res = judge_res;
      d.judge_depth = judge_depth;
    }
    /* pairs/contacts and the group allocator are per step; hits, items and
     * levels add up over the call */
    ck(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * 2, stream), "memset");
    ck(cudaMemsetAsync(counters + shapes::kCntGroupAlloc, 0, sizeof(unsigned long long), stream), "memset");
    const bool inc = any_grid && d.nbr != nullptr;
    const bool sap = any_sap && !inc;
    if (!sap) d.world_sap = nullptr;
    if (inc) {
      stage(0, 7, [&]() {
        ck(cudaMemsetAsync(bucket_cnt, 0, sizeof(int32_t) * ((size_t)n_buckets + 1), stream), "memset");
        if (n_ext_chunks) shapes::k_extent_parts<<<n_ext_chunks, 256, 0, stream>>>(d, 1);
        shapes::k_inc_stats<<<grid_for(W, 128), 128, 0, stream>>>(d);
        shapes::k_inc_mark<<<grid_for(N, 256), 256, 0, stream>>>(d);
        shapes::k_inc_decide<<<grid_for(W, 128), 128, 0, stream>>>(d);
        shapes::k_inc_remove<<<grid_for(N, 128), 128, 0, stream>>>(d);
        shapes::k_inc_refat<<<grid_for(N, 256), 256, 0, stream>>>(d);
      });
      scan(bucket_cnt, n_buckets, nullptr, bucket_off);
      stage(0, 2, [&]() {
        shapes::k_inc_scatter<<<grid_for(N, 256), 256, 0, stream>>>(d);
        shapes::k_inc_query<<<grid_for(N, 128), 128, 0, stream>>>(d);
      });
    } else if (any_grid) {
      stage(0, 4, [&]() {
        ck(cudaMemsetAsync(bucket_cnt, 0, sizeof(int32_t) * ((size_t)n_buckets + 1), stream), "memset");
        if (n_ext_chunks) shapes::k_extent_parts<<<n_ext_chunks, 256, 0, stream>>>(d, 0);
        shapes::k_grid_stats<<<grid_for(W, 128), 128, 0, stream>>>(d);
        shapes::k_grid_bin<<<grid_for(N, 256), 256, 0, stream>>>(d);
      });
      scan(bucket_cnt, n_buckets, nullptr, bucket_off);
      stage(0, 1, [&]() { shapes::k_grid_scatter<<<grid_for(N, 256), 256, 0, stream>>>(d); });
      if (sap) {
        stage(0, 2, [&]() {
          ck(cudaMemsetAsync(sap_cnt, 0, sizeof(int32_t) * ((size_t)n_sap_buckets + 1), stream), "memset");
          shapes::k_sap_count<<<grid_for(N, 256), 256, 0, stream>>>(d);
        });
        scan(sap_cnt, n_sap_buckets, nullptr, sap_off);
        stage(0, 2, [&]() {
          shapes::k_sap_scatter<<<grid_for(N, 256), 256, 0, stream>>>(d);
          shapes::k_sap_ends<<<grid_for(W, 128), 128, 0, stream>>>(d);
        });
      }
    }
    stage(0, any_grid ? (sap ? 3 : 2) : 1, [&]() {
      shapes::k_broadphase<true><<<grid_for((long long)N * 32, 256), 256, 0, stream>>>(d);
      if (inc)
        shapes::k_inc_rows<true><<<grid_for(N, 128), 128, 0, stream>>>(d);
      else if (any_grid)
        shapes::k_grid_rows<true><<<grid_for(N, 128), 128, 0, stream>>>(d);
      if (sap) shapes::k_sap_rows<true><<<grid_for(N, 128), 128, 0, stream>>>(d);
    });
    scan(row_cnt, N, nullptr, row_off);
    stage(0, any_grid ? (sap ? 4 : 3) : 1, [&]() {
      shapes::k_broadphase<false><<<grid_for((long long)N * 32, 256), 256, 0, stream>>>(d);
      if (inc)
        shapes::k_inc_rows<false><<<grid_for(N, 128), 128, 0, stream>>>(d);
      else if (any_grid)
        shapes::k_grid_rows<false><<<grid_for(N, 128), 128, 0, stream>>>(d);
      if (sap) shapes::k_sap_rows<false><<<grid_for(N, 128), 128, 0, stream>>>(d);
      if (any_grid) shapes::k_grid_sort_rows<<<grid_for(N, 128), 128, 0, stream>>>(d);
    });
    stage(6, 1, [&]() { shapes::k_world_pair_offsets<<<grid_for(W + 1, 128), 128, 0, stream>>>(d); });
    stage(1, 4, [&]() {
      ck(cudaMemsetAsync(np_cls, 0, sizeof(int32_t) * shapes::kNpClasses, stream), "memset");
      shapes::k_np_count<<<grid_for(pair_cap, 256), 256, 0, stream>>>(d);
      shapes::k_np_offsets<<<1, 32, 0, stream>>>(d);
      shapes::k_np_scatter<<<grid_for(pair_cap, 256), 256, 0, stream>>>(d);
      switch (np_lanes) {
        case 2: shapes::k_narrowphase_lanes<2><<<grid_for(2LL * pair_cap, 128), 128, 0, stream>>>(d); break;
        case 4: shapes::k_narrowphase_lanes<4><<<grid_for(4LL * pair_cap, 128), 128, 0, stream>>>(d); break;
        case 8: shapes::k_narrowphase_lanes<8><<<grid_for(8LL * pair_cap, 128), 128, 0, stream>>>(d); break;
        case 16: shapes::k_narrowphase_lanes<16><<<grid_for(16LL * pair_cap, 128), 128, 0, stream>>>(d); break;
        case 32: shapes::k_narrowphase_lanes<32><<<grid_for(32LL * pair_cap, 128), 128, 0, stream>>>(d); break;
        default: shapes::k_narrowphase<<<grid_for(pair_cap, 128), 128, 0, stream>>>(d);
      }
    });
    scan(slot_cnt, pair_cap, counters + shapes::kCntPairs, slot_off);
    stage(6, 1, [&]() { shapes::k_world_contact_offsets<<<grid_for(W + 1, 128), 128, 0, stream>>>(d); });
    stage(2, 2, [&]() {
      shapes::k_contact_slots<<<grid_for(2LL * pair_cap, 256), 256, 0, stream>>>(d);
      shapes::k_build<<<grid_for(contact_cap, 128), 128, 0, stream>>>(d, cfg.dt, cfg.baumgarte, cfg.slop,
                                                                      cfg.warm_start, solve ? 1 : 0);
    });
    if (!solve) return;
    if (learn || collect) {
      stage(7, 4 + (learn ? 2 : 0), [&]() {
        scan_raw(miss_flag, contact_cap, counters + shapes::kCntContacts, miss_off);
        shapes::k_learned_features<<<grid_for(contact_cap, 128), 128, 0, stream>>>(d, cfg.external, cfg.accel_x,
                                                                                  cfg.accel_y, cfg.dt);
        if (learn) {
          ck(mlp::launch_predict_contacts(mlp::device_params(mlp_model), mlp::device_norm(mlp_model), mfeat, miss_n,
                                          miss_ids, d.lam, c_hit, shapes::kInfoHit,
                                          counters + shapes::kCntPredicted,
                                          reinterpret_cast<int*>(counters + shapes::kCntMlpErr), contact_cap, stream),
             "k_mlp_predict");
          if (judge_set) world_metric_kernels(d, false);
        }
      });
    }
    const int G = num_groups(); /* groups for cfg.iterations were built by run() before this view */
    const int wpc = solve_threads / 32;
    /* each warp's slice of last levels: 40 KB of dynamic shared memory in all (static use is ~1 KB) */
    const int per_warp = std::min<int>(smem_last_cap, (40 * 1024 / (int)sizeof(int32_t)) / wpc) & ~1;
    if (G > 0 && group_warps > 1) {
      /* one group per CTA of group_warps warps, the group's slice up to 40 KB */
      const int ints = std::min<int>(smem_last_cap, 40 * 1024 / (int)sizeof(int32_t)) & ~1;
      const size_t bytes = (size_t)ints * sizeof(int32_t);
      stage(4, 1, [&]() {
#define SHAPES_GROUP_SOLVE(PW, PL)                                                                              \
  shapes::k_group_solve<PW, PL><<<G, 32 * PW, bytes, stream>>>(d, cfg.iterations, cfg.warm_start, cfg.external, \
                                                               cfg.accel_x, cfg.accel_y, cfg.dt, G, ints,  \
                                                               spread_heavy ? num_sms() : 0)
        if (parallel_levels) {
          if (group_warps == 2) SHAPES_GROUP_SOLVE(2, true);
          else if (group_warps == 4) SHAPES_GROUP_SOLVE(4, true);
          else SHAPES_GROUP_SOLVE(8, true);
        } else {
          if (group_warps == 2) SHAPES_GROUP_SOLVE(2, false);
          else if (group_warps == 4) SHAPES_GROUP_SOLVE(4, false);
          else SHAPES_GROUP_SOLVE(8, false);
        }
#undef SHAPES_GROUP_SOLVE
      });
    } else if (G > 0) {
      stage(4, 1, [&]() {
        shapes::k_schedule_solve<<<(G + wpc - 1) / wpc, solve_threads, (size_t)wpc * per_warp * sizeof(int32_t),
                                   stream>>>(d, cfg.iterations, cfg.warm_start, cfg.external, cfg.accel_x,
                                             cfg.accel_y, cfg.dt, G, per_warp);
      });
    }
    for (size_t k = 0; k < large_worlds.size(); ++k) solve_large_world(d, k, cfg);
    if ((cfg.flags & SHAPES_FLAG_RESIDUAL) || (learn && judge_set))
      stage(4, 1 + 2 * (int)large_worlds.size(), [&]() { world_metric_kernels(d, true); });
    if (learn && judge_set)
      stage(7, 1, [&]() { shapes::k_learned_judge<<<grid_for(W, 128), 128, 0, stream>>>(d); });
    if (collect)
      stage(7, 2, [&]() {
        shapes::k_collect<<<grid_for(contact_cap, 256), 256, 0, stream>>>(d, ds_feat, ds_tgt, ds_count, ds_cap);
        shapes::k_collect_advance<<<1, 1, 0, stream>>>(miss_n, ds_count, ds_cap);
      });
    stage(5, 1, [&]() { shapes::k_integrate_pose<<<grid_for(N, 128), 128, 0, stream>>>(d, cfg.dt, 1); });
  }

  /* The state a refused or regrown step returns to: the pose-and-velocity
   * fields, the cache (keys, Lagrangians, world offsets), the learned mask and
   * the sample count, copied in one launch. */
  void snapshot_segments(shapes::Segments& sg, int& n, bool to_snap, int cap) {
    n = 0;
    auto add = [&](void* live, void* snap, unsigned long long bytes) {
      sg.src[n] = to_snap ? live : snap;
      sg.dst[n] = to_snap ? snap : live;
      sg.bytes[n] = bytes;
      ++n;
    };
    for (int k = 0; k < 6; ++k) add(body[k], snap_body[k], sizeof(double) * (unsigned long long)N);
    add(c_key[cache_buf], snap_key, sizeof(uint64_t) * (unsigned long long)cap);
    add(lam[cache_buf], snap_lam, sizeof(double) * 2ull * (unsigned long long)cap);
    add(cwo[cache_buf], snap_cwo, sizeof(int32_t) * (unsigned long long)(W + 1));
    if (learned_mask) add(learned_mask, snap_mask, (unsigned long long)W);
    if (ds_count) add(ds_count, snap_ds_count, sizeof(unsigned long long));
  }
  void copy_segments(const shapes::Segments& sg, int n) {
    unsigned long long most = 0;
    for (int k = 0; k < n; ++k) most = std::max(most, sg.bytes[k]);
    const unsigned blocks = (unsigned)std::max<unsigned long long>(1, std::min<unsigned long long>((most / 8 + 255) / 256, 512));
    shapes::k_copy_segments<<<dim3(blocks, (unsigned)n), 256, 0, stream>>>(sg);
    ck(cudaGetLastError(), "launch");
  }
  void snapshot() {
    shapes::Segments sg{};
    int n = 0;
    snapshot_segments(sg, n, true, contact_cap);
    copy_segments(sg, n);
  }

  /* Restore into buffer `buf` (which becomes the cache buffer). */
  void restore(int saved_cap) {
    shapes::Segments sg{};
    int n = 0;
    snapshot_segments(sg, n, false, saved_cap);
    copy_segments(sg, n);
  }

  /* Asynchronous body-state upload for shapes_batches_step_io: caller arrays
   * into the staging arrays with the finiteness check into the bad-input
   * counter, then the staged state into the live arrays unless the check
   * failed, and a re-pose of the bodies whose pose inputs changed. */
  void io_upload(const shapes_bodies* in, double* const* mapped = nullptr);
  void io_commit() {
    shapes::Ptr10 p{};
    for (int k = 0; k < 10; ++k) {
      p.src[k] = body_stage[k];
      p.dst[k] = body[k];
    }
    shapes::k_commit_bodies<<<grid_for(N, 256), 256, 0, stream>>>(p, N, body_changed,
                                                                  counters + shapes::kCntBadInput);
    Dev d = view(0);
    shapes::k_integrate_pose<<<grid_for(N, 128), 128, 0, stream>>>(d, 0.0, 0, body_changed);
    ck(cudaGetLastError(), "launch");
  }
  /* The first `fields` body arrays (10: all; kStepFields: velocities and pose,
   * the only ones a step writes) into the caller's arrays. */
  void io_download(shapes_bodies* out, double* const* mapped = nullptr, int fields = 10);
  /* After an io step was enqueued: waits, and on refused input undoes the
   * step (SHAPES_E_NAN); otherwise finishes it, re-running the staged input
   * alone after a buffer regrowth. */
  int io_finish(const shapes_config& cfg, shapes_bodies* out, double* const* mapped_out = nullptr, int fields = 10);

  /* One call of `nsteps` steps (or one collide when !solve) in three parts,
   * so that several handles can have their steps in flight at once
   * (shapes_batches_step): prepare() sizes buffers and groups, enqueue()
   * snapshots the state for a retry and launches the steps and the read-back
   * of the counters without waiting, finish() (after the stream is drained)
   * checks them: kRunRetry means the buffers were too small, the state was
   * restored and grown, and the call must be enqueued again. */
  static constexpr int kRunRetry = 1;
  int run_retries = 0, run_saved_cache_buf = 0, run_saved_cap = 0;
  /* pinned host copy of the step counters (kCntSlots), so that reading them
   * back is an asynchronous copy and the wait happens where the caller waits */
  unsigned long long* run_counters = nullptr;

  void prepare(const shapes_config& cfg, bool solve) {
    ensure_items(solve ? cfg.iterations : 0);
    /* (re)build the solver groups before any device view of this call is
     * taken: make_groups reallocates the group arrays */
    if (solve && grouped_iterations != cfg.iterations) make_groups(cfg.iterations);
    if (solve && (learned_on(cfg) || collect_on(cfg))) ensure_row_buffers();
  }

  void enqueue_begin(bool solve) {
    ck(cudaMemsetAsync(counters, 0, sizeof(unsigned long long) * shapes::kCntSlots, stream), "memset");
    if (lw_ctl) /* the large-world timeout flags stay set through the run's steps */
      ck(cudaMemsetAsync(lw_ctl, 0, sizeof(unsigned long long) * 8 * large_worlds.size(), stream), "memset");
    run_saved_cache_buf = cache_buf;
    run_saved_cap = contact_cap;
    if (solve) snapshot();
  }
  void enqueue_one(const shapes_config& cfg, bool solve) {
    const int wb = 1 - cache_buf;
    if (solve)
      launch_step(cfg, wb);
    else
      enqueue_step(cfg, false, wb);
    if (solve) cache_buf = wb;
    results_buf = wb;
  }
  void enqueue_end() {
    if (!run_counters) {
      ck(cudaMallocHost(&run_counters, sizeof(unsigned long long) * shapes::kCntSlots), "cudaMallocHost");
      std::memset(run_counters, 0, sizeof(unsigned long long) * shapes::kCntSlots);
    }
    ck(cudaMemcpyAsync(run_counters, counters, sizeof(unsigned long long) * shapes::kCntSlots, cudaMemcpyDeviceToHost,
                       stream),
       "read counters");
  }
  void enqueue(const shapes_config& cfg, int32_t nsteps, bool solve) {
    enqueue_begin(solve);
    for (int s = 0; s < (solve ? nsteps : 1); ++s) enqueue_one(cfg, solve);
    enqueue_end();
  }

  int finish(const shapes_config& cfg, bool solve) {
    ck(cudaStreamSynchronize(stream), "step");
    ck(cudaGetLastError(), "launch");
    if (profiling) collect_profile();
    const unsigned long long* agg = run_counters;
    if (agg[shapes::kCntMlpErr]) {
      g_last_error = "learned warm start: a bounded tensor-core wait gave up";
      return SHAPES_E_TIMEOUT;
    }
    if (!agg[shapes::kCntOverflow] && solve && !large_worlds.empty()) {
      std::vector<unsigned long long> ctl(8 * large_worlds.size());
      ck(cudaMemcpy(ctl.data(), lw_ctl, sizeof(unsigned long long) * ctl.size(), cudaMemcpyDeviceToHost), "ctl");
      for (size_t k = 0; k < large_worlds.size(); ++k)
        if (ctl[8 * k + 1]) {
          g_last_error = "large-world solver: a bounded wait gave up";
          return SHAPES_E_TIMEOUT;
        }
    }
    if (!agg[shapes::kCntOverflow]) {
      stats.pairs = (int64_t)agg[shapes::kCntPairs];
      stats.contacts = (int64_t)agg[shapes::kCntContacts];
      stats.cache_hits = (int64_t)agg[shapes::kCntHits] - (int64_t)agg[shapes::kCntPredicted];
      stats.predicted = (int64_t)agg[shapes::kCntPredicted];
      stats.reverted = (int64_t)agg[shapes::kCntReverted];
      stats.solver_items = (int64_t)agg[shapes::kCntItems];
      stats.solver_levels = (int64_t)agg[shapes::kCntLevels];
      stats.retries = run_retries;
      have_results = true;
      return SHAPES_OK;
    }
    if (++run_retries > 6) return SHAPES_E_CAPACITY;
    /* undo, grow, redo */
    const unsigned long long overflow = agg[shapes::kCntOverflow];
    cache_buf = run_saved_cache_buf;
    if (solve) restore(run_saved_cap);
    ck(cudaStreamSynchronize(stream), "restore");
    if (overflow & 4ull) { /* an adjacency list was full */
      if (nbr_cap > (1 << 14)) return SHAPES_E_CAPACITY;
      nbr_cap *= 2;
      invalidate_graphs();
      setup_incremental();
    }
    reset_incremental(); /* the lists follow the undone steps' poses */
    if (overflow & ~4ull) {
      const int64_t np = (int64_t)pair_cap * ((overflow & 1ull) ? 2 : 1);
      const int64_t nc = (int64_t)contact_cap * 2;
      if (np > INT32_MAX / 2 || nc > INT32_MAX / 2) return SHAPES_E_CAPACITY;
      alloc_step_buffers((int32_t)np, (int32_t)std::max<int64_t>(nc, 2 * np), solve ? cfg.iterations : 0);
    }
    ensure_items(solve ? cfg.iterations : 0);
    if (solve && (learned_on(cfg) || collect_on(cfg))) ensure_row_buffers();
    if (solve) pose(0, 0.0);
    return kRunRetry;
  }

  /* Runs `nsteps` steps (or one collide when !solve) with overflow retries. */
  int run(const shapes_config& cfg, int32_t nsteps, bool solve) {
    prepare(cfg, solve);
    run_retries = 0;
    for (;;) {
      enqueue(cfg, nsteps, solve);
      const int rc = finish(cfg, solve);
      if (rc != kRunRetry) return rc;
    }
  }

  /* The local points in the caller's convention (a circle as (radius, 0)). */
  std::vector<double> local_xy_host() {
    std::vector<double> xs(V), ys(V), xy(2 * (size_t)V);
    ck(cudaMemcpyAsync(xs.data(), lx, sizeof(double) * V, cudaMemcpyDeviceToHost, stream), "download");
    ck(cudaMemcpyAsync(ys.data(), ly, sizeof(double) * V, cudaMemcpyDeviceToHost, stream), "download");
    ck(cudaStreamSynchronize(stream), "download");
    for (int64_t v = 0; v < V; ++v) {
      xy[2 * v] = xs[v];
      xy[2 * v + 1] = ys[v];
    }
    for (int32_t b = 0; b < N; ++b)
      if (h_radius[b] > 0.0) xy[2 * (size_t)h_vert_off[b]] = h_radius[b];
    return xy;
  }

  /* (Re)builds everything sized by the bodies and vertices from host arrays:
   * world offsets [W+1], the ten body arrays, vertex offsets [N+1] and local
   * vertices [2V].  Used by creation and by appends that change the
   * topology; settings, the stream, the network and the judge stay.  The
   * contact cache comes back empty (the caller restores it). */
  void init_topology(const int32_t* world_body_offsets, double* const bp[10], const int32_t* vert_offsets,
                     const double* local_verts_xy) {
    if (stream) ck(cudaStreamSynchronize(stream), "sync");
    invalidate_graphs();
    free_step_buffers();
    dfree(world_body_off); dfree(body_world); dfree(vert_off); dfree(lx); dfree(ly); dfree(emin); dfree(emax);
    dfree(radius);
    dfree(pose_order);
    radius = nullptr;
    for (int k = 0; k < 10; ++k) {
      dfree(body[k]);
      dfree(body_stage[k]);
    }
    dfree(wx); dfree(wy); dfree(nx); dfree(ny); dfree(box); dfree(boxk); dfree(flags); dfree(body_changed);
    dfree(plo); dfree(phi);
    dfree(row_cnt); dfree(row_off); dfree(world_pair_off); dfree(last); dfree(last_hit); dfree(world_levels);
    for (int k = 0; k < 6; ++k) dfree(snap_body[k]);
    dfree(active);
    active = nullptr;
    const int32_t n_worlds = W;
    N = world_body_offsets[n_worlds];
    V = vert_offsets[N];
    h_world_body_off.assign(world_body_offsets, world_body_offsets + n_worlds + 1);
    h_vert_off.assign(vert_offsets, vert_offsets + N + 1);
    h_active.assign(N, 1);
    h_body_world.resize(N);
    for (int w = 0; w < n_worlds; ++w)
      for (int32_t b = world_body_offsets[w]; b < world_body_offsets[w + 1]; ++b) h_body_world[b] = w;
    world_body_off = dalloc<int32_t>(n_worlds + 1, "cudaMalloc");
    body_world = dalloc<int32_t>(N, "cudaMalloc");
    vert_off = dalloc<int32_t>((size_t)N + 1, "cudaMalloc");
    lx = dalloc<double>(V, "cudaMalloc");
    ly = dalloc<double>(V, "cudaMalloc");
    emin = dalloc<int32_t>(V, "cudaMalloc");
    emax = dalloc<int32_t>(V, "cudaMalloc");
    for (int k = 0; k < 10; ++k) body[k] = dalloc<double>(N, "cudaMalloc bodies");
    for (int k = 0; k < 10; ++k) body_stage[k] = dalloc<double>(N, "cudaMalloc bodies");
    wx = dalloc<double>(V, "cudaMalloc");
    wy = dalloc<double>(V, "cudaMalloc");
    nx = dalloc<double>(V, "cudaMalloc");
    ny = dalloc<double>(V, "cudaMalloc");
    plo = dalloc<double>(V, "cudaMalloc");
    phi = dalloc<double>(V, "cudaMalloc");
    box = dalloc<double>(4 * (size_t)N, "cudaMalloc");
    boxk = dalloc<uint64_t>(4 * (size_t)N, "cudaMalloc");
    flags = dalloc<uint8_t>(N, "cudaMalloc");
    body_changed = dalloc<uint8_t>(N, "cudaMalloc");
    row_cnt = dalloc<int32_t>(N, "cudaMalloc");
    row_off = dalloc<int32_t>((size_t)N + 1, "cudaMalloc");
    world_pair_off = dalloc<int32_t>(n_worlds + 1, "cudaMalloc");
    if (!cwo[0])
      for (int k = 0; k < 2; ++k) cwo[k] = dalloc<int32_t>(n_worlds + 1, "cudaMalloc");
    last = dalloc<int32_t>(N, "cudaMalloc");
    last_hit = dalloc<int32_t>(N, "cudaMalloc");
    world_levels = dalloc<int32_t>(n_worlds, "cudaMalloc");
    ck(cudaMemset(world_levels, 0, sizeof(int32_t) * n_worlds), "memset");
    if (!counters) counters = dalloc<unsigned long long>(shapes::kCntSlots, "cudaMalloc");
    if (!np_cls) np_cls = dalloc<int32_t>(2 * shapes::kNpClasses + 1, "cudaMalloc");
    if (!world_residual) world_residual = dalloc<double>(n_worlds, "cudaMalloc");
    if (!world_depth) world_depth = dalloc<double>(n_worlds, "cudaMalloc");
    for (int k = 0; k < 6; ++k) snap_body[k] = dalloc<double>(N, "cudaMalloc snapshot");
    if (!snap_cwo) snap_cwo = dalloc<int32_t>(n_worlds + 1, "cudaMalloc snapshot");
    ck(cudaMemcpy(world_body_off, world_body_offsets, sizeof(int32_t) * (n_worlds + 1), cudaMemcpyHostToDevice),
       "upload");
    ck(cudaMemcpy(body_world, h_body_world.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "upload");
    ck(cudaMemcpy(vert_off, vert_offsets, sizeof(int32_t) * (N + 1), cudaMemcpyHostToDevice), "upload");
    {
      /* pose order: stable counting sort by vertex count within each chunk of
       * 1024 bodies (a warp of the pose kernel then runs one loop length;
       * chunks keep the gathers local) */
      std::vector<int32_t> order(N);
      constexpr int32_t kChunk = 1024;
      for (int32_t c0 = 0; c0 < N; c0 += kChunk) {
        const int32_t c1 = std::min<int32_t>(N, c0 + kChunk);
        int32_t cnt[shapes::kMaxVerts + 2] = {0};
        for (int32_t b = c0; b < c1; ++b) ++cnt[std::min<int32_t>(vert_offsets[b + 1] - vert_offsets[b], shapes::kMaxVerts + 1)];
        int32_t pos[shapes::kMaxVerts + 2];
        int32_t acc = c0;
        for (int k = 0; k < shapes::kMaxVerts + 2; ++k) {
          pos[k] = acc;
          acc += cnt[k];
        }
        for (int32_t b = c0; b < c1; ++b)
          order[pos[std::min<int32_t>(vert_offsets[b + 1] - vert_offsets[b], shapes::kMaxVerts + 1)]++] = b;
      }
      pose_order = dalloc<int32_t>(std::max<int32_t>(N, 1), "cudaMalloc");
      if (N) ck(cudaMemcpy(pose_order, order.data(), sizeof(int32_t) * N, cudaMemcpyHostToDevice), "upload");
    }
    /* a circle's one local point (radius, 0) becomes radius[b] and the local
     * centre (0, 0) (circleWithRadius, Contact/Circle.hs:24-25) */
    h_radius.assign(N, 0.0);
    bool any_circle = false;
    for (int32_t b = 0; b < N; ++b)
      if (vert_offsets[b + 1] - vert_offsets[b] == 1) {
        h_radius[b] = local_verts_xy[2 * (size_t)vert_offsets[b]];
        any_circle = true;
      }
    std::vector<double> tmp(V);
    for (int32_t v = 0; v < V; ++v) tmp[v] = local_verts_xy[2 * (size_t)v];
    for (int32_t b = 0; b < N; ++b)
      if (h_radius[b] > 0.0) tmp[vert_offsets[b]] = 0.0;
    ck(cudaMemcpy(lx, tmp.data(), sizeof(double) * V, cudaMemcpyHostToDevice), "upload");
    for (int32_t v = 0; v < V; ++v) tmp[v] = local_verts_xy[2 * (size_t)v + 1];
    for (int32_t b = 0; b < N; ++b)
      if (h_radius[b] > 0.0) tmp[vert_offsets[b]] = 0.0;
    ck(cudaMemcpy(ly, tmp.data(), sizeof(double) * V, cudaMemcpyHostToDevice), "upload");
    if (any_circle) {
      radius = dalloc<double>(N, "cudaMalloc");
      ck(cudaMemcpy(radius, h_radius.data(), sizeof(double) * N, cudaMemcpyHostToDevice), "upload");
    }
    for (int k = 0; k < 10; ++k) ck(cudaMemcpy(body[k], bp[k], sizeof(double) * N, cudaMemcpyHostToDevice), "upload bodies");
    /* empty cache: every world offset 0 */
    for (int k = 0; k < 2; ++k) ck(cudaMemset(cwo[k], 0, sizeof(int32_t) * (n_worlds + 1)), "memset");
    cache_buf = 0;
    results_buf = 0;
    have_results = false;
    residual_valid = false;
    setup_grid();
    setup_large_worlds();
    contact_cap = 0;
    item_cap = 0;
    const int32_t pcap = (int32_t)std::min<int64_t>(std::max<int64_t>(1024, 8LL * N), INT32_MAX / 4);
    alloc_step_buffers(pcap, 2 * pcap, 8);
    make_groups(grouped_iterations > 0 ? grouped_iterations : 2);
    Dev d = view(0);
    shapes::k_init_extents<<<grid_for(V, 128), 128, 0, stream>>>(d);
    pose(0, 0.0);
    ck(cudaGetLastError(), "launch");
    ck(cudaStreamSynchronize(stream), "create");
  }

  /* Uploads the filled-slot flags (allocated on first use; the step graphs
   * hold the array, so its first allocation re-captures them) and re-poses,
   * which recomputes every body's broadphase flags. */
  void upload_active() {
    bool all = true;
    for (uint8_t a : h_active) all = all && a;
    if (all && !active) return;
    if (!active) {
      if (stream) ck(cudaStreamSynchronize(stream), "sync");
      active = dalloc<uint8_t>(N, "cudaMalloc");
      invalidate_graphs();
    }
    ck(cudaMemcpyAsync(active, h_active.data(), N, cudaMemcpyHostToDevice, stream), "upload");
    pose(0, 0.0);
    ck(cudaStreamSynchronize(stream), "upload");
    have_results = false;
  }

  ~shapes_batch() {
    if (stream) cudaStreamSynchronize(stream);
    drop_graphs();
    free_step_buffers();
    dfree(world_body_off); dfree(body_world); dfree(vert_off); dfree(lx); dfree(ly);
    dfree(emin); dfree(emax);
    dfree(pose_order);
    for (int k = 0; k < 10; ++k) {
      dfree(body[k]);
      dfree(body_stage[k]);
    }
    dfree(wx); dfree(wy); dfree(nx); dfree(ny); dfree(box); dfree(boxk); dfree(flags); dfree(body_changed);
    dfree(plo); dfree(phi);
    dfree(row_cnt); dfree(row_off); dfree(world_pair_off);
    dfree(grid_T); dfree(grid_base); dfree(grid_inv_s); dfree(grid_lim); dfree(bucket_cnt); dfree(bucket_off);
    dfree(grid_ids); dfree(cell_x); dfree(cell_y); dfree(row_mode); dfree(large_cnt); dfree(large_ids);
    dfree(ext_chunk); dfree(ext_chunk_off); dfree(ext_part_sum); dfree(ext_part_cnt);
    free_sap();
    free_incremental();
    dfree(radius);
    dfree(metric_part);
    for (int k = 0; k < 2; ++k) dfree(cwo[k]);
    dfree(last); dfree(last_hit); dfree(world_levels); dfree(group_depth); dfree(group_world_off); dfree(group_worlds);
    dfree(phase_clock);
    dfree(counters);
    dfree(np_cls);
    dfree(export_keys);
    dfree(export_vals);
    dfree(lw_bcnt); dfree(lw_bstart); dfree(lw_bh); dfree(lw_bn); dfree(lw_done); dfree(lw_color_cnt); dfree(lw_ctl);
    dfree(world_residual);
    dfree(world_depth);
    dfree(learned_mask); dfree(judge_res); dfree(judge_depth);
    dfree(active);
    dfree(ds_feat); dfree(ds_tgt); dfree(ds_count); dfree(snap_ds_count); dfree(snap_mask);
    for (int k = 0; k < 6; ++k) dfree(snap_body[k]);
    dfree(snap_cwo);
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
    if (run_counters) cudaFreeHost(run_counters);
    if (own_stream) cudaStreamDestroy(own_stream);
  }
};

namespace {

bool body_arrays_ok(const shapes_bodies* b) {
  return b && b->vel_x && b->vel_y && b->rot_vel && b->pos_x && b->pos_y && b->rot &&
         b->inv_mass_lin && b->inv_mass_rot && b->mu && b->bounce;
}

double* const* body_ptrs(const shapes_bodies* b, double* out[10]) {
  out[0] = b->vel_x; out[1] = b->vel_y; out[2] = b->rot_vel; out[3] = b->pos_x; out[4] = b->pos_y;
  out[5] = b->rot; out[6] = b->inv_mass_lin; out[7] = b->inv_mass_rot; out[8] = b->mu; out[9] = b->bounce;
  return out;
}

/* Body arrays a step writes: vel_x, vel_y, rot_vel, pos_x, pos_y, rot (the
 * first six of the shapes_bodies order); inverse masses and material stay. */
constexpr int kStepFields = 6;

/* Strictly convex, counter-clockwise, no zero-length edge. */
int check_hull(int nv, const double* xy) {
  if (nv < 3) return SHAPES_E_INVALID_ARG;
  if (nv > shapes::kMaxVerts) return SHAPES_E_UNSUPPORTED;
  for (int k = 0; k < 2 * nv; ++k)
    if (!std::isfinite(xy[k])) return SHAPES_E_NAN;
  for (int k = 0; k < nv; ++k) {
    const int k1 = (k + 1) % nv, k2 = (k + 2) % nv;
    const double ex = xy[2 * k1] - xy[2 * k], ey = xy[2 * k1 + 1] - xy[2 * k + 1];
    const double fx = xy[2 * k2] - xy[2 * k1], fy = xy[2 * k2 + 1] - xy[2 * k1 + 1];
    if (ex == 0.0 && ey == 0.0) return SHAPES_E_INVALID_ARG;
    if (ex * fy - ey * fx <= 0.0) return SHAPES_E_NONCONVEX;
  }
  return SHAPES_OK;
}

/* A circle is one local point (radius, 0) with 0 < radius < 2^500. */
int check_shape(uint8_t kind, int nv, const double* xy) {
  if (kind == SHAPES_SHAPE_HULL) {
    const int rc = check_hull(nv, xy);
    if (rc != SHAPES_OK) g_last_error = "a hull needs 3..64 finite, strictly convex, counter-clockwise vertices";
    return rc;
  }
  g_last_error = "a circle is one local point (radius, 0) with 0 < radius < 2^500";
  if (kind != SHAPES_SHAPE_CIRCLE || nv != 1) {
    if (kind != SHAPES_SHAPE_CIRCLE) g_last_error = "unknown shape kind";
    return SHAPES_E_INVALID_ARG;
  }
  if (!std::isfinite(xy[0]) || !std::isfinite(xy[1])) return SHAPES_E_NAN;
  if (!(xy[0] > 0.0) || xy[0] >= 0x1p500 || xy[1] != 0.0) return SHAPES_E_INVALID_ARG;
  g_last_error.clear();
  return SHAPES_OK;
}

template <typename F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const CudaError&) {
    return SHAPES_E_CUDA;
  } catch (const std::bad_alloc&) {
    g_last_error = "host allocation failed";
    return SHAPES_E_CAPACITY;
  }
}

}  // namespace

extern "C" {

const char* shapes_strerror(int status) {
  switch (status) {
    case SHAPES_OK: return "ok";
    case SHAPES_E_INVALID_ARG: return "invalid argument";
    case SHAPES_E_UNSUPPORTED: return "unsupported shape or option";
    case SHAPES_E_NONCONVEX: return "hull is not strictly convex and counter-clockwise";
    case SHAPES_E_CAPACITY: return "internal buffer could not grow";
    case SHAPES_E_CUDA: return "CUDA error";
    case SHAPES_E_TIMEOUT: return "bounded device wait gave up";
    case SHAPES_E_NAN: return "non-finite body state";
    case SHAPES_E_BUFFER: return "caller buffer too small";
    default: return "unknown status";
  }
}

const char* shapes_last_error_detail(void) { return g_last_error.c_str(); }

int shapes_batch_create(int32_t n_worlds, const int32_t* world_body_offsets, const shapes_bodies* bodies,
                        const int32_t* vert_offsets, const double* local_verts_xy, const uint8_t* shape_kind,
                        shapes_batch** out) {
  g_last_error.clear();
  if (!out || n_worlds < 1 || !world_body_offsets || !vert_offsets || !local_verts_xy || !body_arrays_ok(bodies))
    return SHAPES_E_INVALID_ARG;
  *out = nullptr;
  if (world_body_offsets[0] != 0) return SHAPES_E_INVALID_ARG;
  for (int w = 0; w < n_worlds; ++w) {
    const int32_t n = world_body_offsets[w + 1] - world_body_offsets[w];
    if (n < 0 || n >= (1 << 20)) return SHAPES_E_INVALID_ARG;
  }
  const int32_t N = world_body_offsets[n_worlds];
  if (N < 1) return SHAPES_E_INVALID_ARG;
  if (vert_offsets[0] != 0) return SHAPES_E_INVALID_ARG;
  for (int32_t b = 0; b < N; ++b) {
    const int32_t nv = vert_offsets[b + 1] - vert_offsets[b];
    const int rc = check_shape(shape_kind ? shape_kind[b] : (uint8_t)SHAPES_SHAPE_HULL, nv,
                               local_verts_xy + 2 * (size_t)vert_offsets[b]);
    if (rc != SHAPES_OK) return rc;
  }
  double* bp[10];
  body_ptrs(bodies, bp);
  for (int k = 0; k < 10; ++k)
    for (int32_t b = 0; b < N; ++b)
      if (!std::isfinite(bp[k][b])) return SHAPES_E_NAN;
  return guarded([&]() -> int {
    shapes_batch* h = new shapes_batch();
    try {
      ck(cudaGetDevice(&h->device), "cudaGetDevice");
      ck(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking), "cudaStreamCreate");
      h->stream = h->own_stream;
      h->W = n_worlds;
      h->h_empties.assign(n_worlds, {});
      h->init_topology(world_body_offsets, bp, vert_offsets, local_verts_xy);
    } catch (...) {
      delete h;
      throw;
    }
    *out = h;
    return SHAPES_OK;
  });
}

int shapes_world_create(int32_t n_bodies, const shapes_bodies* bodies, const int32_t* vert_offsets,
                        const double* local_verts_xy, const uint8_t* shape_kind, shapes_batch** out) {
  const int32_t off[2] = {0, n_bodies};
  return shapes_batch_create(1, off, bodies, vert_offsets, local_verts_xy, shape_kind, out);
}

void shapes_batch_destroy(shapes_batch* b) { delete b; }

static int check_cfg(const shapes_config* c) {
  if (!c) return SHAPES_E_INVALID_ARG;
  if (!std::isfinite(c->dt) || !std::isfinite(c->baumgarte) || !std::isfinite(c->slop) ||
      !std::isfinite(c->accel_x) || !std::isfinite(c->accel_y))
    return SHAPES_E_INVALID_ARG;
  if (c->iterations < 0 || c->iterations > 64) return SHAPES_E_INVALID_ARG;
  if (c->warm_start != SHAPES_WARM_START_OFF && c->warm_start != SHAPES_WARM_START_CACHE)
    return SHAPES_E_UNSUPPORTED;
  if (c->external != SHAPES_EXTERNAL_NONE && c->external != SHAPES_EXTERNAL_CONSTANT_ACCEL)
    return SHAPES_E_UNSUPPORTED;
  if (c->flags & ~(SHAPES_FLAG_RESIDUAL | SHAPES_FLAG_COLOURED | SHAPES_FLAG_LEARNED)) return SHAPES_E_INVALID_ARG;
  return SHAPES_OK;
}

int shapes_batch_step(shapes_batch* b, const shapes_config* cfg, int32_t nsteps) {
  if (!b || nsteps < 0) return SHAPES_E_INVALID_ARG;
  const int rc = check_cfg(cfg);
  if (rc != SHAPES_OK) return rc;
  if (nsteps == 0) return SHAPES_OK;
  return guarded([&]() -> int {
    ck(cudaSetDevice(b->device), "cudaSetDevice");
    const int rc = b->run(*cfg, nsteps, true);
    b->residual_valid = rc == SHAPES_OK && ((cfg->flags & SHAPES_FLAG_RESIDUAL) || b->learned_on(*cfg));
    return rc;
  });
}

int shapes_batches_step(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, int32_t nsteps) {
  if (!bs || n < 1 || nsteps < 0) return SHAPES_E_INVALID_ARG;
  for (int32_t k = 0; k < n; ++k) {
    if (!bs[k]) return SHAPES_E_INVALID_ARG;
    for (int32_t j = 0; j < k; ++j)
      if (bs[j] == bs[k] || bs[j]->stream == bs[k]->stream) return SHAPES_E_INVALID_ARG;
  }
  const int rc0 = check_cfg(cfg);
  if (rc0 != SHAPES_OK) return rc0;
  if (nsteps == 0) return SHAPES_OK;
  return guarded([&]() -> int {
    /* every handle's steps in flight on its own stream, launched step by
     * step in turn (a stream's launch queue is finite: launching all of one
     * handle's steps first would block until most of them had run), then
     * each finished */
    for (int32_t k = 0; k < n; ++k) {
      ck(cudaSetDevice(bs[k]->device), "cudaSetDevice");
      bs[k]->prepare(*cfg, true);
      bs[k]->run_retries = 0;
      bs[k]->enqueue_begin(true);
    }
    for (int32_t s = 0; s < nsteps; ++s)
      for (int32_t k = 0; k < n; ++k) bs[k]->enqueue_one(*cfg, true);
    for (int32_t k = 0; k < n; ++k) bs[k]->enqueue_end();
    int rc = SHAPES_OK;
    for (int32_t k = 0; k < n; ++k) {
      shapes_batch* b = bs[k];
      int r = b->finish(*cfg, true);
      while (r == shapes_batch::kRunRetry) { /* this handle alone, as shapes_batch_step would */
        b->enqueue(*cfg, nsteps, true);
        r = b->finish(*cfg, true);
      }
      b->residual_valid = r == SHAPES_OK && ((cfg->flags & SHAPES_FLAG_RESIDUAL) || b->learned_on(*cfg));
      if (r != SHAPES_OK && rc == SHAPES_OK) rc = r;
    }
    return rc;
  });
}

int shapes_batches_step_io(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, const shapes_bodies* in,
                           shapes_bodies* out) {
  if (!bs || n < 1 || !in || !out) return SHAPES_E_INVALID_ARG;
  for (int32_t k = 0; k < n; ++k) {
    if (!bs[k] || !body_arrays_ok(&in[k]) || !body_arrays_ok(&out[k])) return SHAPES_E_INVALID_ARG;
    for (int32_t j = 0; j < k; ++j)
      if (bs[j] == bs[k] || bs[j]->stream == bs[k]->stream) return SHAPES_E_INVALID_ARG;
  }
  const int rc0 = check_cfg(cfg);
  if (rc0 != SHAPES_OK) return rc0;
  return guarded([&]() -> int {
    for (int32_t k = 0; k < n; ++k) {
      shapes_batch* b = bs[k];
      ck(cudaSetDevice(b->device), "cudaSetDevice");
      b->prepare(*cfg, true);
      b->run_retries = 0;
      b->enqueue_begin(true); /* zeroes the counters and keeps the state a refusal returns to */
      b->io_upload(&in[k]);
      b->io_commit();
    }
    for (int32_t k = 0; k < n; ++k) bs[k]->enqueue_one(*cfg, true);
    for (int32_t k = 0; k < n; ++k) {
      bs[k]->io_download(&out[k]);
      bs[k]->enqueue_end();
    }
    int rc = SHAPES_OK;
    for (int32_t k = 0; k < n; ++k) {
      const int r = bs[k]->io_finish(*cfg, &out[k]);
      if (r != SHAPES_OK && rc == SHAPES_OK) rc = r;
    }
    return rc;
  });
}

static bool mapped_host10(double* const host[10], double* dev[10]);

int shapes_batches_run_io(shapes_batch* const* bs, int32_t n, const shapes_config* cfg, int32_t nsteps,
                          shapes_bodies* state, shapes_step_callback on_step, void* user) {
  if (!bs || n < 1 || nsteps < 0 || !state) return SHAPES_E_INVALID_ARG;
  for (int32_t k = 0; k < n; ++k) {
    if (!bs[k] || !body_arrays_ok(&state[k])) return SHAPES_E_INVALID_ARG;
    for (int32_t j = 0; j < k; ++j)
      if (bs[j] == bs[k] || bs[j]->stream == bs[k]->stream) return SHAPES_E_INVALID_ARG;
  }
  const int rc0 = check_cfg(cfg);
  if (rc0 != SHAPES_OK) return rc0;
  std::vector<int> status(n, SHAPES_OK);
  std::vector<std::string> detail(n);
  /* handle k's loop: its steps in order, one wait per step */
  auto lane = [&](int32_t k) {
    shapes_batch* b = bs[k];
    status[k] = guarded([&]() -> int {
      ck(cudaSetDevice(b->device), "cudaSetDevice");
      double* bp[10];
      body_ptrs(&state[k], bp);
      double* mapped[10];
      const bool is_mapped = mapped_host10(bp, mapped); /* resolved once for the whole run */
      double* const* mp = is_mapped ? mapped : nullptr;
      for (int32_t s = 0; s < nsteps; ++s) {
        b->prepare(*cfg, true);
        b->run_retries = 0;
        b->enqueue_begin(true);
        b->io_upload(&state[k], mp);
        b->io_commit();
        b->enqueue_one(*cfg, true);
        b->io_download(&state[k], mp, kStepFields); /* the other four arrays are the ones just uploaded */
        b->enqueue_end();
        const int r = b->io_finish(*cfg, &state[k], mp, kStepFields);
        if (r != SHAPES_OK) return r;
        if (on_step && on_step(user, k, s) != 0) break;
      }
      return SHAPES_OK;
    });
    detail[k] = g_last_error;
  };
  std::vector<std::thread> threads;
  try {
    for (int32_t k = 1; k < n; ++k) threads.emplace_back(lane, k);
  } catch (const std::system_error&) {
    for (auto& t : threads) t.join();
    g_last_error = "could not start a host thread";
    return SHAPES_E_CAPACITY;
  }
  lane(0);
  for (auto& t : threads) t.join();
  for (int32_t k = 0; k < n; ++k)
    if (status[k] != SHAPES_OK) {
      g_last_error = detail[k];
      return status[k];
    }
  g_last_error.clear();
  return SHAPES_OK;
}

int shapes_batch_collide(shapes_batch* b) {
  if (!b) return SHAPES_E_INVALID_ARG;
  shapes_config cfg{};
  cfg.dt = 1.0;
  return guarded([&]() -> int {
    ck(cudaSetDevice(b->device), "cudaSetDevice");
    return b->run(cfg, 1, false);
  });
}

/* Device addresses of ten caller arrays when every one is pinned host memory
 * mapped into the device address space (then one copy kernel moves them);
 * false for pageable memory, which goes through cudaMemcpyAsync. */
static bool mapped_host10(double* const host[10], double* dev[10]) {
  for (int k = 0; k < 10; ++k) {
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, host[k]) != cudaSuccess) {
      cudaGetLastError(); /* clear: an unknown pointer is simply not mapped */
      return false;
    }
    if (a.type != cudaMemoryTypeHost || !a.devicePointer) return false;
    dev[k] = static_cast<double*>(a.devicePointer);
  }
  return true;
}

static dim3 copy10_grid(int n, int fields = 10) {
  const int64_t per_block = 256 * shapes::kCopy10PerThread;
  return dim3((unsigned)std::max<int64_t>(1, std::min<int64_t>((n + per_block - 1) / per_block, 1024)),
              (unsigned)fields);
}

int shapes_batch::io_finish(const shapes_config& cfg, shapes_bodies* out, double* const* mapped_out, int fields) {
  ck(cudaStreamSynchronize(stream), "step");
  if (run_counters[shapes::kCntBadInput]) { /* refused: undo the step taken on the old state */
    cache_buf = run_saved_cache_buf;
    restore(run_saved_cap);
    pose(0, 0.0);
    ck(cudaStreamSynchronize(stream), "restore");
    have_results = false;
    return SHAPES_E_NAN;
  }
  int r = finish(cfg, true);
  while (r == kRunRetry) { /* grown and restored: the staged input again, alone */
    enqueue_begin(true);
    io_commit();
    enqueue_one(cfg, true);
    io_download(out, mapped_out, fields);
    enqueue_end();
    r = finish(cfg, true);
  }
  residual_valid = r == SHAPES_OK && ((cfg.flags & SHAPES_FLAG_RESIDUAL) || learned_on(cfg));
  return r;
}

void shapes_batch::io_upload(const shapes_bodies* in, double* const* mapped) {
  double* bp[10];
  body_ptrs(in, bp);
  double* dp[10];
  if (mapped || mapped_host10(bp, dp)) {
    if (mapped) std::copy(mapped, mapped + 10, dp);
    shapes::Ptr10 p{};
    for (int k = 0; k < 10; ++k) {
      p.src[k] = dp[k];
      p.dst[k] = body_stage[k];
    }
    shapes::k_copy10<<<copy10_grid(N), 256, 0, stream>>>(p, N, counters + shapes::kCntBadInput);
  } else {
    for (int k = 0; k < 10; ++k)
      ck(cudaMemcpyAsync(body_stage[k], bp[k], sizeof(double) * N, cudaMemcpyHostToDevice, stream), "upload");
    shapes::k_check_finite<<<grid_for(10LL * N, 256), 256, 0, stream>>>(
        body_stage[0], body_stage[1], body_stage[2], body_stage[3], body_stage[4], body_stage[5], body_stage[6],
        body_stage[7], body_stage[8], body_stage[9], N, counters + shapes::kCntBadInput);
  }
  ck(cudaGetLastError(), "launch");
}

void shapes_batch::io_download(shapes_bodies* out, double* const* mapped, int fields) {
  double* bp[10];
  body_ptrs(out, bp);
  double* dp[10];
  if (mapped || mapped_host10(bp, dp)) {
    if (mapped) std::copy(mapped, mapped + 10, dp);
    shapes::Ptr10 p{};
    for (int k = 0; k < 10; ++k) {
      p.src[k] = body[k];
      p.dst[k] = dp[k];
    }
    shapes::k_copy10<<<copy10_grid(N, fields), 256, 0, stream>>>(p, N, nullptr);
    ck(cudaGetLastError(), "launch");
  } else {
    for (int k = 0; k < fields; ++k)
      ck(cudaMemcpyAsync(bp[k], body[k], sizeof(double) * N, cudaMemcpyDeviceToHost, stream), "download");
  }
}

int shapes_batch_get_bodies(shapes_batch* b, shapes_bodies* out) {
  if (!b || !body_arrays_ok(out)) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    double* bp[10];
    body_ptrs(out, bp);
    double* dp[10];
    if (b->N > 0 && mapped_host10(bp, dp)) {
      shapes::Ptr10 p{};
      for (int k = 0; k < 10; ++k) {
        p.src[k] = b->body[k];
        p.dst[k] = dp[k];
      }
      shapes::k_copy10<<<copy10_grid(b->N), 256, 0, b->stream>>>(p, b->N, nullptr);
      ck(cudaGetLastError(), "launch");
    } else {
      for (int k = 0; k < 10; ++k)
        ck(cudaMemcpyAsync(bp[k], b->body[k], sizeof(double) * b->N, cudaMemcpyDeviceToHost, b->stream), "download");
    }
    ck(cudaStreamSynchronize(b->stream), "download");
    return SHAPES_OK;
  });
}

int shapes_batch_set_bodies(shapes_batch* b, const shapes_bodies* in) {
  if (!b || !body_arrays_ok(in)) return SHAPES_E_INVALID_ARG;
  double* bp[10];
  body_ptrs(in, bp);
  return guarded([&]() -> int {
    ck(cudaMemsetAsync(b->counters + shapes::kCntBadInput, 0, sizeof(unsigned long long), b->stream), "memset");
    double* dp[10];
    if (mapped_host10(bp, dp)) { /* copy and check in one pass over NVLink-C2C / PCIe */
      shapes::Ptr10 p{};
      for (int k = 0; k < 10; ++k) {
        p.src[k] = dp[k];
        p.dst[k] = b->body_stage[k];
      }
      shapes::k_copy10<<<copy10_grid(b->N), 256, 0, b->stream>>>(p, b->N, b->counters + shapes::kCntBadInput);
    } else {
      for (int k = 0; k < 10; ++k)
        ck(cudaMemcpyAsync(b->body_stage[k], bp[k], sizeof(double) * b->N, cudaMemcpyHostToDevice, b->stream),
           "upload");
      shapes::k_check_finite<<<grid_for(10LL * b->N, 256), 256, 0, b->stream>>>(
          b->body_stage[0], b->body_stage[1], b->body_stage[2], b->body_stage[3], b->body_stage[4],
          b->body_stage[5], b->body_stage[6], b->body_stage[7], b->body_stage[8], b->body_stage[9], b->N,
          b->counters + shapes::kCntBadInput);
    }
    ck(cudaGetLastError(), "launch");
    unsigned long long bad = 0;
    ck(cudaMemcpyAsync(&bad, b->counters + shapes::kCntBadInput, sizeof(bad), cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "validate");
    if (bad) return SHAPES_E_NAN; /* live state untouched */
    /* copied, not swapped: the live arrays keep their addresses, which the
     * captured step graphs hold */
    shapes::Ptr10 p{};
    for (int k = 0; k < 10; ++k) {
      p.src[k] = b->body_stage[k];
      p.dst[k] = b->body[k];
    }
    /* only bodies whose position, rotation or inverse masses changed get a
     * new pose: every other body's pose is already that of the state written
     * back (the live pose always follows the live state) */
    shapes::k_commit_bodies<<<grid_for(b->N, 256), 256, 0, b->stream>>>(p, b->N, b->body_changed);
    {
      Dev d = b->view(0);
      shapes::k_integrate_pose<<<grid_for(b->N, 128), 128, 0, b->stream>>>(d, 0.0, 0, b->body_changed);
    }
    ck(cudaGetLastError(), "launch");
    ck(cudaStreamSynchronize(b->stream), "upload");
    b->have_results = false;
    return SHAPES_OK;
  });
}

int shapes_batch_num_worlds(shapes_batch* b, int32_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->W;
  return SHAPES_OK;
}

int shapes_batch_num_bodies(shapes_batch* b, int64_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->N;
  return SHAPES_OK;
}

int shapes_batch_num_vertices(shapes_batch* b, int64_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->V;
  return SHAPES_OK;
}

int shapes_batch_get_shapes(shapes_batch* b, double* world_xy, double* normal_xy) {
  if (!b || !world_xy || !normal_xy) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    std::vector<double> x(b->V), y(b->V), nx(b->V), ny(b->V);
    ck(cudaMemcpyAsync(x.data(), b->wx, sizeof(double) * b->V, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaMemcpyAsync(y.data(), b->wy, sizeof(double) * b->V, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaMemcpyAsync(nx.data(), b->nx, sizeof(double) * b->V, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaMemcpyAsync(ny.data(), b->ny, sizeof(double) * b->V, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "download");
    for (int32_t v = 0; v < b->V; ++v) {
      world_xy[2 * (size_t)v] = x[v];
      world_xy[2 * (size_t)v + 1] = y[v];
      normal_xy[2 * (size_t)v] = nx[v];
      normal_xy[2 * (size_t)v + 1] = ny[v];
    }
    return SHAPES_OK;
  });
}

int shapes_batch_num_pairs(shapes_batch* b, int64_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->have_results ? b->stats.pairs : 0;
  return SHAPES_OK;
}

static void world_counts_from(shapes_batch* b, const int32_t* dev_off, int32_t* counts) {
  std::vector<int32_t> off(b->W + 1);
  ck(cudaMemcpyAsync(off.data(), dev_off, sizeof(int32_t) * (b->W + 1), cudaMemcpyDeviceToHost, b->stream), "download");
  ck(cudaStreamSynchronize(b->stream), "download");
  for (int w = 0; w < b->W; ++w) counts[w] = off[w + 1] - off[w];
}

int shapes_batch_get_pairs(shapes_batch* b, int32_t* ij, int64_t capacity, int32_t* world_counts) {
  if (!b || (!ij && capacity > 0)) return SHAPES_E_INVALID_ARG;
  const int64_t P = b->have_results ? b->stats.pairs : 0;
  if (capacity < P) return SHAPES_E_BUFFER;
  return guarded([&]() -> int {
    std::vector<int32_t> pa(P), pb(P);
    if (P > 0) {
      ck(cudaMemcpyAsync(pa.data(), b->pair_a, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaMemcpyAsync(pb.data(), b->pair_b, sizeof(int32_t) * P, cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    for (int64_t p = 0; p < P; ++p) {
      const int32_t off = b->h_world_body_off[b->h_body_world[pa[p]]];
      ij[2 * p] = pa[p] - off;
      ij[2 * p + 1] = pb[p] - off;
    }
    if (world_counts) {
      if (b->have_results) world_counts_from(b, b->world_pair_off, world_counts);
      else std::fill(world_counts, world_counts + b->W, 0);
    }
    return SHAPES_OK;
  });
}

int shapes_batch_num_contacts(shapes_batch* b, int64_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->have_results ? b->stats.contacts : 0;
  return SHAPES_OK;
}

static void decode_key(uint64_t k, int32_t* out4) {
  out4[0] = (int32_t)(k >> 44);
  out4[1] = (int32_t)((k >> 24) & 0xfffff);
  out4[2] = (int32_t)((k >> 12) & 0xfff);
  out4[3] = (int32_t)(k & 0xfff);
}

int shapes_batch_get_contacts(shapes_batch* b, int32_t* keys5, double* vals5, int64_t capacity,
                              int32_t* world_counts) {
  if (!b || ((!keys5 || !vals5) && capacity > 0)) return SHAPES_E_INVALID_ARG;
  const int64_t C = b->have_results ? b->stats.contacts : 0;
  if (capacity < C) return SHAPES_E_BUFFER;
  return guarded([&]() -> int {
    if (C > 0) {
      /* decoded on the device; straight into the caller's arrays when both
       * are mapped pinned host memory, else through a device staging area */
      cudaPointerAttributes ak{}, av{};
      const bool mk = cudaPointerGetAttributes(&ak, keys5) == cudaSuccess && ak.type == cudaMemoryTypeHost &&
                      ak.devicePointer;
      const bool mv = cudaPointerGetAttributes(&av, vals5) == cudaSuccess && av.type == cudaMemoryTypeHost &&
                      av.devicePointer;
      cudaGetLastError();
      const int grid = (int)std::min<int64_t>((C + 255) / 256, 4096);
      if (mk && mv) {
        shapes::k_export_contacts<<<grid, 256, 0, b->stream>>>(
            b->c_key[b->results_buf], b->c_flip, b->c_val, (int)C, static_cast<int32_t*>(ak.devicePointer),
            static_cast<double*>(av.devicePointer));
        ck(cudaGetLastError(), "launch");
      } else {
        if (b->export_cap < C) {
          dfree(b->export_keys);
          dfree(b->export_vals);
          b->export_keys = nullptr;
          b->export_vals = nullptr;
          b->export_keys = dalloc<int32_t>(5 * (size_t)C, "cudaMalloc export");
          b->export_vals = dalloc<double>(5 * (size_t)C, "cudaMalloc export");
          b->export_cap = C;
        }
        shapes::k_export_contacts<<<grid, 256, 0, b->stream>>>(b->c_key[b->results_buf], b->c_flip, b->c_val,
                                                              (int)C, b->export_keys, b->export_vals);
        ck(cudaGetLastError(), "launch");
        ck(cudaMemcpyAsync(keys5, b->export_keys, sizeof(int32_t) * 5 * C, cudaMemcpyDeviceToHost, b->stream),
           "download");
        ck(cudaMemcpyAsync(vals5, b->export_vals, sizeof(double) * 5 * C, cudaMemcpyDeviceToHost, b->stream),
           "download");
      }
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    if (world_counts) {
      if (b->have_results) world_counts_from(b, b->cwo[b->results_buf], world_counts);
      else std::fill(world_counts, world_counts + b->W, 0);
    }
    return SHAPES_OK;
  });
}

int shapes_batch_num_cache(shapes_batch* b, int64_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    int32_t total = 0;
    ck(cudaMemcpyAsync(&total, b->cwo[b->cache_buf] + b->W, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "download");
    *out = total;
    return SHAPES_OK;
  });
}

int shapes_batch_get_cache(shapes_batch* b, int32_t* keys4, double* lam2, int64_t capacity, int32_t* world_counts) {
  if (!b) return SHAPES_E_INVALID_ARG;
  int64_t n = 0;
  int rc = shapes_batch_num_cache(b, &n);
  if (rc != SHAPES_OK) return rc;
  if (capacity < n) return SHAPES_E_BUFFER;
  if (n > 0 && (!keys4 || !lam2)) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    std::vector<uint64_t> key(n);
    if (n > 0) {
      ck(cudaMemcpyAsync(key.data(), b->c_key[b->cache_buf], sizeof(uint64_t) * n, cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaMemcpyAsync(lam2, b->lam[b->cache_buf], sizeof(double) * 2 * n, cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    for (int64_t c = 0; c < n; ++c) decode_key(key[c], keys4 + 4 * c);
    if (world_counts) world_counts_from(b, b->cwo[b->cache_buf], world_counts);
    return SHAPES_OK;
  });
}

int shapes_batch_set_cache(shapes_batch* b, const int32_t* world_counts, const int32_t* keys4, const double* lam2) {
  if (!b || !world_counts) return SHAPES_E_INVALID_ARG;
  std::vector<int32_t> off(b->W + 1, 0);
  for (int w = 0; w < b->W; ++w) {
    if (world_counts[w] < 0) return SHAPES_E_INVALID_ARG;
    off[w + 1] = off[w] + world_counts[w];
  }
  const int64_t n = off[b->W];
  if (n > 0 && (!keys4 || !lam2)) return SHAPES_E_INVALID_ARG;
  std::vector<uint64_t> key(n);
  for (int w = 0; w < b->W; ++w) {
    const int32_t nw = b->h_world_body_off[w + 1] - b->h_world_body_off[w];
    for (int32_t c = off[w]; c < off[w + 1]; ++c) {
      const int32_t* k = keys4 + 4 * (size_t)c;
      if (k[0] < 0 || k[0] >= nw || k[1] < 0 || k[1] >= nw || k[2] < 0 || k[2] >= 4096 || k[3] < 0 || k[3] >= 4096)
        return SHAPES_E_INVALID_ARG;
      key[c] = ((uint64_t)k[0] << 44) | ((uint64_t)k[1] << 24) | ((uint64_t)k[2] << 12) | (uint64_t)k[3];
      if (c > off[w] && !(key[c] < key[c - 1])) return SHAPES_E_INVALID_ARG;
    }
  }
  return guarded([&]() -> int {
    if (n > b->contact_cap) {
      const int64_t nc = std::max<int64_t>(n, 2LL * b->contact_cap);
      if (nc > INT32_MAX / 2) return SHAPES_E_CAPACITY;
      b->alloc_step_buffers(std::max<int32_t>(b->pair_cap, (int32_t)(nc / 2)), (int32_t)nc, 8);
    }
    if (n > 0) {
      ck(cudaMemcpyAsync(b->c_key[b->cache_buf], key.data(), sizeof(uint64_t) * n, cudaMemcpyHostToDevice, b->stream), "upload");
      ck(cudaMemcpyAsync(b->lam[b->cache_buf], lam2, sizeof(double) * 2 * n, cudaMemcpyHostToDevice, b->stream), "upload");
    }
    ck(cudaMemcpyAsync(b->cwo[b->cache_buf], off.data(), sizeof(int32_t) * (b->W + 1), cudaMemcpyHostToDevice, b->stream), "upload");
    ck(cudaStreamSynchronize(b->stream), "upload");
    return SHAPES_OK;
  });
}

int shapes_batch_get_world_metrics(shapes_batch* b, double* residual, double* max_depth) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    if (residual) {
      if (b->residual_valid)
        ck(cudaMemcpy(residual, b->world_residual, sizeof(double) * b->W, cudaMemcpyDeviceToHost), "download");
      else
        std::fill(residual, residual + b->W, std::nan(""));
    }
    if (max_depth) {
      shapes_config cfg{};
      cfg.dt = 1.0;
      const shapes_stats keep = b->stats; /* the counters stay those of the last step call */
      const int rc = b->run(cfg, 1, false);
      b->stats = keep;
      if (rc != SHAPES_OK) return rc;
      Dev d = b->view(b->results_buf);
      b->world_metric_kernels(d, false);
      ck(cudaGetLastError(), "launch");
      ck(cudaMemcpyAsync(max_depth, b->world_depth, sizeof(double) * b->W, cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    return SHAPES_OK;
  });
}

int shapes_batch_get_stats(shapes_batch* b, shapes_stats* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  *out = b->stats;
  return SHAPES_OK;
}

int shapes_batch_autotune(shapes_batch* b, const shapes_config* cfg, int32_t steps_per_trial,
                          int32_t* chosen_worlds_per_group, int32_t* chosen_threads) {
  if (!b || steps_per_trial < 1) return SHAPES_E_INVALID_ARG;
  const int rc0 = check_cfg(cfg);
  if (rc0 != SHAPES_OK) return rc0;
  return guarded([&]() -> int {
    const int N = b->N, W = b->W;
    /* save the state the trials start from */
    int32_t n_cache = 0;
    ck(cudaMemcpyAsync(&n_cache, b->cwo[b->cache_buf] + W, sizeof(int32_t), cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "sync");
    std::vector<void*> saved;
    auto keep = [&](const void* src, size_t bytes) {
      void* p = nullptr;
      ck(cudaMalloc(&p, std::max<size_t>(bytes, 1)), "cudaMalloc autotune");
      saved.push_back(p);
      ck(cudaMemcpyAsync(p, src, bytes, cudaMemcpyDeviceToDevice, b->stream), "copy");
      return p;
    };
    const int cache_buf0 = b->cache_buf;
    void* sb[6];
    for (int k = 0; k < 6; ++k) sb[k] = keep(b->body[k], sizeof(double) * N);
    void* skey = keep(b->c_key[cache_buf0], sizeof(uint64_t) * n_cache);
    void* slam = keep(b->lam[cache_buf0], sizeof(double) * 2 * n_cache);
    void* scwo = keep(b->cwo[cache_buf0], sizeof(int32_t) * (W + 1));
    const int32_t wpg0 = b->worlds_per_group_override, thr0 = b->solve_threads, tgt0 = b->target_group_bodies;
    const int32_t gw0 = b->group_warps;
    const std::vector<int32_t> order0 = b->world_order;
    const bool prof0 = b->profiling;
    b->profiling = false;
    auto restore_state = [&]() {
      b->cache_buf = cache_buf0;
      for (int k = 0; k < 6; ++k)
        ck(cudaMemcpyAsync(b->body[k], sb[k], sizeof(double) * N, cudaMemcpyDeviceToDevice, b->stream), "copy");
      if (n_cache > b->contact_cap) throw CudaError{cudaErrorMemoryAllocation};
      ck(cudaMemcpyAsync(b->c_key[cache_buf0], skey, sizeof(uint64_t) * n_cache, cudaMemcpyDeviceToDevice, b->stream), "copy");
      ck(cudaMemcpyAsync(b->lam[cache_buf0], slam, sizeof(double) * 2 * n_cache, cudaMemcpyDeviceToDevice, b->stream), "copy");
      ck(cudaMemcpyAsync(b->cwo[cache_buf0], scwo, sizeof(int32_t) * (W + 1), cudaMemcpyDeviceToDevice, b->stream), "copy");
      b->pose(0, 0.0);
    };
    const int base = std::max(1, std::min(shapes::kMaxGroupWorlds, 32 / (cfg->iterations + 1)));
    /* The level-ordered packing: worlds sorted by the dependency levels of
     * one step from the saved state (deepest first, then by size), so that a
     * group's worlds end their levels together. */
    restore_state();
    b->world_order.clear();
    b->make_groups(cfg->iterations);
    const int rc0 = b->run(*cfg, 1, true);
    std::vector<int32_t> lv(W, 0), by_levels(W);
    if (rc0 == SHAPES_OK)
      ck(cudaMemcpy(lv.data(), b->world_levels, sizeof(int32_t) * W, cudaMemcpyDeviceToHost), "download");
    for (int w = 0; w < W; ++w) by_levels[w] = w;
    std::stable_sort(by_levels.begin(), by_levels.end(), [&](int a, int c) {
      if (lv[a] != lv[c]) return lv[a] > lv[c];
      return (b->h_world_body_off[a + 1] - b->h_world_body_off[a]) > (b->h_world_body_off[c + 1] - b->h_world_body_off[c]);
    });
    /* (worlds per group, threads per CTA, warps per group, level order,
     * parallel levels, heavy groups spread, target bodies per group: when
     * non-zero, groups close at that many bodies instead of at a world
     * count, so the largest worlds of a ragged batch get groups of their own) */
    std::vector<std::array<int, 7>> cands;
    auto add = [&](int wpg, int thr, int gw, int lo, int par, int spread = 0, int target = 0) {
      const std::array<int, 7> c{wpg, thr, gw, lo, par, spread, target};
      if (wpg >= 1 && wpg <= shapes::kMaxGroupWorlds && std::find(cands.begin(), cands.end(), c) == cands.end())
        cands.push_back(c);
    };
    for (int lo : {0, 1}) {
      for (int wpg : {1, base / 2, base, base + 1, 2 * base})
        for (int thr : {32, 64, 128}) add(std::min(wpg, W), thr, 1, lo, 0);
      for (int wpg : {1, 2, base, base + 1, 2 * base, 3 * base, 4 * base})
        for (int gw : {2, 4, 8})
          for (int par : {0, 1}) {
            add(std::min(wpg, W), 32 * gw, gw, lo, par);
            if (par) add(std::min(wpg, W), 32 * gw, gw, lo, par, 1);
          }
    }
    int32_t min_n = INT32_MAX, max_n = 0;
    for (int w = 0; w < W; ++w) {
      const int32_t n = b->h_world_body_off[w + 1] - b->h_world_body_off[w];
      if (n >= b->large_world_bodies) continue;
      min_n = std::min(min_n, n);
      max_n = std::max(max_n, n);
    }
    if (max_n > 2 * min_n) /* ragged batches: packings by body count */
      for (int target : {256, 512, 1024, 2048})
        for (int gw : {2, 4, 8})
          for (int par : {0, 1}) add(1, 32 * gw, gw, 0, par, 1, target);
    cudaEvent_t e0, e1;
    ck(cudaEventCreate(&e0), "event");
    ck(cudaEventCreate(&e1), "event");
    float best = 1e30f;
    const bool par0 = b->parallel_levels, spread0 = b->spread_heavy;
    std::array<int, 7> best_c{wpg0, thr0, gw0, -1, par0 ? 1 : 0, spread0 ? 1 : 0, tgt0};
    int rc = rc0;
    if (rc0 != SHAPES_OK) cands.clear();
    for (const auto& c : cands) {
      restore_state();
      b->worlds_per_group_override = c[6] ? 0 : c[0];
      b->target_group_bodies = c[6];
      b->solve_threads = c[1];
      b->group_warps = c[2];
      b->parallel_levels = c[4] != 0;
      b->spread_heavy = c[5] != 0;
      b->invalidate_graphs();
      if (c[3]) b->world_order = by_levels; else b->world_order.clear();
      b->make_groups(cfg->iterations);
      rc = b->run(*cfg, 1, true); /* untimed: captures this packing's step graphs */
      if (rc != SHAPES_OK) break;
      ck(cudaEventRecord(e0, b->stream), "event");
      rc = b->run(*cfg, steps_per_trial, true);
      if (rc != SHAPES_OK) break;
      ck(cudaEventRecord(e1, b->stream), "event");
      ck(cudaEventSynchronize(e1), "event");
      float ms = 0.f;
      ck(cudaEventElapsedTime(&ms, e0, e1), "event");
      if (ms < best) {
        best = ms;
        best_c = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    restore_state();
    if (rc == SHAPES_OK && best_c[3] >= 0) {
      b->worlds_per_group_override = best_c[6] ? 0 : best_c[0];
      b->target_group_bodies = best_c[6];
      b->solve_threads = best_c[1];
      b->group_warps = best_c[2];
      b->parallel_levels = best_c[4] != 0;
      b->spread_heavy = best_c[5] != 0;
      if (best_c[3]) b->world_order = by_levels; else b->world_order.clear();
    } else {
      b->worlds_per_group_override = wpg0;
      b->target_group_bodies = tgt0;
      b->solve_threads = thr0;
      b->group_warps = gw0;
      b->parallel_levels = par0;
      b->spread_heavy = spread0;
      b->world_order = order0;
    }
    b->invalidate_graphs();
    b->make_groups(cfg->iterations);
    ck(cudaStreamSynchronize(b->stream), "sync");
    for (void* p : saved) cudaFree(p);
    b->profiling = prof0;
    b->have_results = false;
    if (chosen_worlds_per_group) *chosen_worlds_per_group = b->worlds_per_group_override;
    if (chosen_threads) *chosen_threads = b->solve_threads;
    return rc;
  });
}

/* ---- world mutation (World.append / World.delete) ------------------------ */

int shapes_batch_delete_body(shapes_batch* b, int32_t world, int32_t slot) {
  if (!b || world < 0 || world >= b->W) return SHAPES_E_INVALID_ARG;
  const int32_t n = b->h_world_body_off[world + 1] - b->h_world_body_off[world];
  if (slot < 0 || slot >= n) return SHAPES_E_INVALID_ARG;
  const int32_t g = b->h_world_body_off[world] + slot;
  if (!b->h_active[g]) return SHAPES_E_INVALID_ARG; /* safeDelete: the slot must be filled */
  return guarded([&]() -> int {
    b->h_active[g] = 0;
    b->h_empties[world].push_back(slot);
    b->upload_active();
    return SHAPES_OK;
  });
}

int shapes_batch_append_body(shapes_batch* b, int32_t world, const double* body10, int32_t n_verts,
                             const double* local_verts_xy, int32_t* slot_out) {
  if (!b || !body10 || !local_verts_xy || !slot_out || world < 0 || world >= b->W) return SHAPES_E_INVALID_ARG;
  for (int k = 0; k < 10; ++k)
    if (!std::isfinite(body10[k])) return SHAPES_E_NAN;
  const int hrc = check_shape(n_verts == 1 ? SHAPES_SHAPE_CIRCLE : SHAPES_SHAPE_HULL, n_verts, local_verts_xy);
  if (hrc != SHAPES_OK) return hrc;
  return guarded([&]() -> int {
    const int32_t W = b->W, N = b->N;
    const int32_t w0 = b->h_world_body_off[world];
    auto& empties = b->h_empties[world];
    const bool reuse = !empties.empty();
    const int32_t slot = reuse ? empties.back() : b->h_world_body_off[world + 1] - w0;
    if (slot >= (1 << 20)) return SHAPES_E_CAPACITY;
    if (reuse) {
      const int32_t g = w0 + slot;
      const int32_t v0 = b->h_vert_off[g];
      if (b->h_vert_off[g + 1] - v0 == n_verts) { /* same vertex count: in place */
        ck(cudaStreamSynchronize(b->stream), "sync");
        for (int k = 0; k < 10; ++k)
          ck(cudaMemcpyAsync(b->body[k] + g, body10 + k, sizeof(double), cudaMemcpyHostToDevice, b->stream), "upload");
        std::vector<double> xs(n_verts), ys(n_verts);
        for (int32_t v = 0; v < n_verts; ++v) {
          xs[v] = local_verts_xy[2 * v];
          ys[v] = local_verts_xy[2 * v + 1];
        }
        if (n_verts == 1) { /* a circle into a circle's slot */
          b->h_radius[g] = xs[0];
          xs[0] = ys[0] = 0.0;
          ck(cudaMemcpyAsync(b->radius + g, &b->h_radius[g], sizeof(double), cudaMemcpyHostToDevice, b->stream),
             "upload");
        }
        ck(cudaMemcpyAsync(b->lx + v0, xs.data(), sizeof(double) * n_verts, cudaMemcpyHostToDevice, b->stream), "upload");
        ck(cudaMemcpyAsync(b->ly + v0, ys.data(), sizeof(double) * n_verts, cudaMemcpyHostToDevice, b->stream), "upload");
        Dev d = b->view(0);
        shapes::k_init_extents<<<grid_for(b->V, 128), 128, 0, b->stream>>>(d);
        ck(cudaGetLastError(), "launch");
        empties.pop_back();
        b->h_active[g] = 1;
        b->upload_active();
        if (!b->active) { /* every slot filled again: the in-place shape still needs its pose */
          b->pose(0, 0.0);
          ck(cudaStreamSynchronize(b->stream), "upload");
        }
        *slot_out = slot;
        return SHAPES_OK;
      }
    }
    /* the topology changes: rebuild from the host copies, keeping state and cache */
    std::vector<double> body(10 * (size_t)N);
    shapes_bodies cur{};
    double* bp[10];
    for (int k = 0; k < 10; ++k) bp[k] = body.data() + (size_t)k * N;
    cur.vel_x = bp[0]; cur.vel_y = bp[1]; cur.rot_vel = bp[2]; cur.pos_x = bp[3]; cur.pos_y = bp[4];
    cur.rot = bp[5]; cur.inv_mass_lin = bp[6]; cur.inv_mass_rot = bp[7]; cur.mu = bp[8]; cur.bounce = bp[9];
    int rc = shapes_batch_get_bodies(b, &cur);
    if (rc != SHAPES_OK) return rc;
    int64_t nc = 0;
    rc = shapes_batch_num_cache(b, &nc);
    if (rc != SHAPES_OK) return rc;
    std::vector<int32_t> keys(4 * (size_t)std::max<int64_t>(nc, 1)), wc(W);
    std::vector<double> lam(2 * (size_t)std::max<int64_t>(nc, 1));
    rc = shapes_batch_get_cache(b, keys.data(), lam.data(), nc, wc.data());
    if (rc != SHAPES_OK) return rc;
    const int64_t V = b->V;
    const std::vector<double> xyh = b->local_xy_host();
    const int32_t g = w0 + slot; /* replaced or inserted body */
    const int32_t N2 = reuse ? N : N + 1;
    std::vector<int32_t> off(W + 1);
    for (int w = 0; w <= W; ++w) off[w] = b->h_world_body_off[w] + ((!reuse && w > world) ? 1 : 0);
    std::vector<double> body2(10 * (size_t)N2);
    std::vector<uint8_t> act2(N2);
    std::vector<int32_t> vo2(N2 + 1, 0);
    std::vector<double> xy2;
    xy2.reserve(2 * (size_t)(V + n_verts));
    for (int32_t i = 0; i < N2; ++i) {
      const bool is_new = i == g;
      const int32_t src = (!reuse && i > g) ? i - 1 : i; /* old index */
      for (int k = 0; k < 10; ++k) body2[(size_t)k * N2 + i] = is_new ? body10[k] : body[(size_t)k * N + src];
      act2[i] = is_new ? 1 : b->h_active[src];
      if (is_new) {
        for (int32_t v = 0; v < 2 * n_verts; ++v) xy2.push_back(local_verts_xy[v]);
        vo2[i + 1] = vo2[i] + n_verts;
      } else {
        for (int32_t v = b->h_vert_off[src]; v < b->h_vert_off[src + 1]; ++v) {
          xy2.push_back(xyh[2 * (size_t)v]);
          xy2.push_back(xyh[2 * (size_t)v + 1]);
        }
        vo2[i + 1] = vo2[i] + (b->h_vert_off[src + 1] - b->h_vert_off[src]);
      }
    }
    double* bp2[10];
    for (int k = 0; k < 10; ++k) bp2[k] = body2.data() + (size_t)k * N2;
    b->init_topology(off.data(), bp2, vo2.data(), xy2.data());
    if (reuse) empties.pop_back();
    b->h_active = act2;
    b->upload_active();
    rc = shapes_batch_set_cache(b, wc.data(), keys.data(), lam.data());
    if (rc != SHAPES_OK) return rc;
    *slot_out = slot;
    return SHAPES_OK;
  });
}

int shapes_batch_get_active(shapes_batch* b, uint8_t* out) {
  if (!b || !out) return SHAPES_E_INVALID_ARG;
  std::copy(b->h_active.begin(), b->h_active.end(), out);
  return SHAPES_OK;
}

/* ---- checkpoint file (EngineState: World + EngineCache) ------------------ */

}  // extern "C"

namespace {

constexpr char kCkMagic[8] = {'S', 'H', 'A', 'P', 'E', 'S', 'C', 'K'};
constexpr uint32_t kCkVersion = 1;
constexpr uint32_t kCkEndian = 0x01020304u;

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 0xcbf29ce484222325ull) {
  for (size_t k = 0; k < n; ++k) {
    h ^= p[k];
    h *= 0x100000001b3ull;
  }
  return h;
}

struct CkWriter {
  std::vector<unsigned char> buf;
  template <class T>
  void put(const T* p, size_t n) {
    const unsigned char* c = reinterpret_cast<const unsigned char*>(p);
    buf.insert(buf.end(), c, c + sizeof(T) * n);
  }
  template <class T>
  void put1(T v) { put(&v, 1); }
};

struct CkReader {
  const std::vector<unsigned char>& buf;
  size_t at = 0;
  bool ok = true;
  template <class T>
  void get(T* p, size_t n) {
    const size_t bytes = sizeof(T) * n;
    if (!ok || buf.size() - at < bytes) {
      ok = false;
      return;
    }
    std::memcpy(p, buf.data() + at, bytes);
    at += bytes;
  }
  template <class T>
  T get1() {
    T v{};
    get(&v, 1);
    return v;
  }
};

}  // namespace

extern "C" {

int shapes_batch_save(shapes_batch* b, const char* path) {
  if (!b || !path) return SHAPES_E_INVALID_ARG;
  const int32_t W = b->W, N = b->N;
  const int64_t V = b->V;
  std::vector<double> body(10 * (size_t)N);
  shapes_bodies out{};
  double* bp[10];
  for (int k = 0; k < 10; ++k) bp[k] = body.data() + (size_t)k * N;
  out.vel_x = bp[0]; out.vel_y = bp[1]; out.rot_vel = bp[2]; out.pos_x = bp[3]; out.pos_y = bp[4];
  out.rot = bp[5]; out.inv_mass_lin = bp[6]; out.inv_mass_rot = bp[7]; out.mu = bp[8]; out.bounce = bp[9];
  int rc = shapes_batch_get_bodies(b, &out);
  if (rc != SHAPES_OK) return rc;
  int64_t nc = 0;
  rc = shapes_batch_num_cache(b, &nc);
  if (rc != SHAPES_OK) return rc;
  std::vector<int32_t> keys(4 * (size_t)std::max<int64_t>(nc, 1)), wc(W);
  std::vector<double> lam(2 * (size_t)std::max<int64_t>(nc, 1));
  rc = shapes_batch_get_cache(b, keys.data(), lam.data(), nc, wc.data());
  if (rc != SHAPES_OK) return rc;
  const std::vector<int32_t>& vo = b->h_vert_off;
  std::vector<double> xy;
  rc = guarded([&]() -> int {
    xy = b->local_xy_host();
    return SHAPES_OK;
  });
  if (rc != SHAPES_OK) return rc;
  CkWriter w;
  w.put(kCkMagic, 8);
  w.put1(kCkVersion);
  w.put1(kCkEndian);
  w.put1(W);
  w.put1(N);
  w.put1(V);
  w.put1(nc);
  w.put(b->h_world_body_off.data(), (size_t)W + 1);
  w.put(vo.data(), (size_t)N + 1);
  w.put(xy.data(), 2 * (size_t)V);
  w.put(body.data(), body.size());
  w.put(wc.data(), (size_t)W);
  w.put(keys.data(), 4 * (size_t)nc);
  w.put(lam.data(), 2 * (size_t)nc);
  w.put(b->h_active.data(), (size_t)N);
  for (int32_t k = 0; k < W; ++k) w.put1((int32_t)b->h_empties[k].size());
  for (int32_t k = 0; k < W; ++k) w.put(b->h_empties[k].data(), b->h_empties[k].size());
  w.put1(fnv1a(w.buf.data(), w.buf.size()));
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) {
    g_last_error = "cannot open " + tmp;
    return SHAPES_E_INVALID_ARG;
  }
  const bool wrote = std::fwrite(w.buf.data(), 1, w.buf.size(), f) == w.buf.size();
  const bool closed = std::fclose(f) == 0;
  if (!wrote || !closed || std::rename(tmp.c_str(), path) != 0) {
    std::remove(tmp.c_str());
    g_last_error = std::string("cannot write ") + path;
    return SHAPES_E_INVALID_ARG;
  }
  return SHAPES_OK;
}

int shapes_batch_load(const char* path, shapes_batch** out) {
  if (!path || !out) return SHAPES_E_INVALID_ARG;
  *out = nullptr;
  std::vector<unsigned char> buf;
  {
    FILE* f = std::fopen(path, "rb");
    if (!f) {
      g_last_error = std::string("cannot open ") + path;
      return SHAPES_E_INVALID_ARG;
    }
    unsigned char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + got);
    std::fclose(f);
  }
  auto bad = [&](const char* why) {
    g_last_error = std::string("checkpoint ") + path + ": " + why;
    return SHAPES_E_INVALID_ARG;
  };
  if (buf.size() < 40 + sizeof(uint64_t)) return bad("too short"); /* 40-byte header + hash */
  uint64_t sum = 0;
  std::memcpy(&sum, buf.data() + buf.size() - sizeof(uint64_t), sizeof sum);
  if (fnv1a(buf.data(), buf.size() - sizeof(uint64_t)) != sum) return bad("checksum mismatch");
  CkReader r{buf};
  char magic[8];
  r.get(magic, 8);
  if (std::memcmp(magic, kCkMagic, 8) != 0) return bad("not a shapes checkpoint");
  if (r.get1<uint32_t>() != kCkVersion) return bad("unsupported version");
  if (r.get1<uint32_t>() != kCkEndian) return bad("byte order differs");
  const int32_t W = r.get1<int32_t>(), N = r.get1<int32_t>();
  const int64_t V = r.get1<int64_t>(), nc = r.get1<int64_t>();
  if (!r.ok || W < 1 || N < 1 || V < 1 || nc < 0 || V > (int64_t)INT32_MAX || nc > (int64_t)INT32_MAX)
    return bad("bad sizes");
  const uint64_t need = 40ull + 4ull * (W + 1) + 4ull * (N + 1) + 16ull * V + 80ull * N + 4ull * W + 16ull * nc +
                        16ull * nc + 1ull * N + 4ull * W + 8ull; /* + the empty-slot stacks */
  if (buf.size() < need) return bad("size does not match the header");
  std::vector<int32_t> off(W + 1), vo(N + 1), wc(W), keys(4 * (size_t)std::max<int64_t>(nc, 1));
  std::vector<double> xy(2 * (size_t)V), body(10 * (size_t)N), lam(2 * (size_t)std::max<int64_t>(nc, 1));
  r.get(off.data(), off.size());
  r.get(vo.data(), vo.size());
  r.get(xy.data(), xy.size());
  r.get(body.data(), body.size());
  r.get(wc.data(), wc.size());
  r.get(keys.data(), 4 * (size_t)nc);
  r.get(lam.data(), 2 * (size_t)nc);
  std::vector<uint8_t> act(N);
  r.get(act.data(), act.size());
  std::vector<int32_t> elen(W);
  r.get(elen.data(), elen.size());
  std::vector<std::vector<int32_t>> empties(W);
  uint64_t total_empty = 0;
  for (int32_t k = 0; k < W && r.ok; ++k) {
    const int32_t nw = off[k + 1] - off[k];
    if (elen[k] < 0 || elen[k] > nw) return bad("bad empty-slot stack");
    total_empty += (uint64_t)elen[k];
    empties[k].resize(elen[k]);
    r.get(empties[k].data(), empties[k].size());
    for (int32_t e : empties[k])
      if (e < 0 || e >= nw || act[off[k] + e]) return bad("bad empty-slot stack");
  }
  if (!r.ok || buf.size() != need + 4ull * total_empty) return bad("size does not match the header");
  shapes_bodies in{};
  double* bp[10];
  for (int k = 0; k < 10; ++k) bp[k] = body.data() + (size_t)k * N;
  in.vel_x = bp[0]; in.vel_y = bp[1]; in.rot_vel = bp[2]; in.pos_x = bp[3]; in.pos_y = bp[4];
  in.rot = bp[5]; in.inv_mass_lin = bp[6]; in.inv_mass_rot = bp[7]; in.mu = bp[8]; in.bounce = bp[9];
  if (vo[0] != 0 || vo[N] != V) return bad("bad vertex offsets");
  std::vector<uint8_t> kind(N);
  for (int32_t i = 0; i < N && r.ok; ++i) {
    if (vo[i + 1] < vo[i] || vo[i + 1] > V) return bad("bad vertex offsets");
    kind[i] = vo[i + 1] - vo[i] == 1 ? SHAPES_SHAPE_CIRCLE : SHAPES_SHAPE_HULL;
  }
  shapes_batch* h = nullptr;
  int rc = shapes_batch_create(W, off.data(), &in, vo.data(), xy.data(), kind.data(), &h);
  if (rc != SHAPES_OK) return rc;
  rc = shapes_batch_set_cache(h, wc.data(), keys.data(), lam.data());
  if (rc == SHAPES_OK)
    rc = guarded([&]() -> int {
      for (int32_t i = 0; i < N; ++i) h->h_active[i] = act[i] ? 1 : 0;
      h->h_empties = empties;
      h->upload_active();
      return SHAPES_OK;
    });
  if (rc != SHAPES_OK) {
    shapes_batch_destroy(h);
    return rc;
  }
  *out = h;
  return SHAPES_OK;
}

int shapes_batch_set_graphs(shapes_batch* b, int32_t enabled) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->graphs_enabled = enabled != 0;
    b->drop_graphs();
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_set_mlp(shapes_batch* b, const shapes_mlp* m) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    if (m && !b->learned_mask) {
      b->learned_mask = dalloc<uint8_t>(b->W, "cudaMalloc");
      b->snap_mask = dalloc<uint8_t>(b->W, "cudaMalloc");
    }
    if (m) ck(cudaMemsetAsync(b->learned_mask, 1, b->W, b->stream), "memset");
    if (m) ck(mlp::prepare_device(), "network set-up");
    b->mlp_model = m;
    b->invalidate_graphs();
    ck(cudaStreamSynchronize(b->stream), "sync");
    return SHAPES_OK;
  });
}

int shapes_batch_get_learned_mask(shapes_batch* b, uint8_t* mask) {
  if (!b || !mask) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    if (!b->learned_mask) {
      std::fill(mask, mask + b->W, (uint8_t)0);
      return SHAPES_OK;
    }
    ck(cudaMemcpyAsync(mask, b->learned_mask, b->W, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "download");
    return SHAPES_OK;
  });
}

int shapes_batch_set_learned_mask(shapes_batch* b, const uint8_t* mask) {
  if (!b || !mask || !b->learned_mask) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    std::vector<uint8_t> m(b->W);
    for (int32_t w = 0; w < b->W; ++w) m[w] = mask[w] ? 1 : 0;
    ck(cudaMemcpyAsync(b->learned_mask, m.data(), b->W, cudaMemcpyHostToDevice, b->stream), "upload");
    ck(cudaStreamSynchronize(b->stream), "upload");
    return SHAPES_OK;
  });
}

int shapes_batch_set_judge(shapes_batch* b, const double* max_residual, const double* max_depth) {
  if (!b) return SHAPES_E_INVALID_ARG;
  for (int32_t w = 0; w < b->W; ++w)
    if ((max_residual && std::isnan(max_residual[w])) || (max_depth && std::isnan(max_depth[w])))
      return SHAPES_E_NAN;
  return guarded([&]() -> int {
    if (!b->judge_res) {
      b->judge_res = dalloc<double>(b->W, "cudaMalloc");
      b->judge_depth = dalloc<double>(b->W, "cudaMalloc");
    }
    const double inf = std::numeric_limits<double>::infinity();
    std::vector<double> r(b->W, inf), dd(b->W, inf);
    if (max_residual) std::copy(max_residual, max_residual + b->W, r.begin());
    if (max_depth) std::copy(max_depth, max_depth + b->W, dd.begin());
    ck(cudaMemcpyAsync(b->judge_res, r.data(), sizeof(double) * b->W, cudaMemcpyHostToDevice, b->stream), "upload");
    ck(cudaMemcpyAsync(b->judge_depth, dd.data(), sizeof(double) * b->W, cudaMemcpyHostToDevice, b->stream),
       "upload");
    ck(cudaStreamSynchronize(b->stream), "upload");
    b->judge_set = max_residual || max_depth;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_collect(shapes_batch* b, int64_t capacity) {
  if (!b || capacity < 0 || capacity > INT32_MAX) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->invalidate_graphs();
    dfree(b->ds_feat); dfree(b->ds_tgt); dfree(b->ds_count); dfree(b->snap_ds_count);
    b->ds_feat = b->ds_tgt = nullptr;
    b->ds_count = b->snap_ds_count = nullptr;
    b->ds_cap = 0;
    if (capacity == 0) return SHAPES_OK;
    b->ds_feat = dalloc<float>((size_t)capacity * mlp::kIn, "cudaMalloc samples");
    b->ds_tgt = dalloc<float>((size_t)capacity * mlp::kOut, "cudaMalloc samples");
    b->ds_count = dalloc<unsigned long long>(1, "cudaMalloc samples");
    b->snap_ds_count = dalloc<unsigned long long>(1, "cudaMalloc samples");
    ck(cudaMemsetAsync(b->ds_count, 0, sizeof(unsigned long long), b->stream), "memset");
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->ds_cap = capacity;
    return SHAPES_OK;
  });
}

int shapes_batch_get_samples(shapes_batch* b, float* features, float* targets, int64_t capacity, int64_t* n) {
  if (!b || !n || capacity < 0 || (capacity > 0 && (!features || !targets))) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    unsigned long long cnt = 0;
    if (b->ds_count) {
      ck(cudaMemcpyAsync(&cnt, b->ds_count, sizeof(cnt), cudaMemcpyDeviceToHost, b->stream), "download");
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    *n = (int64_t)cnt;
    const int64_t k = std::min<int64_t>((int64_t)cnt, capacity);
    if (k > 0) {
      ck(cudaMemcpyAsync(features, b->ds_feat, sizeof(float) * mlp::kIn * k, cudaMemcpyDeviceToHost, b->stream),
         "download");
      ck(cudaMemcpyAsync(targets, b->ds_tgt, sizeof(float) * mlp::kOut * k, cudaMemcpyDeviceToHost, b->stream),
         "download");
      ck(cudaStreamSynchronize(b->stream), "download");
    }
    return (int64_t)cnt > capacity ? SHAPES_E_BUFFER : SHAPES_OK;
  });
}

int shapes_batch_set_stream(shapes_batch* b, void* cuda_stream) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->stream = cuda_stream ? static_cast<cudaStream_t>(cuda_stream) : b->own_stream;
    return SHAPES_OK;
  });
}

int shapes_batch_set_incremental(shapes_batch* b, int32_t enabled) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->incremental = enabled != 0;
    b->invalidate_graphs();
    b->reset_incremental();
    return SHAPES_OK;
  });
}

int shapes_batch_set_sweep_prune(shapes_batch* b, int32_t min_bodies) {
  if (!b || min_bodies < 0) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->sap_min_bodies = min_bodies;
    b->invalidate_graphs();
    b->setup_sap();
    return SHAPES_OK;
  });
}

int shapes_batch_set_wait_limit(shapes_batch* b, int64_t polls) {
  if (!b || polls < 0) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->lw_poll_limit = polls ? (long long)polls : shapes::kPollLimit;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_set_narrowphase_lanes(shapes_batch* b, int32_t lanes) {
  if (!b || (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32))
    return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->np_lanes = lanes;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_set_profiling(shapes_batch* b, int32_t enabled) {
  if (!b) return SHAPES_E_INVALID_ARG;
  b->profiling = enabled != 0;
  for (int k = 0; k < SHAPES_STAGE_COUNT; ++k) {
    b->prof_ms[k] = 0.0;
    b->prof_launches[k] = 0;
  }
  return SHAPES_OK;
}

int shapes_batch_get_profile(shapes_batch* b, double* ms, int64_t* launches) {
  if (!b || !ms || !launches) return SHAPES_E_INVALID_ARG;
  for (int k = 0; k < SHAPES_STAGE_COUNT; ++k) {
    ms[k] = b->prof_ms[k];
    launches[k] = b->prof_launches[k];
    b->prof_ms[k] = 0.0;
    b->prof_launches[k] = 0;
  }
  return SHAPES_OK;
}

int shapes_batch_get_group_clocks(shapes_batch* b, int64_t* out, int32_t* n_groups) {
  if (!b || !n_groups) return SHAPES_E_INVALID_ARG;
  *n_groups = b->phase_clock_groups;
  if (!out) return SHAPES_OK;
  return guarded([&]() -> int {
    ck(cudaMemcpy(out, b->phase_clock, sizeof(long long) * 8 * b->phase_clock_groups, cudaMemcpyDeviceToHost),
       "download");
    return SHAPES_OK;
  });
}

int shapes_batch_set_launch_groups(shapes_batch* b, int32_t worlds_per_group, int32_t threads) {
  if (!b || worlds_per_group < 1 || worlds_per_group > shapes::kMaxGroupWorlds || threads < 0 || threads > 256 ||
      (threads % 32) != 0)
    return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    b->target_group_bodies = 0;
    b->worlds_per_group_override = worlds_per_group;
    b->solve_threads = threads > 0 ? threads : 32;
    b->make_groups(b->grouped_iterations >= 0 ? b->grouped_iterations : 2);
    return SHAPES_OK;
  });
}

int shapes_batch_set_group_warps(shapes_batch* b, int32_t warps) {
  if (!b || (warps != 1 && warps != 2 && warps != 4 && warps != 8)) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->group_warps = warps;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_set_world_order(shapes_batch* b, const int32_t* order) {
  if (!b) return SHAPES_E_INVALID_ARG;
  if (order) {
    std::vector<char> seen(b->W, 0);
    for (int32_t k = 0; k < b->W; ++k) {
      if (order[k] < 0 || order[k] >= b->W || seen[order[k]]) return SHAPES_E_INVALID_ARG;
      seen[order[k]] = 1;
    }
  }
  return guarded([&]() -> int {
    if (order)
      b->world_order.assign(order, order + b->W);
    else
      b->world_order.clear();
    b->make_groups(b->grouped_iterations >= 0 ? b->grouped_iterations : 2);
    return SHAPES_OK;
  });
}

int shapes_batch_get_world_order(shapes_batch* b, int32_t* order) {
  if (!b || !order) return SHAPES_E_INVALID_ARG;
  if ((int)b->world_order.size() == b->W) {
    std::copy(b->world_order.begin(), b->world_order.end(), order);
  } else {
    for (int32_t k = 0; k < b->W; ++k) order[k] = k;
    std::stable_sort(order, order + b->W, [&](int a, int c) {
      return (b->h_world_body_off[a + 1] - b->h_world_body_off[a]) > (b->h_world_body_off[c + 1] - b->h_world_body_off[c]);
    });
  }
  return SHAPES_OK;
}

int shapes_batch_get_world_levels(shapes_batch* b, int32_t* levels) {
  if (!b || !levels) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaMemcpyAsync(levels, b->world_levels, sizeof(int32_t) * b->W, cudaMemcpyDeviceToHost, b->stream), "download");
    ck(cudaStreamSynchronize(b->stream), "download");
    return SHAPES_OK;
  });
}

int shapes_batch_set_parallel_levels(shapes_batch* b, int32_t enabled) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->parallel_levels = enabled != 0;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_get_group_target(shapes_batch* b, int32_t* target_bodies) {
  if (!b || !target_bodies) return SHAPES_E_INVALID_ARG;
  *target_bodies = b->target_group_bodies;
  return SHAPES_OK;
}

int shapes_batch_get_launch(shapes_batch* b, int32_t* worlds_per_group, int32_t* threads, int32_t* group_warps) {
  if (!b) return SHAPES_E_INVALID_ARG;
  if (worlds_per_group) *worlds_per_group = b->worlds_per_group_override;
  if (threads) *threads = b->solve_threads;
  if (group_warps) *group_warps = b->group_warps;
  return SHAPES_OK;
}

int shapes_batch_set_spread_heavy(shapes_batch* b, int32_t enabled) {
  if (!b) return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    ck(cudaStreamSynchronize(b->stream), "sync");
    b->spread_heavy = enabled != 0;
    b->invalidate_graphs();
    return SHAPES_OK;
  });
}

int shapes_batch_get_spread_heavy(shapes_batch* b, int32_t* enabled) {
  if (!b || !enabled) return SHAPES_E_INVALID_ARG;
  *enabled = b->spread_heavy ? 1 : 0;
  return SHAPES_OK;
}

int shapes_batch_get_parallel_levels(shapes_batch* b, int32_t* enabled) {
  if (!b || !enabled) return SHAPES_E_INVALID_ARG;
  *enabled = b->parallel_levels ? 1 : 0;
  return SHAPES_OK;
}

int shapes_batch_set_launch(shapes_batch* b, int32_t target_bodies_per_group, int32_t threads) {
  if (!b || target_bodies_per_group < 0 || threads < 0 || threads > 256 || (threads % 32) != 0)
    return SHAPES_E_INVALID_ARG;
  return guarded([&]() -> int {
    b->target_group_bodies = target_bodies_per_group;
    b->worlds_per_group_override = 0;
    b->solve_threads = threads > 0 ? threads : 32;
    b->make_groups(b->grouped_iterations >= 0 ? b->grouped_iterations : 2);
    return SHAPES_OK;
  });
}

}  // extern "C"

/* ------------------------------------------------------------------------ */
/* Broadphase + contact generation without allocating                        */
/* ------------------------------------------------------------------------ */
/*
 * shapes_collide_noalloc serves callers that cannot allocate device memory
 * themselves: plugins whose host application owns every device buffer and
 * hands out pre-planned memory, and loops with a latency budget in which
 * cudaMalloc/cudaFree (which synchronize the whole device) are not allowed.
 * Its scratch lives in the fixed device array below, sized for at most
 * SHAPES_NOALLOC_MAX_BODIES bodies, SHAPES_NOALLOC_MAX_VERTS vertices and
 * SHAPES_NOALLOC_MAX_PAIRS broadphase pairs.  Every GPU that loads this
 * library holds that array until the process exits.
 */
namespace {

constexpr int kNaMaxBodies = SHAPES_NOALLOC_MAX_BODIES;
constexpr int kNaMaxVerts = SHAPES_NOALLOC_MAX_VERTS;
constexpr int kNaMaxPairs = SHAPES_NOALLOC_MAX_PAIRS;
constexpr int kNaMaxContacts = 2 * kNaMaxPairs;
constexpr int kNaTiles = (kNaMaxPairs + 1 + shapes::kScanTile - 1) / shapes::kScanTile + 1;

/* Byte offsets of the scratch arrays, each 256-byte aligned. */
struct NaPlan {
  size_t world_body_off, body_world, lx, ly, emin, emax, wx, wy, nx, ny, box, boxk, flags, row_mode, row_cnt,
      row_off, pair_a, pair_b, slot_cnt, slot_off, slot_feat, slot_val, world_pair_off, cwo, c_key, c_ga, c_gb,
      c_flip, c_hit, c_val, tile_sums, counters, total;
};

constexpr size_t na_take(size_t& o, size_t bytes) {
  const size_t at = o;
  o += (bytes + 255) & ~size_t(255);
  return at;
}

constexpr NaPlan na_plan() {
  NaPlan p{};
  size_t o = 0;
  p.world_body_off = na_take(o, 2 * sizeof(int32_t));
  p.body_world = na_take(o, kNaMaxBodies * sizeof(int32_t));
  p.lx = na_take(o, kNaMaxVerts * sizeof(double));
  p.ly = na_take(o, kNaMaxVerts * sizeof(double));
  p.emin = na_take(o, kNaMaxVerts * sizeof(int32_t));
  p.emax = na_take(o, kNaMaxVerts * sizeof(int32_t));
  p.wx = na_take(o, kNaMaxVerts * sizeof(double));
  p.wy = na_take(o, kNaMaxVerts * sizeof(double));
  p.nx = na_take(o, kNaMaxVerts * sizeof(double));
  p.ny = na_take(o, kNaMaxVerts * sizeof(double));
  p.box = na_take(o, 4 * kNaMaxBodies * sizeof(double));
  p.boxk = na_take(o, 4 * kNaMaxBodies * sizeof(uint64_t));
  p.flags = na_take(o, kNaMaxBodies);
  p.row_mode = na_take(o, kNaMaxBodies);
  p.row_cnt = na_take(o, kNaMaxBodies * sizeof(int32_t));
  p.row_off = na_take(o, (kNaMaxBodies + 1) * sizeof(int32_t));
  p.pair_a = na_take(o, kNaMaxPairs * sizeof(int32_t));
  p.pair_b = na_take(o, kNaMaxPairs * sizeof(int32_t));
  p.slot_cnt = na_take(o, kNaMaxPairs * sizeof(int32_t));
  p.slot_off = na_take(o, (kNaMaxPairs + 1) * sizeof(int32_t));
  p.slot_feat = na_take(o, 2 * (size_t)kNaMaxPairs * sizeof(int32_t));
  p.slot_val = na_take(o, 10 * (size_t)kNaMaxPairs * sizeof(double));
  p.world_pair_off = na_take(o, 2 * sizeof(int32_t));
  p.cwo = na_take(o, 2 * sizeof(int32_t));
  p.c_key = na_take(o, kNaMaxContacts * sizeof(uint64_t));
  p.c_ga = na_take(o, kNaMaxContacts * sizeof(int32_t));
  p.c_gb = na_take(o, kNaMaxContacts * sizeof(int32_t));
  p.c_flip = na_take(o, kNaMaxContacts);
  p.c_hit = na_take(o, kNaMaxContacts);
  p.c_val = na_take(o, 5 * (size_t)kNaMaxContacts * sizeof(double));
  p.tile_sums = na_take(o, kNaTiles * sizeof(int32_t));
  p.counters = na_take(o, 8 * sizeof(unsigned long long));
  p.total = o;
  return p;
}

constexpr NaPlan kNaPlan = na_plan();

}  // namespace

/* The scratch.  Device code may name it directly; in host code the name is a
 * host-side stand-in, not a device address, so the host uses the address that
 * cudaGetSymbolAddress returns (resolved once per device below). */
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNaPlan.total];

namespace {

/* Reasons the set-up kernel rejects an input (bits of the bad-input counter). */
constexpr unsigned long long kNaBadOffsets = 1, kNaBadNaN = 2, kNaBadNonconvex = 4, kNaBadEdge = 8;

/* Per-call set-up in scratch: the one-world offsets, de-interleaved local
 * vertices and zeroed row modes.  Validates the caller's input as
 * shapes_batch_create does on the host, so that no later kernel indexes
 * outside the vertex arrays or meets a hull it cannot handle: every body needs
 * 3..64 vertices inside [0, n_verts) (offsets starting at 0 and ending at
 * n_verts), a strictly convex counter-clockwise hull of finite points with no
 * zero-length edge (the same products and comparisons as the host check), and
 * finite position, angle and inverse masses.  The counters were zeroed by the
 * host before this kernel. */
__global__ void k_noalloc_setup(int n, int nv, const int32_t* vert_off, const double* local_xy, const double* px,
                                const double* py, const double* th, const double* iml, const double* imr,
                                unsigned char* base) {
  int32_t* wbo = reinterpret_cast<int32_t*>(base + kNaPlan.world_body_off);
  int32_t* bw = reinterpret_cast<int32_t*>(base + kNaPlan.body_world);
  uint8_t* mode = base + kNaPlan.row_mode;
  double* lx = reinterpret_cast<double*>(base + kNaPlan.lx);
  double* ly = reinterpret_cast<double*>(base + kNaPlan.ly);
  unsigned long long* cnt = reinterpret_cast<unsigned long long*>(base + kNaPlan.counters);
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  if (t0 == 0) {
    wbo[0] = 0;
    wbo[1] = n;
    if (vert_off[0] != 0 || vert_off[n] != nv) atomicOr(&cnt[shapes::kCntBadInput], kNaBadOffsets);
  }
  for (int i = t0; i < n; i += stride) {
    bw[i] = 0;
    mode[i] = 0;
    unsigned long long bad = 0;
    if (!isfinite(px[i]) || !isfinite(py[i]) || !isfinite(th[i]) || !isfinite(iml[i]) || !isfinite(imr[i]))
      bad |= kNaBadNaN;
    const int o0 = vert_off[i], o1 = vert_off[i + 1], c = o1 - o0;
    if (o0 < 0 || o1 > nv || c < 3 || c > shapes::kMaxVerts) {
      bad |= kNaBadOffsets;
    } else { /* the hull lies inside the caller's vertex array: check it */
      const double* xy = local_xy + 2 * (size_t)o0;
      for (int k = 0; k < 2 * c; ++k)
        if (!isfinite(xy[k])) bad |= kNaBadNaN;
      if (!(bad & kNaBadNaN)) {
        for (int k = 0; k < c; ++k) {
          const int k1 = k + 1 < c ? k + 1 : k + 1 - c, k2 = k + 2 < c ? k + 2 : k + 2 - c;
          const double ex = xy[2 * k1] - xy[2 * k], ey = xy[2 * k1 + 1] - xy[2 * k + 1];
          const double fx = xy[2 * k2] - xy[2 * k1], fy = xy[2 * k2 + 1] - xy[2 * k1 + 1];
          if (ex == 0.0 && ey == 0.0) bad |= kNaBadEdge;
          else if (ex * fy - ey * fx <= 0.0) bad |= kNaBadNonconvex;
        }
      }
    }
    if (bad) atomicOr(&cnt[shapes::kCntBadInput], bad);
  }
  for (int v = t0; v < nv; v += stride) {
    lx[v] = local_xy[2 * (size_t)v];
    ly[v] = local_xy[2 * (size_t)v + 1];
  }
}

/* Copies pairs and contacts from scratch into the caller's buffers. */
__global__ void k_noalloc_out(int n_pairs, int n_contacts, const unsigned char* base, int32_t* pairs_ij,
                              int32_t* keys5, double* vals5) {
  const int32_t* pa = reinterpret_cast<const int32_t*>(base + kNaPlan.pair_a);
  const int32_t* pb = reinterpret_cast<const int32_t*>(base + kNaPlan.pair_b);
  const uint64_t* key = reinterpret_cast<const uint64_t*>(base + kNaPlan.c_key);
  const uint8_t* flip = base + kNaPlan.c_flip;
  const double* val = reinterpret_cast<const double*>(base + kNaPlan.c_val);
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int p = t0; p < n_pairs; p += stride) {
    pairs_ij[2 * p] = pa[p];
    pairs_ij[2 * p + 1] = pb[p];
  }
  for (int c = t0; c < n_contacts; c += stride) {
    const uint64_t k = key[c];
    keys5[5 * c] = (int32_t)(k >> 44);
    keys5[5 * c + 1] = (int32_t)((k >> 24) & 0xfffff);
    keys5[5 * c + 2] = (int32_t)((k >> 12) & 0xfff);
    keys5[5 * c + 3] = (int32_t)(k & 0xfff);
    keys5[5 * c + 4] = flip[c];
    for (int q = 0; q < 5; ++q) vals5[5 * c + q] = val[5 * (size_t)c + q];
  }
}

constexpr int kMaxDevices = 64;

/* Device address of g_noalloc_scratch on the current device, looked up once
 * per device (the first call on a device does this set-up). */
int noalloc_scratch_ptr(unsigned char** out) {
  static std::atomic<unsigned char*> ptrs[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SHAPES_E_CUDA;
  unsigned char* p = ptrs[dev].load();
  if (!p) {
    void* addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess) {
      g_last_error = std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return SHAPES_E_CUDA;
    }
    p = static_cast<unsigned char*>(addr);
    ptrs[dev].store(p);
  }
  *out = p;
  return SHAPES_OK;
}

}  // namespace

extern "C" int shapes_collide_noalloc(int32_t n_bodies, const double* pos_x, const double* pos_y, const double* rot,
                                      const double* inv_mass_lin, const double* inv_mass_rot,
                                      const int32_t* vert_offsets, const double* local_verts_xy, int32_t n_verts,
                                      int32_t* pairs_ij, int64_t pair_capacity, int32_t* contact_keys5,
                                      double* contact_vals5, int64_t contact_capacity, void* cuda_stream,
                                      int64_t* n_pairs, int64_t* n_contacts) {
  if (!pos_x || !pos_y || !rot || !inv_mass_lin || !inv_mass_rot || !vert_offsets || !local_verts_xy || !n_pairs ||
      !n_contacts || n_bodies < 1 || n_verts < 3 * n_bodies) {
    g_last_error = "shapes_collide_noalloc: a null pointer, no bodies, or fewer than 3 vertices per body";
    return SHAPES_E_INVALID_ARG;
  }
  if (n_bodies > kNaMaxBodies || n_verts > kNaMaxVerts) {
    g_last_error = "shapes_collide_noalloc: more than SHAPES_NOALLOC_MAX_BODIES bodies or SHAPES_NOALLOC_MAX_VERTS vertices";
    return SHAPES_E_CAPACITY;
  }
  unsigned char* base = nullptr;
  const int rc = noalloc_scratch_ptr(&base);
  if (rc != SHAPES_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
  Dev d{};
  d.n_worlds = 1;
  d.n_bodies = n_bodies;
  d.n_verts = n_verts;
  d.pair_cap = kNaMaxPairs;
  d.contact_cap = kNaMaxContacts;
  d.world_body_off = reinterpret_cast<int32_t*>(base + kNaPlan.world_body_off);
  d.body_world = reinterpret_cast<int32_t*>(base + kNaPlan.body_world);
  d.vert_off = vert_offsets;
  d.lx = reinterpret_cast<double*>(base + kNaPlan.lx);
  d.ly = reinterpret_cast<double*>(base + kNaPlan.ly);
  d.emin = reinterpret_cast<int32_t*>(base + kNaPlan.emin);
  d.emax = reinterpret_cast<int32_t*>(base + kNaPlan.emax);
  d.px = const_cast<double*>(pos_x);
  d.py = const_cast<double*>(pos_y);
  d.th = const_cast<double*>(rot);
  d.iml = inv_mass_lin;
  d.imr = inv_mass_rot;
  d.wx = reinterpret_cast<double*>(base + kNaPlan.wx);
  d.wy = reinterpret_cast<double*>(base + kNaPlan.wy);
  d.nx = reinterpret_cast<double*>(base + kNaPlan.nx);
  d.ny = reinterpret_cast<double*>(base + kNaPlan.ny);
  d.box = reinterpret_cast<double*>(base + kNaPlan.box);
  d.boxk = reinterpret_cast<uint64_t*>(base + kNaPlan.boxk);
  d.flags = base + kNaPlan.flags;
  d.row_mode = base + kNaPlan.row_mode;
  d.row_cnt = reinterpret_cast<int32_t*>(base + kNaPlan.row_cnt);
  d.row_off = reinterpret_cast<int32_t*>(base + kNaPlan.row_off);
  d.pair_a = reinterpret_cast<int32_t*>(base + kNaPlan.pair_a);
  d.pair_b = reinterpret_cast<int32_t*>(base + kNaPlan.pair_b);
  d.slot_cnt = reinterpret_cast<int32_t*>(base + kNaPlan.slot_cnt);
  d.slot_off = reinterpret_cast<int32_t*>(base + kNaPlan.slot_off);
  d.slot_feat = reinterpret_cast<int32_t*>(base + kNaPlan.slot_feat);
  d.slot_val = reinterpret_cast<double*>(base + kNaPlan.slot_val);
  d.world_pair_off = reinterpret_cast<int32_t*>(base + kNaPlan.world_pair_off);
  d.world_contact_off = reinterpret_cast<int32_t*>(base + kNaPlan.cwo);
  d.c_key = reinterpret_cast<uint64_t*>(base + kNaPlan.c_key);
  d.c_ga = reinterpret_cast<int32_t*>(base + kNaPlan.c_ga);
  d.c_gb = reinterpret_cast<int32_t*>(base + kNaPlan.c_gb);
  d.c_flip = base + kNaPlan.c_flip;
  d.c_hit = base + kNaPlan.c_hit;
  d.c_val = reinterpret_cast<double*>(base + kNaPlan.c_val);
  d.counters = reinterpret_cast<unsigned long long*>(base + kNaPlan.counters);
  int32_t* tile_sums = reinterpret_cast<int32_t*>(base + kNaPlan.tile_sums);
  auto scan = [&](const int32_t* in, int n_cap, const unsigned long long* n_dev, int32_t* out) {
    const int tiles = (n_cap + 1 + shapes::kScanTile - 1) / shapes::kScanTile;
    shapes::k_scan_tiles<<<tiles, shapes::kScanThreads, 0, st>>>(in, n_cap, n_dev, tile_sums);
    shapes::k_scan_tile_sums<<<1, 1024, 0, st>>>(tile_sums, tiles);
    shapes::k_scan_apply<<<tiles, shapes::kScanThreads, 0, st>>>(in, n_cap, n_dev, tile_sums, out);
  };
  /* counters start at zero; the set-up kernel validates the vertex offsets */
  cudaError_t e = cudaMemsetAsync(d.counters, 0, 8 * sizeof(unsigned long long), st);
  unsigned long long cnt[8] = {0};
  if (e == cudaSuccess) {
    k_noalloc_setup<<<grid_for(std::max(n_bodies, n_verts), 256), 256, 0, st>>>(
        n_bodies, n_verts, vert_offsets, local_verts_xy, pos_x, pos_y, rot, inv_mass_lin, inv_mass_rot, base);
    e = cudaMemcpyAsync(cnt, d.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_last_error = std::string("shapes_collide_noalloc: ") + cudaGetErrorString(e);
    return SHAPES_E_CUDA;
  }
  if (const unsigned long long bad = cnt[shapes::kCntBadInput]) {
    if (bad & (kNaBadOffsets | kNaBadEdge)) {
      g_last_error = (bad & kNaBadOffsets)
                         ? "shapes_collide_noalloc: vert_offsets must start at 0, end at n_verts and give every body "
                           "3..64 vertices (circles are not accepted)"
                         : "shapes_collide_noalloc: a hull has a zero-length edge";
      return SHAPES_E_INVALID_ARG;
    }
    if (bad & kNaBadNaN) {
      g_last_error = "shapes_collide_noalloc: a position, angle, inverse mass or hull point is not finite";
      return SHAPES_E_NAN;
    }
    g_last_error = "shapes_collide_noalloc: a hull is not strictly convex and counter-clockwise";
    return SHAPES_E_NONCONVEX;
  }
  shapes::k_init_extents<<<grid_for(n_verts, 128), 128, 0, st>>>(d);
  shapes::k_integrate_pose<<<grid_for(n_bodies, 128), 128, 0, st>>>(d, 0.0, 0);
  shapes::k_broadphase<true><<<grid_for((long long)n_bodies * 32, 256), 256, 0, st>>>(d);
  scan(d.row_cnt, n_bodies, nullptr, d.row_off);
  shapes::k_broadphase<false><<<grid_for((long long)n_bodies * 32, 256), 256, 0, st>>>(d);
  shapes::k_world_pair_offsets<<<1, 32, 0, st>>>(d);
  shapes::k_narrowphase<<<grid_for(kNaMaxPairs, 128), 128, 0, st>>>(d);
  scan(d.slot_cnt, kNaMaxPairs, d.counters + shapes::kCntPairs, d.slot_off);
  shapes::k_world_contact_offsets<<<1, 32, 0, st>>>(d);
  shapes::k_build<<<grid_for(2LL * kNaMaxPairs, 128), 128, 0, st>>>(d, 1.0, 0.0, 0.0, 0, 0);
  e = cudaMemcpyAsync(cnt, d.counters, sizeof(cnt), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) {
    g_last_error = std::string("shapes_collide_noalloc: ") + cudaGetErrorString(e);
    return SHAPES_E_CUDA;
  }
  *n_pairs = (int64_t)cnt[shapes::kCntPairs];
  *n_contacts = (int64_t)cnt[shapes::kCntContacts];
  if (cnt[shapes::kCntOverflow]) {
    g_last_error = "shapes_collide_noalloc: more than SHAPES_NOALLOC_MAX_PAIRS broadphase pairs";
    return SHAPES_E_CAPACITY;
  }
  if (*n_pairs > pair_capacity || *n_contacts > contact_capacity) {
    g_last_error = "shapes_collide_noalloc: pair_capacity or contact_capacity below *n_pairs / *n_contacts";
    return SHAPES_E_BUFFER;
  }
  if ((*n_pairs > 0 && !pairs_ij) || (*n_contacts > 0 && (!contact_keys5 || !contact_vals5))) {
    g_last_error = "shapes_collide_noalloc: null output buffer";
    return SHAPES_E_INVALID_ARG;
  }
  if (*n_pairs > 0 || *n_contacts > 0) {
    k_noalloc_out<<<grid_for(std::max(*n_pairs, *n_contacts), 256), 256, 0, st>>>(
        (int)*n_pairs, (int)*n_contacts, base, pairs_ij, contact_keys5, contact_vals5);
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) {
      g_last_error = std::string("shapes_collide_noalloc: ") + cudaGetErrorString(e);
      return SHAPES_E_CUDA;
    }
  }
  return SHAPES_OK;
}
