// Host side of the C ABI in include/nclr_gpu.h.  A handle holds one or more scenes (a plain
// simulation is a batch of one) and owns one CUDA stream; all scenes share one device-resident
// particle store (two SoA buffers that the block sort ping-pongs between; scene s owns a fixed
// slot range), the two grids (G: the coming step's P2G accumulator; V: the last step's updated
// grid; scene s owns a node range of each) and the sort scratch.  advance() enqueues per step
//   [every sort_interval steps: block keys -> scan -> active-block list -> move]
//   grid sweep (V = grid_op(G), G = 0 on touched blocks) -> g2p2g (G2P + next P2G)
// for every scene at once, after a P2G-only launch when the particle state was just
// uploaded, replaying a captured CUDA graph for whole sort intervals.  Only the last step of
// a call writes v and C.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mpm_device.cuh"
#include "mpm_launch.h"
#include "nclr_gpu.h"

using mpm::Params;
using mpm::PState;
using mpm::Scene;

struct nclr_sim {
  int dim = 0, device = 0, nscenes = 0;
  int64_t n = 0;  // particles of all scenes
  nclr_options opt{};
  bool ref = true;
  bool has_mat = false;
  cudaStream_t stream = nullptr;

  std::vector<Scene> scenes;   // host copy of the scene table
  Scene *scenes_d = nullptr;
  uint16_t *block_scene = nullptr;  // scene of every global block (batches only)
  int64_t total_nodes = 0;
  int total_blocks = 0;
  int64_t nkeys = 0;

  void *slab[2] = {nullptr, nullptr};  // particle SoA buffers
  PState ps[2]{};
  float2 *lame_buf = nullptr;  // per-particle (mu_0, lambda_0) of ps[0] and ps[1] (2 n), if set
  int cur = 0;
  int sms = 1;         // streaming multiprocessors of the device
  int g2p2g_ctas = 1;  // persistent CTAs of the fused kernel
  int g2p_ctas = 1;    // persistent CTAs of its G2P-only final step

  float4 *G = nullptr;        // P2G accumulator of the coming step
  float4 *V = nullptr;        // updated grid of the last step (grid())
  uint8_t *flags = nullptr;   // per grid block: pending contributions in G / non-zero V
  int *key = nullptr, *rank = nullptr, *count = nullptr, *tile_sums = nullptr;
  int *btotal = nullptr;      // particles per grid block (the last sort)
  int *start = nullptr;       // first slot of every grid block (exclusive scan of btotal)
  int4 *rounds = nullptr;     // per-block round tables of the slot order (see sort_move_kernel)
  int *blocks = nullptr;      // non-empty blocks of the last sort (the dense ones)
  int *nblocks_active = nullptr;  // [0], [2]: blocks at the front and back of `blocks`, [1]
                                  // slots in `sparse`, [3] capacity of `blocks`
  int *sparse = nullptr;      // particle slots of the thin blocks (stepped without a tile)
  int sparse_max = 0;         // blocks with fewer particles than this are thin
  int tail_max = 0;           // a block's last pass of fewer particles goes to the chunks
  mpm::Record record{};       // where final-mode steps also write the caller-order state
  int *inv = nullptr;         // global caller id -> slot (the permutation of the last sort)
  int *slot_block = nullptr;  // slot -> grid block it was sorted into
  int *moved_d = nullptr;     // rows of the last host upload that left their slot's block
  int *moved_h = nullptr;     // pinned copy
  bool sorted_once = false;   // slot_block is valid
  cudaStream_t copy_stream = nullptr;  // host transfers, pipelined field by field
  unsigned *bar = nullptr;    // the small-scene kernels' barriers (2 counters per scene)
  mpm::BarrierTest bar_test;  // nclr_debug_set_barrier: the barrier's poll limit and extra arrivals
  mpm::SnowFix fix;           // the FP64 snow clamps of a fused launch (allocated when snow may occur)
  uint16_t *cta_scene = nullptr;  // batches: scene of each CTA of the small-scene kernel
  int *group_first = nullptr;     // batches: first CTA of each scene's group (nscenes + 1)
  int batch_ctas = 0;             // batches: CTAs of that launch (0: not possible)
  int small_max = 0;          // particles up to which advance() uses the small-scene kernel
  bool small_auto = false;    // the default limits: also at most kSmallNodesPerParticle nodes
  int small_ctas = 0;         // its CTAs that fit on the device at once (0: no cooperative launch)
  int cluster_max = 0;        // CTAs of the largest cluster it can run as (0: no cluster launch)
  cudaEvent_t field_ev[5] = {};        // x, v, F, C, Jp ready (staged / imported)
  int *work = nullptr;        // fused kernel's block counter
  int *err_d = nullptr;       // per scene: [2s] this call's steps, [2s+1] the P2G after them
  int *err_h = nullptr;       // pinned copy
  std::vector<int> deferred_err;  // [2s+1] of the previous call, reported by the next one
  std::vector<int> scene_err;     // the last call's errors per scene
  bool acc_valid = false;     // G holds the P2G of the coming step
  // The last call's pending P2G was thrown away by an upload before the next step (the caller
  // replaces the state between calls): the next call ends with a G2P-only step, and the call
  // after it recomputes its first P2G.  A call that finds no upload in between switches back.
  bool p2g_discarded = false;
  bool replaced = false;      // an upload (or new moduli) since the last advance() call
  bool need_sort = true;      // the block lists do not describe the particles yet

  float *staging = nullptr;       // particle-major transfer buffer (n * row floats)
  float *grid_staging = nullptr;  // grid export buffer (largest scene)

  bool stepped = false;  // grid() is empty until the first advance (src/nclr.h:101)
  int64_t steps_since_sort = 0;
  // [parity][0: a chunk that does not end the call, 1: the call's last chunk, 2: the same
  // ending with the G2P-only step]
  cudaGraphExec_t graph[2][3] = {{nullptr, nullptr, nullptr}, {nullptr, nullptr, nullptr}};
  int64_t graph_launches = 0;
  int64_t launches = 0;
  int64_t active_nodes = 0;
  unsigned long long *active_d = nullptr;

  // opt.profile: event pairs of the current advance() call, folded into per-phase totals
  std::vector<cudaEvent_t> ev_pool;
  struct Timed {
    int phase;
    cudaEvent_t a, b;
  };
  std::vector<Timed> pending;
  double prof_ms[NCLR_NUM_PHASES] = {};
  int64_t prof_launches[NCLR_NUM_PHASES] = {};
  std::string error;

  const Params &P0() const { return scenes[0].P; }
};

namespace {

thread_local std::string g_create_error;

// Default thin-block thresholds (particles per block at the last sort): below them the
// shared-memory tile of a block (load, clear, flush of 8^3 nodes in 3D, 12^2 in 2D) costs more
// than the block's particles gathering and scattering through L2 directly.
constexpr int kSparseMax3 = 64;
constexpr int kSparseMax2 = 32;
constexpr int kBatchThin = 32;  // batches: blocks below this many particles skip the tiles
// Default tail threshold of a single simulation: a block's last 256-particle pass of fewer
// particles than this goes to the thin-block chunks.  Measured per fused launch against no
// tail rule, twice each: with the block list in block order, 1M-particle jelly 144-148 ->
// 142-144 us (reference physics) and 162-165 -> 157-158 us (corrected), corrected snow 180
// -> 174 us, the 4.19M-particle liquid + snow scene 1297 -> 1271 us.  With multi-pass blocks
// first (compact_blocks_kernel) most of that gain is already there: jelly 141 -> 142 us,
// corrected jelly 158 -> 157, corrected snow 170 -> 169, liquid + snow 1289 -> 1267.  32 and
// 96 come within 1-2% of 64; 128 is slower on jelly and 192 everywhere (too many particles
// leave the tiles).  The autotuner has it as a knob.
constexpr int kTailMax = 64;
// Default small-scene limits: up to them one persistent launch per advance() call beats two
// launches per step.  Measured on GB300: up to 64k particles in 2D and 32k in 3D, and only
// while the grid has at most about 8 nodes per particle -- the small kernel updates every
// node each step, so a sparse scene on a large grid (1,000 particles on a 65^3 grid: 210 us
// per step against 17 us) belongs on the tile path, which visits only touched blocks.
constexpr int kSmallMax2 = 65536;
constexpr int kSmallMax3 = 32768;
constexpr int64_t kSmallNodesPerParticle = 8;

int row_floats(int dim) { return 2 * dim + 2 * dim * dim + 1; }  // x, v, F, C, Jp

nclr_status fail(nclr_sim *s, nclr_status st, const std::string &msg) {
  if (s)
    s->error = msg;
  else
    g_create_error = msg;
  return st;
}

#define CUDA_TRY(sim, call)                                                                \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return fail((sim), NCLR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Carves the SoA fields of one particle buffer out of a single allocation.
nclr_status alloc_particles(nclr_sim *s, int which) {
  const int D = s->dim;
  const size_t n = (size_t)std::max<int64_t>(s->n, 1);
  const size_t fbytes = align_up(n * sizeof(float), 256);
  const int nfloat_fields = 2 * D + 2 * D * D + 3;
  const size_t total = fbytes * nfloat_fields + align_up(n * sizeof(int), 256) + align_up(n, 256) +
                       align_up(n * sizeof(uint16_t), 256);
  char *base = nullptr;
  CUDA_TRY(s, cudaMalloc((void **)&base, total));
  s->slab[which] = base;
  PState &p = s->ps[which];
  size_t off = 0;
  auto take = [&](size_t comps) {
    float *r = (float *)(base + off);
    off += fbytes * comps;
    return r;
  };
  p.x = take(D);
  p.v = take(D);
  p.F = take((size_t)D * D);
  p.C = take((size_t)D * D);
  p.Jp = take(1);
  p.mass = take(1);
  p.vol = take(1);
  p.id = (int *)(base + off);
  off += align_up(n * sizeof(int), 256);
  p.mat = s->has_mat ? (uint8_t *)(base + off) : nullptr;
  off += align_up(n, 256);
  p.scene = s->nscenes > 1 ? (uint16_t *)(base + off) : nullptr;
  p.stride = (int)n;
  return NCLR_OK;
}

template <typename F>
void dispatch_dim(int dim, F &&f) {
  if (dim == 2)
    f(std::integral_constant<int, 2>{});
  else
    f(std::integral_constant<int, 3>{});
}

nclr_status check_launch(nclr_sim *s, const char *what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(s, NCLR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return NCLR_OK;
}

cudaEvent_t take_event(nclr_sim *s) {
  if (s->ev_pool.empty()) {
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  cudaEvent_t e = s->ev_pool.back();
  s->ev_pool.pop_back();
  return e;
}

// Brackets the work enqueued by `body` with a pair of events when profiling.
template <typename Body>
void phase(nclr_sim *s, int which, int launches, Body &&body) {
  if (!s->opt.profile) {
    body();
    return;
  }
  nclr_sim::Timed t{which, take_event(s), take_event(s)};
  cudaEventRecord(t.a, s->stream);
  body();
  cudaEventRecord(t.b, s->stream);
  s->pending.push_back(t);
  s->prof_launches[which] += launches;
}

// After the stream has drained: fold the pending event pairs into the phase totals.
void collect_profile(nclr_sim *s) {
  for (const auto &t : s->pending) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) s->prof_ms[t.phase] += ms;
    s->ev_pool.push_back(t.a);
    s->ev_pool.push_back(t.b);
  }
  s->pending.clear();
}

// Enqueues the block sort of the current buffer into the other one (v and C move too when
// the next P2G reads them, i.e. right after an upload).
void enqueue_sort(nclr_sim *s, bool move_vc) {
  const int nb = s->total_blocks;
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    constexpr int cpb = mpm::Tiling<D>::CPB;
    static_assert(cpb == mpm::kCellsPerBlock, "the round tables assume 64 cells per block");
    phase(s, NCLR_PHASE_SORT, 7, [&] {
      cudaMemsetAsync(s->count, 0, sizeof(int) * (size_t)s->nkeys, s->stream);
      cudaMemsetAsync(s->nblocks_active, 0, 4 * sizeof(int), s->stream);
      mpm::launch_block_keys<D>(s->ps[s->cur], (int)s->n, s->scenes_d, s->key, s->rank, s->count,
                                s->stream);
      mpm::launch_block_tables(s->count, nb, s->btotal, s->rounds, s->stream);
      mpm::launch_exclusive_scan(s->btotal, nb, s->start, s->tile_sums, s->stream);
      mpm::launch_compact_blocks(s->start, nb, 1, s->sparse_max, s->tail_max, s->blocks,
                                 s->nblocks_active, s->sparse, s->stream);
      mpm::launch_sort_move<D>(s->ps[s->cur], s->ps[s->cur ^ 1], (int)s->n, s->key, s->rank,
                               s->start, s->rounds, s->count, move_vc, s->inv, s->slot_block,
                               s->stream);
    });
  });
  s->cur ^= 1;
  s->sorted_once = true;
  s->launches += 7;  // keys, round tables, 3 scan kernels, compaction, move
}

// How a call's last step ends: with the next step's P2G (kept pending in G) or without it.
enum : int { kNotFinal = 0, kFinalWithP2G = 1, kFinalG2POnly = 2 };

// Enqueues one step of every scene (optionally preceded by the block sort) on the handle's
// stream.  The last step of a call (final != kNotFinal) writes v and C and, with its P2G,
// reports the next step's P2G errors separately.
void enqueue_step(nclr_sim *s, bool sort, int final) {
  if (sort && s->n > 0) enqueue_sort(s, false);
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    phase(s, NCLR_PHASE_GRID, 1, [&] {
      mpm::launch_grid_sweep<D>(s->G, s->V, s->flags, s->scenes_d, s->block_scene, s->P0(),
                                s->total_blocks, s->work, s->sms, s->stream, s->fix.count);
    });
    s->launches += 1;
    if (s->n > 0) {
      phase(s, NCLR_PHASE_G2P2G, 1, [&] {
        mpm::launch_g2p2g<D>(s->ps[s->cur], s->P0(), s->scenes_d, s->block_scene, s->V, s->G,
                             s->flags, s->blocks, s->nblocks_active, s->start, s->sparse, s->work, s->err_d,
                             final != kNotFinal ? 1 : 0, s->ref,
                             final == kFinalG2POnly  ? mpm::kModeG2PFinal
                             : final == kNotFinal    ? mpm::kModeStep
                                                     : mpm::kModeFinalStep,
                             final == kFinalG2POnly ? s->g2p_ctas : s->g2p2g_ctas, s->stream,
                             s->record, s->fix, s->opt.batch_item_threads);
      });
      s->launches += 1;
      if (s->fix.count) {  // the snow clamps that launch left for FP64
        phase(s, NCLR_PHASE_SNOW_FIX, 1, [&] {
          mpm::launch_snow_fix<D>(s->ps[s->cur], s->P0(), s->nscenes > 1 ? s->scenes_d : nullptr,
                                  s->fix, s->G, final != kFinalG2POnly, s->ref, s->record, s->sms,
                                  s->stream);
        });
        s->launches += 1;
      }
    }
  });
}

// The P2G of the coming step from the stored state (after an upload, new moduli, or a call
// that ended without it): clears what G holds, then one P2G-only launch.
void enqueue_pending_p2g(nclr_sim *s) {
  std::fill(s->deferred_err.begin(), s->deferred_err.end(), 0);  // discarded with the P2G
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    phase(s, NCLR_PHASE_P2G, 2, [&] {
      mpm::launch_discard_pending<D>(s->G, s->flags, s->scenes_d, s->block_scene,
                                     s->total_blocks, s->sms, s->stream);
      // the fused kernel's block counter (before a regular step the sweep resets it)
      cudaMemsetAsync(s->work, 0, sizeof(int), s->stream);
      if (s->n > 0)
        mpm::launch_g2p2g<D>(s->ps[s->cur], s->P0(), s->scenes_d, s->block_scene, s->V, s->G,
                             s->flags, s->blocks, s->nblocks_active, s->start, s->sparse,
                             s->work, s->err_d, 0, s->ref, mpm::kModeP2GOnly, s->g2p2g_ctas,
                             s->stream, mpm::Record{}, mpm::SnowFix{}, s->opt.batch_item_threads);
    });
  });
  s->launches += (s->n > 0) ? 2 : 1;
  s->acc_valid = true;
}

bool sort_due(const nclr_sim *s) {
  return s->need_sort ||
         (s->opt.sort_interval > 0 && s->steps_since_sort >= s->opt.sort_interval);
}

// Steps per graph: a multiple of the sort interval (the graph starts at a sort boundary).
int64_t chunk_steps(const nclr_sim *s) {
  const int64_t si = s->opt.sort_interval;
  if (s->opt.graph_steps <= 0) return si > 0 ? si : 16;
  return si > 0 ? (s->opt.graph_steps + si - 1) / si * si : s->opt.graph_steps;
}

// Sorts inside one graph (one at the start of every sort interval).
int64_t chunk_sorts(const nclr_sim *s) {
  return s->opt.sort_interval > 0 ? chunk_steps(s) / s->opt.sort_interval : 0;
}

// Captures chunk_steps() steps starting at a sort boundary from buffer parity `parity`; with
// `final` != kNotFinal its last step is the call's final step of that kind (writes v and C).
nclr_status capture_graph(nclr_sim *s, int parity, int final) {
  const int saved_cur = s->cur;
  const int64_t saved_launches = s->launches;
  s->cur = parity;
  cudaGraph_t g = nullptr;
  CUDA_TRY(s, cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
  const int64_t k = chunk_steps(s);
  const int64_t si = s->opt.sort_interval;
  for (int64_t i = 0; i < k; ++i) enqueue_step(s, si > 0 && i % si == 0, i == k - 1 ? final : kNotFinal);
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  s->graph_launches = s->launches - saved_launches;
  s->launches = saved_launches;
  s->cur = saved_cur;
  if (e != cudaSuccess) return fail(s, NCLR_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&s->graph[parity][final], g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(s, NCLR_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
  return NCLR_OK;
}

// The step parameters of one scene (the reference's constructor, src/nclr.h:74-78).
Params scene_params(int dim, int64_t n, int model, int res, float dt, float E, float nu,
                    float gravity) {
  Params P{};
  P.res = res;
  P.N = res + 1;
  P.n = (int)n;
  P.model = model;
  P.dt = dt;
  // dx = 1.0 / res in double, narrowed (src/nclr.h:76); inv_dx = 1 / dx in float
  P.dx = (float)(1.0 / res);
  P.inv_dx = 1.0f / P.dx;
  P.gravity = gravity;
  P.allowed = (float)((double)P.dx * 0.9 / (double)dt);  // src/nclr.h:285
  // mu_0, lambda_0 (src/nclr.h:77-78), evaluated in float like the reference's `real`
  P.mu0 = E / (2.0f * (1.0f + nu));
  P.lambda0 = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  P.Dinv = 4.0f * P.inv_dx * P.inv_dx;
  P.cscale = 4.0f * P.inv_dx;
  P.dt_gravity = dt * gravity;
  int64_t nodes = 1;
  for (int d = 0; d < dim; ++d) nodes *= P.N;
  P.nodes = nodes;
  const int bs = (dim == 3) ? mpm::Tiling<3>::BS : mpm::Tiling<2>::BS;
  P.nb = (P.N + bs - 1) / bs;
  P.nblocks = 1;
  for (int d = 0; d < dim; ++d) P.nblocks *= P.nb;
  return P;
}

// Upload of caller-ordered rows (device memory) into the slots of scene `sc` (-1: all); the
// next advance() then recomputes the coming P2G from them and re-sorts.
// Rows of scene sc (-1: all scenes) -> their slots.  New positions mean a re-sort before the
// next step; with count_moved (and a sort to compare with) the rows that left their slot's
// grid block are counted into moved_h (valid after the stream synchronises), so that a caller
// who synchronises anyway can skip that re-sort when none did.
nclr_status import_rows(nclr_sim *s, int sc, const float *x, const float *v, const float *F,
                        const float *C, const float *Jp, bool count_moved = false) {
  const int id_off = sc < 0 ? 0 : s->scenes[sc].slot_off;
  const int count = sc < 0 ? (int)s->n : s->scenes[sc].P.n;
  int *moved = (count_moved && x && s->sorted_once) ? s->moved_d : nullptr;
  if (moved) CUDA_TRY(s, cudaMemsetAsync(moved, 0, sizeof(int), s->stream));
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    mpm::launch_import_rows<D>(s->ps[s->cur], id_off, count, x, v, F, C, Jp, s->scenes_d,
                               s->slot_block, moved, s->stream);
  });
  if (moved)
    CUDA_TRY(s, cudaMemcpyAsync(s->moved_h, moved, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  else if (count_moved)
    *s->moved_h = -1;  // not counted
  if (s->acc_valid && s->stepped) s->p2g_discarded = true;
  s->acc_valid = false;  // the coming step's P2G must be recomputed from the new state
  s->replaced = true;
  if (x) s->need_sort = true;
  return check_launch(s, "import particles");
}

nclr_status export_rows(nclr_sim *s, int sc, float *x, float *v, float *F, float *C, float *Jp) {
  const int id_off = sc < 0 ? 0 : s->scenes[sc].slot_off;
  const int count = sc < 0 ? (int)s->n : s->scenes[sc].P.n;
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int D = decltype(dc)::value;
    mpm::launch_export_rows<D>(s->ps[s->cur], s->inv, id_off, count, x, v, F, C, Jp, s->stream);
  });
  return check_launch(s, "export particles");
}


nclr_status ensure_staging(nclr_sim *s) {
  if (!s->staging && s->n > 0)
    CUDA_TRY(s, cudaMalloc((void **)&s->staging, sizeof(float) * (size_t)s->n * row_floats(s->dim)));
  return NCLR_OK;
}

struct Rows {
  float *x, *v, *F, *C, *Jp;
};
Rows staging_rows(nclr_sim *s, int64_t n) {
  const int D = s->dim;
  Rows r;
  r.x = s->staging;
  r.v = r.x + n * D;
  r.F = r.v + n * D;
  r.C = r.F + n * D * D;
  r.Jp = r.C + n * D * D;
  return r;
}

// Drops the captured step graphs: they hold the kernels' parameters (scene constants,
// particle buffers) by value, so the next advance() recaptures them.
void drop_graphs(nclr_sim *s) {
  for (auto &row : s->graph)
    for (auto &g : row)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
}

void release(nclr_sim *s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->stream) cudaStreamSynchronize(s->stream);
  drop_graphs(s);
  for (auto p : s->slab) cudaFree(p);
  cudaFree(s->lame_buf);
  cudaFree(s->scenes_d);
  cudaFree(s->block_scene);
  cudaFree(s->G);
  cudaFree(s->V);
  cudaFree(s->flags);
  cudaFree(s->blocks);
  cudaFree(s->nblocks_active);
  cudaFree(s->sparse);
  cudaFree(s->bar);
  cudaFree(s->cta_scene);
  cudaFree(s->group_first);
  cudaFree(s->inv);
  cudaFree(s->slot_block);
  cudaFree(s->moved_d);
  if (s->moved_h) cudaFreeHost(s->moved_h);
  cudaFree(s->work);
  cudaFree(s->fix.count);
  cudaFree(s->fix.slot);
  cudaFree(s->fix.Fh);
  cudaFree(s->fix.Jp);
  cudaFree(s->key);
  cudaFree(s->rank);
  cudaFree(s->count);
  cudaFree(s->start);
  cudaFree(s->btotal);
  cudaFree(s->rounds);
  cudaFree(s->tile_sums);
  cudaFree(s->err_d);
  cudaFree(s->staging);
  cudaFree(s->grid_staging);
  cudaFree(s->active_d);
  for (const auto &t : s->pending) {
    cudaEventDestroy(t.a);
    cudaEventDestroy(t.b);
  }
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  if (s->err_h) cudaFreeHost(s->err_h);
  if (s->copy_stream) {
    cudaStreamSynchronize(s->copy_stream);
    cudaStreamDestroy(s->copy_stream);
  }
  for (auto e : s->field_ev)
    if (e) cudaEventDestroy(e);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

nclr_status validate_scene(const nclr_scene &sc, bool device_arrays) {
  if (sc.n < 0 || sc.n > (int64_t)0x7fffffff / 2) return fail(nullptr, NCLR_ERR_INVALID, "bad particle count");
  if (sc.n > 0 && !sc.x) return fail(nullptr, NCLR_ERR_INVALID, "x is NULL");
  if (sc.res < 1 || sc.res > 1024) return fail(nullptr, NCLR_ERR_INVALID, "res must be in [1, 1024]");
  if (sc.model < 0 || sc.model > 2) return fail(nullptr, NCLR_ERR_INVALID, "unknown material model");
  if (sc.material && !device_arrays)  // device arrays are checked on the device after the copy
    for (int64_t p = 0; p < sc.n; ++p)
      if (sc.material[p] > 2) return fail(nullptr, NCLR_ERR_INVALID, "unknown material in material[]");
  return NCLR_OK;
}

// Creates a handle of `nscenes` scenes (nclr_create is the one-scene case).  With
// device_arrays, the scenes' particle arrays are device pointers (nclr_create_device): the
// defaults are staged from the host as usual and the given arrays are copied over them on
// the device.
nclr_status create_scenes(nclr_sim **out, int dim, int nscenes, const nclr_scene *descs,
                          const nclr_options *opt, bool device_arrays = false) {
  g_create_error.clear();
  if (!out) return fail(nullptr, NCLR_ERR_INVALID, "out is NULL");
  *out = nullptr;
  if (dim != 2 && dim != 3) return fail(nullptr, NCLR_ERR_INVALID, "dim must be 2 or 3");
  if (nscenes < 1 || nscenes > 65535 || !descs) return fail(nullptr, NCLR_ERR_INVALID, "bad scene count");
  int64_t total_n = 0;
  bool any_mat = false;
  for (int i = 0; i < nscenes; ++i) {
    nclr_status st = validate_scene(descs[i], device_arrays);
    if (st != NCLR_OK) return st;
    total_n += descs[i].n;
    any_mat |= descs[i].material != nullptr;
  }
  if (total_n > (int64_t)0x7fffffff / 2) return fail(nullptr, NCLR_ERR_INVALID, "too many particles");

  nclr_sim *s = new (std::nothrow) nclr_sim();
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "out of host memory");
  nclr_default_options(&s->opt);
  if (opt) s->opt = *opt;
  if (s->opt.sort_interval < 0) s->opt.sort_interval = 0;
  if (s->opt.batch_item_threads != 0 && s->opt.batch_item_threads != 128 &&
      s->opt.batch_item_threads != 256) {
    delete s;
    return fail(nullptr, NCLR_ERR_INVALID, "batch_item_threads must be 0, 128 or 256");
  }
  if (s->opt.stress_model != NCLR_STRESS_COROTATED && s->opt.stress_model != NCLR_STRESS_NEOHOOKEAN) {
    delete s;
    return fail(nullptr, NCLR_ERR_INVALID, "unknown stress model");
  }
  if (s->opt.stress_model == NCLR_STRESS_NEOHOOKEAN && dim == 3 &&
      s->opt.physics != NCLR_PHYSICS_CORRECTED) {
    // diag<3>(1) = diag(1,1,0) (src/nclr_math.h:13-19) keeps det F at 0, where ln(J) diverges
    delete s;
    return fail(nullptr, NCLR_ERR_INVALID,
                "the neo-Hookean stress needs det F > 0: use NCLR_PHYSICS_CORRECTED in 3D");
  }
  s->dim = dim;
  s->n = total_n;
  s->nscenes = nscenes;
  s->device = s->opt.device;
  s->ref = s->opt.physics != NCLR_PHYSICS_CORRECTED;
  s->has_mat = any_mat;
  // thin blocks: a single simulation steps their particles in chunks of the sparse list; a
  // batch, whose fused kernel reads its scene per block, steps each as a tile-free item
  const int thin = s->opt.sparse_block_max >= 0 ? s->opt.sparse_block_max
                   : nscenes > 1                ? kBatchThin
                   : dim == 3                   ? kSparseMax3
                                                : kSparseMax2;
  s->sparse_max = nscenes > 1 ? 0 : thin;
  // the tail rule needs the chunks, which only single simulations have
  s->tail_max = nscenes > 1 ? 0 : s->opt.tail_max >= 0 ? s->opt.tail_max : kTailMax;
  s->deferred_err.assign((size_t)nscenes, 0);
  s->scene_err.assign((size_t)nscenes, 0);

  // scene table: slot, node and block ranges
  int64_t slot = 0, node = 0, block = 0;
  for (int i = 0; i < nscenes; ++i) {
    const nclr_scene &d = descs[i];
    Scene sc{};
    sc.P = scene_params(dim, d.n, d.model, d.res, d.dt, d.E, d.nu, d.gravity);
    sc.P.stress = s->opt.stress_model;
    sc.P.thin_max = nscenes > 1 ? thin : 0;
    sc.P.tail_max = s->tail_max;
    sc.slot_off = (int)slot;
    sc.node_off = node;
    sc.block_off = (int)std::min<int64_t>(block, 0x7fffffff);
    slot += d.n;
    node += sc.P.nodes;
    block += sc.P.nblocks;
    s->scenes.push_back(sc);
  }
  const int cpb = (dim == 3) ? mpm::Tiling<3>::CPB : mpm::Tiling<2>::CPB;
  auto bail = [&](nclr_status st) {
    g_create_error = s->error;
    release(s);
    return st;
  };
  if (node > ((int64_t)1 << 34) || block * cpb > 0x7fffffff) {
    s->error = "grids too large";
    return bail(NCLR_ERR_INVALID);
  }
  s->total_nodes = node;
  s->total_blocks = (int)block;
  s->nkeys = block * cpb;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    s->error = "no CUDA device";
    return bail(NCLR_ERR_NO_DEVICE);
  }
  if (s->device < 0 || s->device >= ndev) {
    s->error = "device ordinal out of range";
    return bail(NCLR_ERR_INVALID);
  }
  nclr_status st;
#define CREATE_TRY(call)                                                   \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) {                                               \
      s->error = std::string(#call) + ": " + cudaGetErrorString(e_);       \
      return bail(NCLR_ERR_CUDA);                                          \
    }                                                                      \
  } while (0)
  CREATE_TRY(cudaSetDevice(s->device));
  CREATE_TRY(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
  CREATE_TRY(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
  for (auto &e : s->field_ev) CREATE_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (int b = 0; b < 2; ++b)
    if ((st = alloc_particles(s, b)) != NCLR_OK) return bail(st);
  const size_t np = (size_t)std::max<int64_t>(total_n, 1);
  const size_t nblk = (size_t)block;
  const size_t nodes = (size_t)node;
  CREATE_TRY(cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device));
  s->g2p2g_ctas = s->sms * (dim == 3 ? mpm::g2p2g_ctas_per_sm<3>() : mpm::g2p2g_ctas_per_sm<2>());
  s->g2p_ctas = s->sms * (dim == 3 ? mpm::g2p_final_ctas_per_sm<3>() : mpm::g2p_final_ctas_per_sm<2>());
  {
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, s->device);
    const bool ref = s->opt.physics != NCLR_PHYSICS_CORRECTED;
    s->small_ctas = coop ? s->sms * (dim == 3 ? mpm::small_ctas_per_sm<3>(ref)
                                             : mpm::small_ctas_per_sm<2>(ref))
                         : 0;
    s->cluster_max = dim == 3 ? mpm::small_cluster_max<3>(ref, mpm::kSmallClusterThreads3D)
                              : mpm::small_cluster_max<2>(ref, mpm::kSmallClusterThreads2D);
    // batches keep the tile path unless asked: their small-scene kernel measured 2.9x slower
    // on 256 scenes of 1k-64k particles (its P2G scatters through L2 atomics)
    s->small_max = s->opt.small_scene_max >= 0 ? s->opt.small_scene_max
                   : nscenes > 1               ? 0
                   : dim == 3                  ? kSmallMax3
                                               : kSmallMax2;
    s->small_auto = s->opt.small_scene_max < 0;
    if (nscenes > 1 && coop) {
      // A batch on the small-scene kernel: each scene a group of CTAs in proportion to its
      // particles (at least one), all groups resident at once.
      const int cap = s->sms * (dim == 3 ? mpm::small_batch_ctas_per_sm<3>(ref)
                                         : mpm::small_batch_ctas_per_sm<2>(ref));
      const int64_t per = (int64_t)mpm::kSmallThreadsPerCta * std::max(1, s->opt.p2g_particles_per_thread);
      std::vector<int64_t> want((size_t)nscenes, 0);
      int64_t total = 0, busy = 0;
      for (int i = 0; i < nscenes; ++i) {
        const int64_t n = descs[i].n;
        want[(size_t)i] = n > 0 ? (n + per - 1) / per : 0;
        total += want[(size_t)i];
        busy += n > 0;
      }
      if (busy > 0 && busy <= cap) {
        std::vector<int> ctas((size_t)nscenes, 0);
        int64_t sum = 0;
        for (int i = 0; i < nscenes; ++i) {
          if (!want[(size_t)i]) continue;
          ctas[(size_t)i] = (int)std::max<int64_t>(1, total <= cap ? want[(size_t)i]
                                                                 : want[(size_t)i] * cap / total);
          sum += ctas[(size_t)i];
        }
        while (sum > cap) {  // rounding up the smallest to 1 can overshoot: trim the largest
          auto it = std::max_element(ctas.begin(), ctas.end());
          --*it;
          --sum;
        }
        std::vector<int> first((size_t)nscenes + 1, 0);
        std::vector<uint16_t> owner((size_t)sum);
        for (int i = 0; i < nscenes; ++i) {
          first[(size_t)i + 1] = first[(size_t)i] + ctas[(size_t)i];
          for (int c = first[(size_t)i]; c < first[(size_t)i + 1]; ++c) owner[(size_t)c] = (uint16_t)i;
        }
        CREATE_TRY(cudaMalloc((void **)&s->cta_scene, sizeof(uint16_t) * (size_t)sum));
        CREATE_TRY(cudaMalloc((void **)&s->group_first, sizeof(int) * first.size()));
        CREATE_TRY(cudaMemcpy(s->cta_scene, owner.data(), sizeof(uint16_t) * (size_t)sum, cudaMemcpyHostToDevice));
        CREATE_TRY(cudaMemcpy(s->group_first, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
        s->batch_ctas = (int)sum;
      }
    }
  }
  CREATE_TRY(cudaMalloc((void **)&s->scenes_d, sizeof(Scene) * (size_t)nscenes));
  CREATE_TRY(cudaMemcpyAsync(s->scenes_d, s->scenes.data(), sizeof(Scene) * (size_t)nscenes,
                             cudaMemcpyHostToDevice, s->stream));
  std::vector<uint16_t> block_scene;
  if (nscenes > 1) {
    block_scene.resize(nblk);
    for (int i = 0; i < nscenes; ++i)
      std::fill(block_scene.begin() + s->scenes[i].block_off,
                block_scene.begin() + s->scenes[i].block_off + s->scenes[i].P.nblocks, (uint16_t)i);
    CREATE_TRY(cudaMalloc((void **)&s->block_scene, sizeof(uint16_t) * nblk));
    CREATE_TRY(cudaMemcpyAsync(s->block_scene, block_scene.data(), sizeof(uint16_t) * nblk,
                               cudaMemcpyHostToDevice, s->stream));
  }
  CREATE_TRY(cudaMalloc((void **)&s->G, sizeof(float4) * nodes));
  CREATE_TRY(cudaMalloc((void **)&s->V, sizeof(float4) * nodes));
  CREATE_TRY(cudaMalloc((void **)&s->flags, nblk));
  CREATE_TRY(cudaMalloc((void **)&s->key, sizeof(int) * np));
  CREATE_TRY(cudaMalloc((void **)&s->rank, sizeof(int) * np));
  CREATE_TRY(cudaMalloc((void **)&s->count, sizeof(int) * (size_t)s->nkeys));
  CREATE_TRY(cudaMalloc((void **)&s->start, sizeof(int) * (nblk + 1)));
  CREATE_TRY(cudaMalloc((void **)&s->btotal, sizeof(int) * std::max<size_t>(nblk, 1)));
  CREATE_TRY(cudaMalloc((void **)&s->rounds, sizeof(int4) * mpm::kRoundTable * std::max<size_t>(nblk, 1)));
  CREATE_TRY(cudaMalloc((void **)&s->tile_sums, sizeof(int) * (size_t)std::max<int64_t>(mpm::scan_tiles(s->nkeys), 1)));
  CREATE_TRY(cudaMalloc((void **)&s->blocks, sizeof(int) * nblk));
  CREATE_TRY(cudaMalloc((void **)&s->nblocks_active, 4 * sizeof(int)));
  CREATE_TRY(cudaMalloc((void **)&s->sparse, sizeof(int) * (size_t)std::max<int64_t>(s->n, 1)));
  CREATE_TRY(cudaMalloc((void **)&s->bar, 2 * sizeof(unsigned) * (size_t)nscenes));
  CREATE_TRY(cudaMalloc((void **)&s->inv, sizeof(int) * (size_t)std::max<int64_t>(s->n, 1)));
  CREATE_TRY(cudaMalloc((void **)&s->slot_block, sizeof(int) * (size_t)std::max<int64_t>(s->n, 1)));
  CREATE_TRY(cudaMalloc((void **)&s->moved_d, sizeof(int)));
  CREATE_TRY(cudaMallocHost((void **)&s->moved_h, sizeof(int)));
  CREATE_TRY(cudaMalloc((void **)&s->work, sizeof(int)));
  bool snow = any_mat;  // a material[] may hold snow
  for (int i = 0; i < nscenes; ++i) snow |= descs[i].model == NCLR_SNOW;
  if (snow && np > 0) {  // the FP64 list of the snow clamp: at most one entry per particle
    s->fix.cap = (int)np;
    CREATE_TRY(cudaMalloc((void **)&s->fix.count, sizeof(int)));
    CREATE_TRY(cudaMalloc((void **)&s->fix.slot, sizeof(int) * np));
    CREATE_TRY(cudaMalloc((void **)&s->fix.Fh, sizeof(float) * np * dim * dim));
    CREATE_TRY(cudaMalloc((void **)&s->fix.Jp, sizeof(float) * np));
    CREATE_TRY(cudaMemsetAsync(s->fix.count, 0, sizeof(int), s->stream));
  }
  CREATE_TRY(cudaMalloc((void **)&s->err_d, 2 * sizeof(int) * (size_t)nscenes));
  CREATE_TRY(cudaMallocHost((void **)&s->err_h, 2 * sizeof(int) * (size_t)nscenes));
  CREATE_TRY(cudaMemsetAsync(s->err_d, 0, 2 * sizeof(int) * (size_t)nscenes, s->stream));
  CREATE_TRY(cudaMemsetAsync(s->G, 0, sizeof(float4) * nodes, s->stream));
  CREATE_TRY(cudaMemsetAsync(s->V, 0, sizeof(float4) * nodes, s->stream));
  CREATE_TRY(cudaMemsetAsync(s->flags, 0, nblk, s->stream));
  CREATE_TRY(cudaMemsetAsync(s->nblocks_active, 0, 4 * sizeof(int), s->stream));

  if (total_n > 0) {
    // Per-particle scalars go straight into the SoA (component stride == n there).
    PState &p = s->ps[0];
    std::vector<float> mass((size_t)total_n, 1.0f), vol((size_t)total_n, 1.0f);
    std::vector<int> iota((size_t)total_n);
    std::vector<uint8_t> mat(any_mat ? (size_t)total_n : 0);
    std::vector<uint16_t> pscene(nscenes > 1 ? (size_t)total_n : 0);
    std::vector<float> host((size_t)total_n * row_floats(dim), 0.0f);
    const int64_t N = total_n;
    float *hx = host.data(), *hv = hx + N * dim, *hF = hv + N * dim, *hC = hF + N * dim * dim,
          *hJ = hC + N * dim * dim;
    for (int i = 0; i < nscenes; ++i) {
      const nclr_scene &d = descs[i];
      const int64_t o = s->scenes[i].slot_off;
      const bool h = !device_arrays;  // host arrays may be read here
      for (int64_t q = 0; q < d.n; ++q) {
        iota[(size_t)(o + q)] = (int)(o + q);
        if (h && d.mass) mass[(size_t)(o + q)] = d.mass[q];
        if (h && d.volume) vol[(size_t)(o + q)] = d.volume[q];
        if (any_mat) mat[(size_t)(o + q)] = (h && d.material) ? d.material[q] : (uint8_t)d.model;
        if (nscenes > 1) pscene[(size_t)(o + q)] = (uint16_t)i;
        hJ[o + q] = (h && d.Jp) ? d.Jp[q] : 1.0f;
      }
      // Rows: x, v, F, C with the constructor's defaults for the NULL ones
      // (Particle<dim>: v = 0, F = diag<dim>(1), C = 0, Jp = 1; src/nclr.h:46-47).
      if (h && d.n > 0) std::memcpy(hx + o * dim, d.x, sizeof(float) * d.n * dim);
      if (h && d.v) std::memcpy(hv + o * dim, d.v, sizeof(float) * d.n * dim);
      if (h && d.F) {
        std::memcpy(hF + o * dim * dim, d.F, sizeof(float) * d.n * dim * dim);
      } else {
        for (int64_t q = 0; q < d.n; ++q)
          for (int k = 0; k < dim; ++k)
            hF[((o + q) * dim + k) * dim + k] = (k < 2 || !s->ref) ? 1.0f : 0.0f;
      }
      if (h && d.C) std::memcpy(hC + o * dim * dim, d.C, sizeof(float) * d.n * dim * dim);
    }
    CREATE_TRY(cudaMemcpyAsync(p.mass, mass.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s->stream));
    CREATE_TRY(cudaMemcpyAsync(p.vol, vol.data(), sizeof(float) * N, cudaMemcpyHostToDevice, s->stream));
    CREATE_TRY(cudaMemcpyAsync(p.id, iota.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s->stream));
    CREATE_TRY(cudaMemcpyAsync(s->inv, iota.data(), sizeof(int) * N, cudaMemcpyHostToDevice, s->stream));
    if (any_mat) CREATE_TRY(cudaMemcpyAsync(p.mat, mat.data(), (size_t)N, cudaMemcpyHostToDevice, s->stream));
    if (nscenes > 1)
      CREATE_TRY(cudaMemcpyAsync(p.scene, pscene.data(), sizeof(uint16_t) * N, cudaMemcpyHostToDevice, s->stream));
    if ((st = ensure_staging(s)) != NCLR_OK) return bail(st);
    const Rows r = staging_rows(s, N);
    CREATE_TRY(cudaMemcpyAsync(r.x, host.data(), sizeof(float) * host.size(), cudaMemcpyHostToDevice, s->stream));
    if (device_arrays) {  // the caller's device arrays over the staged defaults
      const auto d2d = cudaMemcpyDeviceToDevice;
      for (int i = 0; i < nscenes; ++i) {
        const nclr_scene &d = descs[i];
        const int64_t o = s->scenes[i].slot_off, q = d.n, dd = dim * dim;
        if (q == 0) continue;
        CREATE_TRY(cudaMemcpyAsync(r.x + o * dim, d.x, sizeof(float) * q * dim, d2d, s->stream));
        if (d.v) CREATE_TRY(cudaMemcpyAsync(r.v + o * dim, d.v, sizeof(float) * q * dim, d2d, s->stream));
        if (d.F) CREATE_TRY(cudaMemcpyAsync(r.F + o * dd, d.F, sizeof(float) * q * dd, d2d, s->stream));
        if (d.C) CREATE_TRY(cudaMemcpyAsync(r.C + o * dd, d.C, sizeof(float) * q * dd, d2d, s->stream));
        if (d.Jp) CREATE_TRY(cudaMemcpyAsync(r.Jp + o, d.Jp, sizeof(float) * q, d2d, s->stream));
        if (d.mass) CREATE_TRY(cudaMemcpyAsync(p.mass + o, d.mass, sizeof(float) * q, d2d, s->stream));
        if (d.volume) CREATE_TRY(cudaMemcpyAsync(p.vol + o, d.volume, sizeof(float) * q, d2d, s->stream));
        if (d.material) {
          CREATE_TRY(cudaMemcpyAsync(p.mat + o, d.material, (size_t)q, d2d, s->stream));
          int bad = 0;
          CREATE_TRY(mpm::count_bad_materials(p.mat + o, q, s->moved_d, &bad, s->stream));
          if (bad) {
            s->error = "unknown material in material[]";
            return bail(NCLR_ERR_INVALID);
          }
        }
      }
    }
    if ((st = import_rows(s, -1, r.x, r.v, r.F, r.C, r.Jp)) != NCLR_OK) return bail(st);
    CREATE_TRY(cudaStreamSynchronize(s->stream));  // the host vectors go out of scope
  }
  CREATE_TRY(cudaStreamSynchronize(s->stream));
#undef CREATE_TRY
  *out = s;
  return NCLR_OK;
}

nclr_status check_scene(nclr_sim *s, int scene) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  if (scene < 0 || scene >= s->nscenes) return fail(s, NCLR_ERR_INVALID, "scene index out of range");
  return NCLR_OK;
}

// Host copies of particle fields of scene `sc` (-1: all scenes, caller order throughout).
nclr_status get_particles_host(nclr_sim *s, int sc, float *x, float *v, float *F, float *C, float *Jp) {
  const int64_t n = sc < 0 ? s->n : s->scenes[sc].P.n;
  if (n == 0) return NCLR_OK;
  CUDA_TRY(s, cudaSetDevice(s->device));
  nclr_status st = ensure_staging(s);
  if (st != NCLR_OK) return st;
  const Rows r = staging_rows(s, n);
  const size_t nn = (size_t)n, D = (size_t)s->dim;
  float *host[5] = {x, v, F, C, Jp}, *stage[5] = {r.x, r.v, r.F, r.C, r.Jp};
  const size_t floats[5] = {nn * D, nn * D, nn * D * D, nn * D * D, nn};
  // Field by field: the copy engine downloads field k (copy stream) while the next field's
  // export kernel runs (the simulation's stream).
  for (int k = 0; k < 5; ++k) {
    if (!host[k]) continue;
    float *o[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    o[k] = stage[k];
    if ((st = export_rows(s, sc, o[0], o[1], o[2], o[3], o[4])) != NCLR_OK) return st;
    CUDA_TRY(s, cudaEventRecord(s->field_ev[k], s->stream));
    CUDA_TRY(s, cudaStreamWaitEvent(s->copy_stream, s->field_ev[k], 0));
    CUDA_TRY(s, cudaMemcpyAsync(host[k], stage[k], sizeof(float) * floats[k],
                                cudaMemcpyDeviceToHost, s->copy_stream));
  }
  CUDA_TRY(s, cudaStreamSynchronize(s->copy_stream));
  return NCLR_OK;
}

nclr_status set_particles_host(nclr_sim *s, int sc, const float *x, const float *v, const float *F,
                               const float *C, const float *Jp) {
  const int64_t n = sc < 0 ? s->n : s->scenes[sc].P.n;
  if (n == 0) return NCLR_OK;
  CUDA_TRY(s, cudaSetDevice(s->device));
  const bool had_sort = s->need_sort;
  // Staged through device memory: the copy engines move whole lines; the import kernel's
  // row accesses straight from mapped host memory measured 1.7x slower over the host link.
  nclr_status st;
  if ((st = ensure_staging(s)) != NCLR_OK) return st;
  const Rows r = staging_rows(s, n);
  const size_t nn = (size_t)n, D = (size_t)s->dim;
  const float *host[5] = {x, v, F, C, Jp};
  float *stage[5] = {r.x, r.v, r.F, r.C, r.Jp};
  const size_t floats[5] = {nn * D, nn * D, nn * D * D, nn * D * D, nn};
  // Field by field: the copy engine uploads field k+1 (copy stream) while field k's import
  // kernel runs (the simulation's stream); the copies start after the stream's earlier work.
  CUDA_TRY(s, cudaEventRecord(s->field_ev[0], s->stream));
  CUDA_TRY(s, cudaStreamWaitEvent(s->copy_stream, s->field_ev[0], 0));
  for (int k = 0; k < 5; ++k) {
    if (!host[k]) continue;
    CUDA_TRY(s, cudaMemcpyAsync(stage[k], host[k], sizeof(float) * floats[k],
                                cudaMemcpyHostToDevice, s->copy_stream));
    CUDA_TRY(s, cudaEventRecord(s->field_ev[k], s->copy_stream));
    CUDA_TRY(s, cudaStreamWaitEvent(s->stream, s->field_ev[k], 0));
    const float *in[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
    in[k] = stage[k];
    if ((st = import_rows(s, sc, in[0], in[1], in[2], in[3], in[4], k == 0)) != NCLR_OK) return st;
  }
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));  // the caller may reuse its buffers
  // New positions that all stayed in their slots' grid blocks leave the block lists valid:
  // no forced re-sort (the regular interval still applies).
  if (x && !had_sort && *s->moved_h == 0) s->need_sort = false;
  return NCLR_OK;
}

nclr_status get_grid_host(nclr_sim *s, int sc, float *velocity, float *mass) {
  if (!s->stepped) return fail(s, NCLR_ERR_INVALID, "grid() is empty before the first advance()");
  CUDA_TRY(s, cudaSetDevice(s->device));
  const Scene &S = s->scenes[sc];
  const size_t nodes = (size_t)S.P.nodes, D = (size_t)s->dim;
  if (!s->grid_staging) {
    size_t mx = 0;
    for (const auto &x : s->scenes) mx = std::max(mx, (size_t)x.P.nodes);
    CUDA_TRY(s, cudaMalloc((void **)&s->grid_staging, sizeof(float) * mx * (D + 1)));
  }
  float *dv = s->grid_staging, *dm = dv + nodes * D;
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    mpm::launch_copy_vgrid<DD>(s->V + S.node_off, S.P.nodes, dv, dm, s->stream);
  });
  nclr_status st = check_launch(s, "export grid");
  if (st != NCLR_OK) return st;
  if (velocity) CUDA_TRY(s, cudaMemcpyAsync(velocity, dv, sizeof(float) * nodes * D, cudaMemcpyDeviceToHost, s->stream));
  if (mass) CUDA_TRY(s, cudaMemcpyAsync(mass, dm, sizeof(float) * nodes, cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return NCLR_OK;
}

// The steps of nclr_advance on the regular path: block sort, fused G2P2G, graphs.
nclr_status advance_regular(nclr_sim *s, int64_t nsteps) {
  // the last call ended without its P2G but nothing replaced the state since: stop guessing
  if (!s->acc_valid && !s->replaced && s->stepped) s->p2g_discarded = false;
  s->replaced = false;
  const int last = (s->p2g_discarded && s->nscenes == 1) ? kFinalG2POnly : kFinalWithP2G;
  if (s->need_sort && s->n > 0) {  // the uploaded particles: sort them (with v and C) first
    enqueue_sort(s, !s->acc_valid);
    s->need_sort = false;
    s->steps_since_sort = 0;
  }
  if (!s->acc_valid) enqueue_pending_p2g(s);  // the first step's P2G, from the uploaded state
  int64_t left = nsteps;
  const int64_t chunk = chunk_steps(s);
  while (left > 0) {
    const bool sort = sort_due(s);
    const bool at_boundary = s->opt.sort_interval == 0 || sort;
    if (s->opt.use_graphs && !s->opt.profile && s->n > 0 && at_boundary && left >= chunk) {
      const int fin = (left == chunk) ? last : kNotFinal;
      if (!s->graph[s->cur][fin]) {
        nclr_status st = capture_graph(s, s->cur, fin);
        if (st != NCLR_OK) return st;
      }
      CUDA_TRY(s, cudaGraphLaunch(s->graph[s->cur][fin], s->stream));
      s->launches += s->graph_launches;
      if (chunk_sorts(s) & 1) s->cur ^= 1;
      if (s->opt.sort_interval > 0) s->steps_since_sort = s->opt.sort_interval;
      left -= chunk;
      continue;
    }
    enqueue_step(s, sort, left == 1 ? last : kNotFinal);
    if (sort) s->steps_since_sort = 0;
    ++s->steps_since_sort;
    --left;
  }
  if (last == kFinalG2POnly && s->n > 0) s->acc_valid = false;  // G holds no pending P2G
  return NCLR_OK;
}

// The steps of nclr_advance for a small scene: one cooperative launch per 2^30 steps.
nclr_status advance_small(nclr_sim *s, int64_t nsteps) {
  const bool batch = s->nscenes > 1;
  const int64_t per_cta = (int64_t)mpm::kSmallThreadsPerCta * std::max(1, s->opt.p2g_particles_per_thread);
  const int ctas = batch ? s->batch_ctas
                         : (int)std::min<int64_t>((s->n + per_cta - 1) / per_cta, s->small_ctas);
  std::fill(s->deferred_err.begin(), s->deferred_err.end(), 0);  // a pending P2G is redone
  if (s->acc_valid) {  // drop the regular path's pending P2G: the kernel starts with its own
    if (batch) {
      dispatch_dim(s->dim, [&](auto dc) {
        constexpr int D = decltype(dc)::value;
        mpm::launch_discard_pending<D>(s->G, s->flags, s->scenes_d, s->block_scene,
                                       s->total_blocks, s->sms, s->stream);
      });
    } else {
      CUDA_TRY(s, cudaMemsetAsync(s->G, 0, sizeof(float4) * (size_t)s->total_nodes, s->stream));
    }
  }
  // A single scene that fits one thread-block cluster runs as one: the step's two barriers are
  // then the cluster's hardware barrier instead of an atomic and a poll in L2 (the barrier
  // test hook keeps the bounded grid barrier, which is what it tests).
  int cl_ctas = 0, cl_threads = 0;
  if (!batch && s->cluster_max > 0 && s->bar_test.extra == 0) {
    const int tmax = s->dim == 3 ? mpm::kSmallClusterThreads3D : mpm::kSmallClusterThreads2D;
    const int64_t ppt = std::max(1, s->opt.p2g_particles_per_thread);
    const int64_t c = std::min<int64_t>(s->cluster_max, std::max<int64_t>(1, ctas));
    const int64_t t = ((s->n + c * ppt - 1) / (c * ppt) + 31) / 32 * 32;
    if (t <= tmax) {
      cl_ctas = (int)c;
      cl_threads = (int)t;
    }
  }
  for (int64_t left = nsteps; left > 0;) {
    const int k = (int)std::min<int64_t>(left, (int64_t)1 << 30);
    CUDA_TRY(s, cudaMemsetAsync(s->bar, 0, 2 * sizeof(unsigned) * (size_t)s->nscenes, s->stream));
    cudaError_t e = cudaSuccess;
    dispatch_dim(s->dim, [&](auto dc) {
      constexpr int D = decltype(dc)::value;
      phase(s, NCLR_PHASE_G2P2G, 1, [&] {
        if (cl_ctas > 0) {
          e = mpm::launch_small_cluster<D>(s->ps[s->cur], s->P0(), s->G, s->V, k, s->err_d,
                                           s->bar, s->ref, cl_ctas, cl_threads, s->stream);
          if (e == cudaSuccess) return;
          cudaGetLastError();  // no cluster of that size now: the cooperative launch below
          cl_ctas = 0;
        }
        e = batch ? mpm::launch_small_batch<D>(s->ps[s->cur], s->scenes_d, s->cta_scene,
                                               s->group_first, s->G, s->V, s->flags, k, s->err_d,
                                               s->bar, s->ref, ctas, s->stream, s->bar_test)
                  : mpm::launch_small_steps<D>(s->ps[s->cur], s->P0(), s->G, s->V, k, s->err_d,
                                               s->bar, s->ref, ctas, s->stream, s->bar_test);
      });
    });
    if (e != cudaSuccess) return fail(s, NCLR_ERR_CUDA, std::string("small-scene launch: ") + cudaGetErrorString(e));
    s->launches += 1;
    left -= k;
  }
  s->acc_valid = false;  // G is clear: the regular path recomputes its P2G if it takes over
  // one scene: V was rewritten everywhere, so the next regular sweep visits every block (a
  // batch's kernel kept the flags itself)
  if (!batch)
    CUDA_TRY(s, cudaMemsetAsync(s->flags, mpm::kFlagVNonzeroBit, (size_t)s->total_blocks, s->stream));
  return NCLR_OK;
}

bool small_scene(const nclr_sim *s) {
  if (s->n <= 0 || s->small_ctas <= 0) return false;
  if (s->nscenes == 1)
    return s->n <= s->small_max &&
           (!s->small_auto || s->P0().nodes <= kSmallNodesPerParticle * s->n);
  if (s->batch_ctas <= 0) return false;
  for (const auto &sc : s->scenes)
    if (sc.P.n > s->small_max) return false;
  return true;
}

}  // namespace

extern "C" {

void nclr_default_options(nclr_options *opt) {
  if (!opt) return;
  opt->physics = NCLR_PHYSICS_REFERENCE;
  opt->sort_interval = 8;
  opt->p2g_particles_per_thread = 1;
  opt->device = 0;
  opt->use_graphs = 1;
  opt->profile = 0;
  opt->batch_item_threads = 0;
  opt->graph_steps = 0;
  opt->sparse_block_max = -1;
  opt->small_scene_max = -1;
  opt->tail_max = -1;
  opt->stress_model = NCLR_STRESS_COROTATED;
}

nclr_status nclr_create(nclr_sim **out, int dim, int64_t n, const float *x, const float *v,
                        const float *F, const float *C, const float *Jp, const float *mass,
                        const float *volume, const uint8_t *material, int model, int res,
                        float dt, float E, float nu, float gravity, const nclr_options *opt) {
  nclr_scene d{};
  d.n = n;
  d.x = x;
  d.v = v;
  d.F = F;
  d.C = C;
  d.Jp = Jp;
  d.mass = mass;
  d.volume = volume;
  d.material = material;
  d.model = model;
  d.res = res;
  d.dt = dt;
  d.E = E;
  d.nu = nu;
  d.gravity = gravity;
  return create_scenes(out, dim, 1, &d, opt);
}

nclr_status nclr_create_device(nclr_sim **out, int dim, int64_t n, const float *x, const float *v,
                               const float *F, const float *C, const float *Jp, const float *mass,
                               const float *volume, const uint8_t *material, int model, int res,
                               float dt, float E, float nu, float gravity,
                               const nclr_options *opt) {
  nclr_scene d{};
  d.n = n;
  d.x = x;
  d.v = v;
  d.F = F;
  d.C = C;
  d.Jp = Jp;
  d.mass = mass;
  d.volume = volume;
  d.material = material;
  d.model = model;
  d.res = res;
  d.dt = dt;
  d.E = E;
  d.nu = nu;
  d.gravity = gravity;
  return create_scenes(out, dim, 1, &d, opt, true);
}

nclr_status nclr_batch_create(nclr_sim **out, int dim, int nscenes, const nclr_scene *scenes,
                              const nclr_options *opt) {
  return create_scenes(out, dim, nscenes, scenes, opt);
}

nclr_status nclr_advance(nclr_sim *s, int64_t nsteps) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  if (nsteps < 0) return fail(s, NCLR_ERR_INVALID, "nsteps < 0");
  if (nsteps == 0) return NCLR_OK;
  CUDA_TRY(s, cudaSetDevice(s->device));
  CUDA_TRY(s, cudaMemsetAsync(s->err_d, 0, 2 * sizeof(int) * (size_t)s->nscenes, s->stream));
  s->launches = 0;
  const nclr_status path = small_scene(s) ? advance_small(s, nsteps) : advance_regular(s, nsteps);
  if (path != NCLR_OK) return path;
  nclr_status st = check_launch(s, "advance");
  if (st != NCLR_OK) return st;
  s->stepped = true;
  CUDA_TRY(s, cudaMemcpyAsync(s->err_h, s->err_d, 2 * sizeof(int) * (size_t)s->nscenes,
                              cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  collect_profile(s);
  int first = -1;
  for (int i = 0; i < s->nscenes; ++i) {
    const int e = s->err_h[2 * i] | s->deferred_err[(size_t)i];
    s->deferred_err[(size_t)i] = s->err_h[2 * i + 1];
    s->scene_err[(size_t)i] = (e & mpm::kErrOutOfRange) ? NCLR_ERR_OUT_OF_RANGE : NCLR_OK;
    if ((e & mpm::kErrOutOfRange) && first < 0) first = i;
  }
  for (int i = 0; i < s->nscenes; ++i)
    if (s->err_h[2 * i] & mpm::kErrBarrier) {
      // Every CTA left the launch at the barrier that ran out: the accumulator may hold a
      // partial P2G, so clear it (the next call starts a fresh P2G); the particle state is that
      // of a step left half done, for the caller to replace.
      CUDA_TRY(s, cudaMemsetAsync(s->G, 0, sizeof(float4) * (size_t)s->total_nodes, s->stream));
      CUDA_TRY(s, cudaMemsetAsync(s->flags, mpm::kFlagVNonzeroBit, (size_t)s->total_blocks, s->stream));
      CUDA_TRY(s, cudaStreamSynchronize(s->stream));
      s->acc_valid = false;
      return fail(s, NCLR_ERR_CUDA, "the small-scene kernel's grid barrier ran out of time");
    }
  if (first >= 0)
    return fail(s, NCLR_ERR_OUT_OF_RANGE,
                "a particle's stencil left the grid (the reference's vector::at throws "
                "std::out_of_range here)" +
                    (s->nscenes > 1 ? std::string(" in scene ") + std::to_string(first) : ""));
  return NCLR_OK;
}

nclr_status nclr_get_particles_device(nclr_sim *s, float *x, float *v, float *F, float *C,
                                      float *Jp) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  CUDA_TRY(s, cudaSetDevice(s->device));
  return export_rows(s, -1, x, v, F, C, Jp);
}

nclr_status nclr_set_particles_device(nclr_sim *s, const float *x, const float *v,
                                      const float *F, const float *C, const float *Jp) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  CUDA_TRY(s, cudaSetDevice(s->device));
  if (s->n == 0) return NCLR_OK;
  return import_rows(s, -1, x, v, F, C, Jp);
}

// Per-particle moduli: E, nu in the caller's row order (host arrays staged first, or device
// arrays), turned into (mu_0, lambda_0) per slot; both NULL returns to the scenes' pairs.
static nclr_status set_moduli(nclr_sim *s, const float *E, const float *nu, bool device) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  if ((!E) != (!nu)) return fail(s, NCLR_ERR_INVALID, "E and nu go together");
  CUDA_TRY(s, cudaSetDevice(s->device));
  if (!E) {
    if (s->lame_buf) {
      CUDA_TRY(s, cudaStreamSynchronize(s->stream));
      cudaFree(s->lame_buf);
      s->lame_buf = nullptr;
      s->ps[0].lame = s->ps[1].lame = nullptr;
      drop_graphs(s);
      s->acc_valid = false;
    }
    return NCLR_OK;
  }
  if (s->n == 0) return NCLR_OK;
  if (!s->lame_buf) {
    CUDA_TRY(s, cudaMalloc((void **)&s->lame_buf, sizeof(float2) * 2 * (size_t)s->n));
    s->ps[0].lame = s->lame_buf;
    s->ps[1].lame = s->lame_buf + s->n;
    drop_graphs(s);  // the captured kernels hold the particle buffers without it
  }
  const float *Ed = E, *nud = nu;
  if (!device) {
    const nclr_status st = ensure_staging(s);
    if (st != NCLR_OK) return st;
    const size_t bytes = sizeof(float) * (size_t)s->n;
    CUDA_TRY(s, cudaMemcpyAsync(s->staging, E, bytes, cudaMemcpyHostToDevice, s->stream));
    CUDA_TRY(s, cudaMemcpyAsync(s->staging + s->n, nu, bytes, cudaMemcpyHostToDevice, s->stream));
    Ed = s->staging;
    nud = s->staging + s->n;
  }
  CUDA_TRY(s, mpm::launch_set_lame(s->ps[s->cur].id, (int)s->n, Ed, nud, s->ps[s->cur].lame,
                                   s->stream));
  if (s->acc_valid && s->stepped) s->p2g_discarded = true;
  s->acc_valid = false;  // the pending P2G used the old moduli
  s->replaced = true;
  if (!device) CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  return NCLR_OK;
}

nclr_status nclr_set_moduli(nclr_sim *s, const float *E, const float *nu) {
  return set_moduli(s, E, nu, false);
}

nclr_status nclr_set_moduli_device(nclr_sim *s, const float *E, const float *nu) {
  return set_moduli(s, E, nu, true);
}

nclr_status nclr_get_particles(nclr_sim *s, float *x, float *v, float *F, float *C, float *Jp) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  return get_particles_host(s, -1, x, v, F, C, Jp);
}

nclr_status nclr_set_particles(nclr_sim *s, const float *x, const float *v, const float *F,
                               const float *C, const float *Jp) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  return set_particles_host(s, -1, x, v, F, C, Jp);
}

nclr_status nclr_get_grid(nclr_sim *s, float *velocity, float *mass) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  return get_grid_host(s, 0, velocity, mass);
}

nclr_status nclr_get_grid_device(nclr_sim *s, float *velocity, float *mass) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  if (!s->stepped) return fail(s, NCLR_ERR_INVALID, "grid() is empty before the first advance()");
  CUDA_TRY(s, cudaSetDevice(s->device));
  const Scene &S = s->scenes[0];
  const size_t nodes = (size_t)S.P.nodes, D = (size_t)s->dim;
  if (!velocity || !mass) {  // the kernel writes both: stage what the caller does not want
    if (!s->grid_staging)
      CUDA_TRY(s, cudaMalloc((void **)&s->grid_staging, sizeof(float) * nodes * (D + 1)));
    if (!velocity) velocity = s->grid_staging;
    if (!mass) mass = s->grid_staging + nodes * D;
  }
  dispatch_dim(s->dim, [&](auto dc) {
    constexpr int DD = decltype(dc)::value;
    mpm::launch_copy_vgrid<DD>(s->V + S.node_off, S.P.nodes, velocity, mass, s->stream);
  });
  return check_launch(s, "export grid");
}

int nclr_num_scenes(const nclr_sim *s) { return s ? s->nscenes : -1; }

nclr_status nclr_scene_get_particles(nclr_sim *s, int scene, float *x, float *v, float *F,
                                     float *C, float *Jp) {
  nclr_status st = check_scene(s, scene);
  if (st != NCLR_OK) return st;
  s->error.clear();
  return get_particles_host(s, scene, x, v, F, C, Jp);
}

nclr_status nclr_scene_set_particles(nclr_sim *s, int scene, const float *x, const float *v,
                                     const float *F, const float *C, const float *Jp) {
  nclr_status st = check_scene(s, scene);
  if (st != NCLR_OK) return st;
  s->error.clear();
  return set_particles_host(s, scene, x, v, F, C, Jp);
}

nclr_status nclr_scene_get_grid(nclr_sim *s, int scene, float *velocity, float *mass) {
  nclr_status st = check_scene(s, scene);
  if (st != NCLR_OK) return st;
  s->error.clear();
  return get_grid_host(s, scene, velocity, mass);
}

nclr_status nclr_scene_status(const nclr_sim *s, int scene) {
  if (!s || scene < 0 || scene >= s->nscenes) return NCLR_ERR_INVALID;
  return (nclr_status)s->scene_err[(size_t)scene];
}

nclr_status nclr_get_lame(const nclr_sim *s, float *mu_0, float *lambda_0) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  if (mu_0) *mu_0 = s->P0().mu0;
  if (lambda_0) *lambda_0 = s->P0().lambda0;
  return NCLR_OK;
}

int64_t nclr_num_particles(const nclr_sim *s) { return s ? s->n : -1; }
int nclr_dim(const nclr_sim *s) { return s ? s->dim : -1; }
int nclr_res(const nclr_sim *s) { return s ? s->P0().res : -1; }
int64_t nclr_num_nodes(const nclr_sim *s) { return s ? s->P0().nodes : -1; }
void *nclr_stream(nclr_sim *s) { return s ? (void *)s->stream : nullptr; }

nclr_status nclr_stats(const nclr_sim *s, int64_t *kernel_launches, int64_t *active_nodes) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  if (kernel_launches) *kernel_launches = s->launches;
  if (active_nodes) *active_nodes = s->active_nodes;
  return NCLR_OK;
}

nclr_status nclr_count_active_nodes(nclr_sim *s, int64_t *active_nodes) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->error.clear();
  CUDA_TRY(s, cudaSetDevice(s->device));
  if (!s->active_d) CUDA_TRY(s, cudaMalloc((void **)&s->active_d, sizeof(unsigned long long)));
  CUDA_TRY(s, cudaMemsetAsync(s->active_d, 0, sizeof(unsigned long long), s->stream));
  mpm::launch_count_active(s->V, s->total_nodes, s->active_d, s->stream);
  nclr_status st = check_launch(s, "count active nodes");
  if (st != NCLR_OK) return st;
  unsigned long long h = 0;
  CUDA_TRY(s, cudaMemcpyAsync(&h, s->active_d, sizeof(h), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(s, cudaStreamSynchronize(s->stream));
  s->active_nodes = (int64_t)h;
  if (active_nodes) *active_nodes = s->active_nodes;
  return NCLR_OK;
}

nclr_status nclr_profile_get(const nclr_sim *s, int which, double *total_ms, int64_t *launches) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  if (which < 0 || which >= NCLR_NUM_PHASES) return NCLR_ERR_INVALID;
  if (total_ms) *total_ms = s->prof_ms[which];
  if (launches) *launches = s->prof_launches[which];
  return NCLR_OK;
}

nclr_status nclr_debug_set_barrier(nclr_sim *s, unsigned extra_arrivals, unsigned spin_limit) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  s->bar_test.extra = extra_arrivals;
  s->bar_test.spins = spin_limit ? spin_limit : mpm::kBarrierSpinsDefault;
  drop_graphs(s);  // captured launches hold the old barrier arguments
  return NCLR_OK;
}

nclr_status nclr_profile_reset(nclr_sim *s) {
  if (!s) return fail(nullptr, NCLR_ERR_INVALID, "sim is NULL");
  for (int i = 0; i < NCLR_NUM_PHASES; ++i) {
    s->prof_ms[i] = 0.0;
    s->prof_launches[i] = 0;
  }
  return NCLR_OK;
}

const char *nclr_last_error(const nclr_sim *s) {
  return s ? s->error.c_str() : g_create_error.c_str();
}

void nclr_destroy(nclr_sim *s) { release(s); }

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Differentiable rollouts: nsteps jelly steps from a given state, keeping a checkpoint every
// `every` steps; the reverse pass recomputes each segment's states and grids forward (the
// regular step kernels) and runs the adjoint kernels (adjoint.cu) backwards through it.  The
// segment records are double-buffered: the recomputation of segment k-1 (the simulation's
// stream) runs while the adjoint of segment k (the rollout's reverse stream) consumes the
// other buffer; events order each buffer's writer and reader.
// ---------------------------------------------------------------------------------------
struct nclr_rollout {
  nclr_sim *sim = nullptr;
  int dim = 0;
  int model = NCLR_JELLY;
  int64_t n = 0, nsteps = 0, nodes = 0;
  int every = 0, nseg = 0;
  float E = 0.0f, nu = 0.0f;
  size_t rowf = 0;            // floats of one state: x, v, F, C rows, then Jp
  float *ckpt = nullptr;      // nseg states
  float *seg[2] = {nullptr, nullptr};     // every + 1 states of a recorded segment
  float4 *grids[2] = {nullptr, nullptr};  // `every` updated grids of that segment
  cudaStream_t rev = nullptr;             // the adjoint steps
  cudaEvent_t recorded[2] = {nullptr, nullptr}, reversed[2] = {nullptr, nullptr};
  float *adj[2] = {nullptr, nullptr};
  float *VB = nullptr;
  float4 *GB = nullptr;
  double *gml = nullptr;      // adjoints of mu_0, lambda_0
  // per-particle moduli of the last forward (nclr_rollout_forward_moduli): E and nu per row,
  // each row's (mu_0, lambda_0), and each row's accumulated mu_0 / lambda_0 adjoints
  bool per_particle = false;
  float *mod_E = nullptr, *mod_nu = nullptr;
  float2 *lame_rows = nullptr;
  double *grad_rows = nullptr;
  int *err = nullptr;
  float *mass = nullptr, *vol = nullptr, *ones = nullptr;
  bool have_forward = false;
  cudaEvent_t ev[2] = {nullptr, nullptr};
  float fwd_ms = 0.0f, bwd_ms = 0.0f;
  // profiling (the simulation's opt.profile): four events per reverse step, folded into the
  // simulation's phase totals once the backward has drained
  std::vector<cudaEvent_t> rev_events;
  std::string error;

  float *x(float *st) const { return st; }
  float *v(float *st) const { return st + n * dim; }
  float *F(float *st) const { return st + 2 * n * dim; }
  float *C(float *st) const { return st + 2 * n * dim + n * dim * dim; }
  float *Jp(float *st) const { return st + 2 * n * dim + 2 * n * dim * dim; }
  float *state(float *base, int64_t i) const { return base + (size_t)i * rowf; }
};

namespace {

nclr_status rfail(nclr_rollout *r, nclr_status st, const std::string &m) {
  if (r) r->error = m;
  return st;
}

#define R_TRY(r, call)                                                                      \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess)                                                                  \
      return rfail((r), NCLR_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

#define R_SIM(r, call)                                                     \
  do {                                                                     \
    nclr_status st_ = (call);                                              \
    if (st_ != NCLR_OK) return rfail((r), st_, nclr_last_error((r)->sim)); \
  } while (0)

void rollout_release(nclr_rollout *r) {
  if (!r) return;
  if (r->sim) {
    cudaSetDevice(r->sim->device);
    cudaStreamSynchronize(r->sim->stream);
  }
  if (r->rev) cudaStreamSynchronize(r->rev);
  cudaFree(r->ckpt);
  for (int b = 0; b < 2; ++b) {
    cudaFree(r->seg[b]);
    cudaFree(r->grids[b]);
    if (r->recorded[b]) cudaEventDestroy(r->recorded[b]);
    if (r->reversed[b]) cudaEventDestroy(r->reversed[b]);
  }
  if (r->rev) cudaStreamDestroy(r->rev);
  cudaFree(r->adj[0]);
  cudaFree(r->adj[1]);
  cudaFree(r->VB);
  cudaFree(r->GB);
  cudaFree(r->gml);
  cudaFree(r->mod_E);
  cudaFree(r->mod_nu);
  cudaFree(r->lame_rows);
  cudaFree(r->grad_rows);
  cudaFree(r->err);
  cudaFree(r->mass);
  cudaFree(r->vol);
  cudaFree(r->ones);
  for (auto e : r->ev)
    if (e) cudaEventDestroy(e);
  for (auto e : r->rev_events) cudaEventDestroy(e);
  if (r->sim) nclr_destroy(r->sim);
  delete r;
}

// New Young's modulus / Poisson ratio for the (single) scene: host and device tables; the
// captured graphs hold the old parameters and are dropped.
void set_material(nclr_sim *s, float E, float nu) {
  Params &P = s->scenes[0].P;
  P.mu0 = E / (2.0f * (1.0f + nu));
  P.lambda0 = E * nu / ((1.0f + nu) * (1.0f - 2.0f * nu));
  cudaMemcpyAsync(s->scenes_d, s->scenes.data(), sizeof(Scene), cudaMemcpyHostToDevice, s->stream);
  drop_graphs(s);
}

// Loads a state (rows) into the simulation; the next advance() starts from it.
nclr_status load_state(nclr_rollout *r, float *st) {
  R_SIM(r, nclr_set_particles_device(r->sim, r->x(st), r->v(st), r->F(st), r->C(st), r->Jp(st)));
  return NCLR_OK;
}

nclr_status save_state(nclr_rollout *r, float *st) {
  R_SIM(r, nclr_get_particles_device(r->sim, r->x(st), r->v(st), r->F(st), r->C(st), r->Jp(st)));
  return NCLR_OK;
}

// Enqueues L steps of the simulation from the loaded state, recording after step i the state
// (into r->seg[buf] state i + 1, caller order, written by the fused kernel) and the step's
// updated grid (r->grids[buf][i]).  Every step writes v and C (they are part of the record).
// No synchronisation: stencil errors accumulate in the simulation's flags, which the caller
// cleared and reads once at the end.
nclr_status record_segment(nclr_rollout *r, int L, int buf) {
  nclr_sim *s = r->sim;
  if (s->need_sort) {
    enqueue_sort(s, !s->acc_valid);
    s->need_sort = false;
    s->steps_since_sort = 0;
  }
  if (!s->acc_valid) enqueue_pending_p2g(s);
  for (int i = 0; i < L; ++i) {
    const bool sort = sort_due(s);
    float *st = r->state(r->seg[buf], i + 1);
    s->record = mpm::Record{r->x(st), r->v(st), r->F(st), r->C(st), r->Jp(st)};  // by the step
    enqueue_step(s, sort, kFinalWithP2G);
    s->record = mpm::Record{};
    if (sort) s->steps_since_sort = 0;
    ++s->steps_since_sort;
    R_TRY(r, cudaMemcpyAsync(r->grids[buf] + (size_t)i * r->nodes, s->V,
                             sizeof(float4) * (size_t)r->nodes, cudaMemcpyDeviceToDevice,
                             s->stream));
  }
  s->stepped = true;
  const nclr_status st = check_launch(s, "segment recomputation");
  return st == NCLR_OK ? st : rfail(r, st, s->error);
}

}  // namespace

extern "C" {

nclr_status nclr_rollout_create(nclr_rollout **out, int dim, int64_t n, const float *x0,
                                const float *mass, const float *volume, int res, float dt,
                                float gravity, int64_t nsteps, int checkpoint_every,
                                const nclr_options *opt) {
  return nclr_rollout_create_model(out, dim, n, x0, mass, volume, NCLR_JELLY, res, dt, gravity,
                                   nsteps, checkpoint_every, opt);
}

nclr_status nclr_rollout_create_model(nclr_rollout **out, int dim, int64_t n, const float *x0,
                                      const float *mass, const float *volume, int model, int res,
                                      float dt, float gravity, int64_t nsteps,
                                      int checkpoint_every, const nclr_options *opt) {
  if (!out) return NCLR_ERR_INVALID;
  *out = nullptr;
  g_create_error.clear();
  if (model < NCLR_SNOW || model > NCLR_LIQUID) return fail(nullptr, NCLR_ERR_INVALID, "unknown material model");
  if (nsteps < 1 || checkpoint_every < 1) return fail(nullptr, NCLR_ERR_INVALID, "nsteps and checkpoint_every must be >= 1");
  if (n < 1 || !x0) return fail(nullptr, NCLR_ERR_INVALID, "a rollout needs particles");
  nclr_rollout *r = new (std::nothrow) nclr_rollout();
  if (!r) return fail(nullptr, NCLR_ERR_INVALID, "out of host memory");
  nclr_status st = nclr_create(&r->sim, dim, n, x0, nullptr, nullptr, nullptr, nullptr, mass, volume,
                               nullptr, model, res, dt, 1e4f, 0.2f, gravity, opt);
  if (st != NCLR_OK) {
    delete r;
    return st;
  }
  nclr_sim *s = r->sim;
  r->dim = dim;
  r->model = model;
  r->n = n;
  r->nsteps = nsteps;
  r->every = (int)std::min<int64_t>(checkpoint_every, nsteps);
  r->nseg = (int)((nsteps + r->every - 1) / r->every);
  r->nodes = s->P0().nodes;
  r->rowf = (size_t)n * (2 * dim + 2 * dim * dim + 1);
  auto bail = [&](const std::string &m) {
    g_create_error = m;
    rollout_release(r);
    return NCLR_ERR_CUDA;
  };
#define RC(call)                                                                          \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess) return bail(std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)
  RC(cudaSetDevice(s->device));
  RC(cudaMalloc((void **)&r->ckpt, sizeof(float) * r->rowf * (size_t)r->nseg));
  for (int b = 0; b < 2; ++b) {
    RC(cudaMalloc((void **)&r->seg[b], sizeof(float) * r->rowf * (size_t)(r->every + 1)));
    RC(cudaMalloc((void **)&r->grids[b], sizeof(float4) * (size_t)r->nodes * (size_t)r->every));
    RC(cudaEventCreateWithFlags(&r->recorded[b], cudaEventDisableTiming));
    RC(cudaEventCreateWithFlags(&r->reversed[b], cudaEventDisableTiming));
  }
  RC(cudaStreamCreateWithFlags(&r->rev, cudaStreamNonBlocking));
  for (auto &a : r->adj) RC(cudaMalloc((void **)&a, sizeof(float) * r->rowf));
  RC(cudaMalloc((void **)&r->VB, sizeof(float4) * (size_t)r->nodes));
  RC(cudaMalloc((void **)&r->GB, sizeof(float4) * (size_t)r->nodes));
  RC(cudaMalloc((void **)&r->gml, 2 * sizeof(double)));
  RC(cudaMalloc((void **)&r->err, sizeof(int)));
  RC(cudaMalloc((void **)&r->mass, sizeof(float) * (size_t)n));
  RC(cudaMalloc((void **)&r->vol, sizeof(float) * (size_t)n));
  RC(cudaMalloc((void **)&r->ones, sizeof(float) * (size_t)n));
  std::vector<float> ones((size_t)n, 1.0f);
  RC(cudaMemcpy(r->mass, mass ? mass : ones.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  RC(cudaMemcpy(r->vol, volume ? volume : ones.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  RC(cudaMemcpy(r->ones, ones.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
  RC(cudaMemset(r->VB, 0, sizeof(float4) * (size_t)r->nodes));
  for (auto &e : r->ev) RC(cudaEventCreate(&e));
#undef RC
  *out = r;
  return NCLR_OK;
}

// The forward of both entry points: the scene's E and nu, or (Ep, nup: device arrays, one per
// row) every particle's own.
static nclr_status rollout_forward(nclr_rollout *r, const float *x0, const float *v0,
                                   const float *F0, const float *C0, float E, float nu,
                                   const float *Ep, const float *nup, float *xT, float *vT,
                                   float *FT, float *CT) {
  if (!r || !x0 || !v0 || !F0 || !C0) return rfail(r, NCLR_ERR_INVALID, "NULL argument");
  nclr_sim *s = r->sim;
  R_TRY(r, cudaSetDevice(s->device));
  r->have_forward = false;
  if (Ep) {
    const size_t row = sizeof(float) * (size_t)r->n;
    if (!r->mod_E) {
      R_TRY(r, cudaMalloc((void **)&r->mod_E, row));
      R_TRY(r, cudaMalloc((void **)&r->mod_nu, row));
      R_TRY(r, cudaMalloc((void **)&r->lame_rows, sizeof(float2) * (size_t)r->n));
      R_TRY(r, cudaMalloc((void **)&r->grad_rows, 2 * sizeof(double) * (size_t)r->n));
    }
    R_TRY(r, cudaMemcpyAsync(r->mod_E, Ep, row, cudaMemcpyDeviceToDevice, s->stream));
    R_TRY(r, cudaMemcpyAsync(r->mod_nu, nup, row, cudaMemcpyDeviceToDevice, s->stream));
    R_TRY(r, mpm::launch_set_lame(nullptr, (int)r->n, r->mod_E, r->mod_nu, r->lame_rows, s->stream));
    R_SIM(r, nclr_set_moduli_device(s, r->mod_E, r->mod_nu));
    r->per_particle = true;
  } else {
    if (r->per_particle) R_SIM(r, nclr_set_moduli(s, nullptr, nullptr));
    r->per_particle = false;
    r->E = E;
    r->nu = nu;
    set_material(s, E, nu);
  }
  float *c0 = r->state(r->ckpt, 0);
  const size_t vec = sizeof(float) * (size_t)r->n * r->dim, mat = vec * r->dim;
  R_TRY(r, cudaMemcpyAsync(r->x(c0), x0, vec, cudaMemcpyDeviceToDevice, s->stream));
  R_TRY(r, cudaMemcpyAsync(r->v(c0), v0, vec, cudaMemcpyDeviceToDevice, s->stream));
  R_TRY(r, cudaMemcpyAsync(r->F(c0), F0, mat, cudaMemcpyDeviceToDevice, s->stream));
  R_TRY(r, cudaMemcpyAsync(r->C(c0), C0, mat, cudaMemcpyDeviceToDevice, s->stream));
  // Jp starts at 1, as Particle<dim> sets it (src/nclr.h:46-47)
  R_TRY(r, cudaMemcpyAsync(r->Jp(c0), r->ones, sizeof(float) * (size_t)r->n,
                           cudaMemcpyDeviceToDevice, s->stream));
  R_TRY(r, cudaEventRecord(r->ev[0], s->stream));
  nclr_status st = load_state(r, c0);
  if (st != NCLR_OK) return st;
  for (int k = 1; k < r->nseg; ++k) {
    R_SIM(r, nclr_advance(s, r->every));
    if ((st = save_state(r, r->state(r->ckpt, k))) != NCLR_OK) return st;
  }
  R_SIM(r, nclr_advance(s, r->nsteps - (int64_t)(r->nseg - 1) * r->every));
  R_SIM(r, nclr_get_particles_device(s, xT, vT, FT, CT, nullptr));
  R_TRY(r, cudaEventRecord(r->ev[1], s->stream));
  R_TRY(r, cudaEventSynchronize(r->ev[1]));
  cudaEventElapsedTime(&r->fwd_ms, r->ev[0], r->ev[1]);
  r->have_forward = true;
  return NCLR_OK;
}

nclr_status nclr_rollout_forward(nclr_rollout *r, const float *x0, const float *v0, const float *F0,
                                 const float *C0, float E, float nu, float *xT, float *vT,
                                 float *FT, float *CT) {
  return rollout_forward(r, x0, v0, F0, C0, E, nu, nullptr, nullptr, xT, vT, FT, CT);
}

nclr_status nclr_rollout_forward_moduli(nclr_rollout *r, const float *x0, const float *v0,
                                        const float *F0, const float *C0, const float *E,
                                        const float *nu, float *xT, float *vT, float *FT,
                                        float *CT) {
  if (!E || !nu) return rfail(r, NCLR_ERR_INVALID, "E and nu are required");
  return rollout_forward(r, x0, v0, F0, C0, 0.0f, 0.0f, E, nu, xT, vT, FT, CT);
}

// The reverse pass of both entry points: scalar E / nu adjoints after a forward with the
// scene's pair, per-row ones (gEp, gnup) after a forward with per-particle moduli.
static nclr_status rollout_backward(nclr_rollout *r, const float *gxT, const float *gvT,
                                    const float *gFT, const float *gCT, float *gx0, float *gv0,
                                    float *gF0, float *gC0, double *gE, double *gnu,
                                    bool per_particle, float *gEp, float *gnup) {
  if (!r) return NCLR_ERR_INVALID;
  if (!r->have_forward) return rfail(r, NCLR_ERR_INVALID, "backward before forward");
  if (per_particle != r->per_particle)
    return rfail(r, NCLR_ERR_INVALID,
                 per_particle ? "the forward used the scene's E and nu: use nclr_rollout_backward"
                              : "the forward used per-particle moduli: use "
                                "nclr_rollout_backward_moduli");
  nclr_sim *s = r->sim;
  R_TRY(r, cudaSetDevice(s->device));
  const int D = r->dim;
  const int n = (int)r->n;
  const size_t vec = sizeof(float) * (size_t)n * D, mat = vec * D;
  R_TRY(r, cudaEventRecord(r->ev[0], s->stream));
  float *a = r->adj[0], *b = r->adj[1];
  auto seed = [&](float *dst, const float *src, size_t bytes) -> cudaError_t {
    return src ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, s->stream)
               : cudaMemsetAsync(dst, 0, bytes, s->stream);
  };
  R_TRY(r, seed(r->x(a), gxT, vec));
  R_TRY(r, seed(r->v(a), gvT, vec));
  R_TRY(r, seed(r->F(a), gFT, mat));
  R_TRY(r, seed(r->C(a), gCT, mat));
  R_TRY(r, seed(r->Jp(a), nullptr, sizeof(float) * (size_t)n));  // nothing depends on Jp_T
  R_TRY(r, cudaMemsetAsync(r->gml, 0, 2 * sizeof(double), s->stream));
  mpm::RowModuli rm;
  if (r->per_particle) {
    R_TRY(r, cudaMemsetAsync(r->grad_rows, 0, 2 * sizeof(double) * (size_t)n, s->stream));
    rm.lame = r->lame_rows;
    rm.grad = r->grad_rows;
  }
  R_TRY(r, cudaMemsetAsync(r->err, 0, sizeof(int), s->stream));
  R_TRY(r, cudaMemsetAsync(s->err_d, 0, 2 * sizeof(int) * (size_t)s->nscenes, s->stream));
  const Params &P = s->P0();
  bool used[2] = {false, false};
  const bool prof = s->opt.profile != 0;
  int64_t rstep = 0;  // reverse steps enqueued so far
  if (prof && r->rev_events.size() < 4 * (size_t)r->nsteps) {
    const size_t want = 4 * (size_t)r->nsteps;
    while (r->rev_events.size() < want) {
      cudaEvent_t e = nullptr;
      R_TRY(r, cudaEventCreate(&e));
      r->rev_events.push_back(e);
    }
  }
  for (int sg = r->nseg - 1; sg >= 0; --sg) {
    const int64_t t0 = (int64_t)sg * r->every;
    const int L = (int)std::min<int64_t>(r->every, r->nsteps - t0);
    const int buf = sg & 1;
    // recompute the segment into buffer `buf` (once the adjoint of the segment that used it
    // last is done): states s_t0..s_t0+L and the grids of its steps
    if (used[buf]) R_TRY(r, cudaStreamWaitEvent(s->stream, r->reversed[buf], 0));
    float *first = r->state(r->seg[buf], 0);
    R_TRY(r, cudaMemcpyAsync(first, r->state(r->ckpt, sg), sizeof(float) * r->rowf,
                             cudaMemcpyDeviceToDevice, s->stream));
    nclr_status st = load_state(r, first);
    if (st != NCLR_OK) return st;
    if ((st = record_segment(r, L, buf)) != NCLR_OK) return st;
    R_TRY(r, cudaEventRecord(r->recorded[buf], s->stream));
    // its adjoint on the reverse stream, overlapping the next recomputation
    R_TRY(r, cudaStreamWaitEvent(r->rev, r->recorded[buf], 0));
    for (int i = L - 1; i >= 0; --i) {
      float *st_t = r->state(r->seg[buf], i), *st_n = r->state(r->seg[buf], i + 1);
      cudaEvent_t *evs = prof ? r->rev_events.data() + 4 * (size_t)rstep : nullptr;
      dispatch_dim(D, [&](auto dc) {
        constexpr int DD = decltype(dc)::value;
        mpm::launch_adjoint_step<DD>(n, r->x(st_t), r->v(st_t), r->F(st_t), r->C(st_t),
                                     r->Jp(st_t), r->C(st_n), r->mass, r->vol,
                                     r->grids[buf] + (size_t)i * r->nodes, P, s->ref, r->x(a),
                                     r->v(a), r->F(a), r->C(a), r->Jp(a), r->x(b), r->v(b),
                                     r->F(b), r->C(b), r->Jp(b), r->VB, r->GB, r->gml, rm, r->err,
                                     r->rev, evs);
      });
      ++rstep;
      std::swap(a, b);
    }
    R_TRY(r, cudaEventRecord(r->reversed[buf], r->rev));
    used[buf] = true;
    nclr_status cst = check_launch(s, "adjoint step");
    if (cst != NCLR_OK) return rfail(r, cst, s->error);
  }
  // join the reverse stream back into the simulation's stream
  for (int b2 = 0; b2 < 2; ++b2)
    if (used[b2]) R_TRY(r, cudaStreamWaitEvent(s->stream, r->reversed[b2], 0));
  int serr[2] = {0, 0};
  R_TRY(r, cudaMemcpyAsync(serr, s->err_d, 2 * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  if (gx0) R_TRY(r, cudaMemcpyAsync(gx0, r->x(a), vec, cudaMemcpyDeviceToDevice, s->stream));
  if (gv0) R_TRY(r, cudaMemcpyAsync(gv0, r->v(a), vec, cudaMemcpyDeviceToDevice, s->stream));
  if (gF0) R_TRY(r, cudaMemcpyAsync(gF0, r->F(a), mat, cudaMemcpyDeviceToDevice, s->stream));
  if (gC0) R_TRY(r, cudaMemcpyAsync(gC0, r->C(a), mat, cudaMemcpyDeviceToDevice, s->stream));
  if (r->per_particle)
    R_TRY(r, mpm::launch_moduli_grads(n, r->mod_E, r->mod_nu, r->grad_rows, gEp, gnup, s->stream));
  double gml[2] = {0.0, 0.0};
  int err = 0;
  R_TRY(r, cudaMemcpyAsync(gml, r->gml, sizeof(gml), cudaMemcpyDeviceToHost, s->stream));
  R_TRY(r, cudaMemcpyAsync(&err, r->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  R_TRY(r, cudaEventRecord(r->ev[1], s->stream));
  R_TRY(r, cudaEventSynchronize(r->ev[1]));
  cudaEventElapsedTime(&r->bwd_ms, r->ev[0], r->ev[1]);
  if (prof) {  // the reverse kernels of every step, and the recomputation's forward kernels
    for (int64_t k = 0; k < rstep; ++k) {
      const cudaEvent_t *e4 = r->rev_events.data() + 4 * (size_t)k;
      const int phases[3] = {NCLR_PHASE_ADJ_G2P, NCLR_PHASE_ADJ_GRID, NCLR_PHASE_ADJ_P2G};
      for (int j = 0; j < 3; ++j) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, e4[j], e4[j + 1]) == cudaSuccess) s->prof_ms[phases[j]] += ms;
        // adj_g2p and adj_p2g do not launch without particles; n >= 1 in a rollout
        s->prof_launches[phases[j]] += 1;
      }
    }
    collect_profile(s);
  }
  // mu_0 = E / (2 (1 + nu)), lambda_0 = E nu / ((1 + nu)(1 - 2 nu)) (src/nclr.h:77-78)
  const double E = r->E, nu = r->nu;
  const double dmu_dE = 1.0 / (2.0 * (1.0 + nu)), dmu_dnu = -E / (2.0 * (1.0 + nu) * (1.0 + nu));
  const double q = (1.0 + nu) * (1.0 - 2.0 * nu);
  const double dl_dE = nu / q, dl_dnu = E * (1.0 + 2.0 * nu * nu) / (q * q);
  if (gE) *gE = gml[0] * dmu_dE + gml[1] * dl_dE;
  if (gnu) *gnu = gml[0] * dmu_dnu + gml[1] * dl_dnu;
  if ((serr[0] | serr[1]) & mpm::kErrOutOfRange)
    return rfail(r, NCLR_ERR_OUT_OF_RANGE, "a stencil left the grid during the recomputation");
  if (err & mpm::kErrOutOfRange) return rfail(r, NCLR_ERR_OUT_OF_RANGE, "a stencil left the grid");
  return NCLR_OK;
}

nclr_status nclr_rollout_backward(nclr_rollout *r, const float *gxT, const float *gvT,
                                  const float *gFT, const float *gCT, float *gx0, float *gv0,
                                  float *gF0, float *gC0, double *gE, double *gnu) {
  return rollout_backward(r, gxT, gvT, gFT, gCT, gx0, gv0, gF0, gC0, gE, gnu, false, nullptr,
                          nullptr);
}

nclr_status nclr_rollout_backward_moduli(nclr_rollout *r, const float *gxT, const float *gvT,
                                         const float *gFT, const float *gCT, float *gx0,
                                         float *gv0, float *gF0, float *gC0, float *gE,
                                         float *gnu) {
  return rollout_backward(r, gxT, gvT, gFT, gCT, gx0, gv0, gF0, gC0, nullptr, nullptr, true, gE,
                          gnu);
}

nclr_status nclr_rollout_profile_get(const nclr_rollout *r, int phase, double *total_ms,
                                     int64_t *launches) {
  if (!r) return NCLR_ERR_INVALID;
  return nclr_profile_get(r->sim, phase, total_ms, launches);
}

nclr_status nclr_rollout_profile_reset(nclr_rollout *r) {
  if (!r) return NCLR_ERR_INVALID;
  return nclr_profile_reset(r->sim);
}

nclr_status nclr_rollout_timing(const nclr_rollout *r, double *forward_ms, double *backward_ms) {
  if (!r) return NCLR_ERR_INVALID;
  if (forward_ms) *forward_ms = r->fwd_ms;
  if (backward_ms) *backward_ms = r->bwd_ms;
  return NCLR_OK;
}

void *nclr_rollout_stream(nclr_rollout *r) { return r ? (void *)r->sim->stream : nullptr; }

const char *nclr_rollout_error(const nclr_rollout *r) {
  return r ? r->error.c_str() : g_create_error.c_str();
}

void nclr_rollout_destroy(nclr_rollout *r) { rollout_release(r); }

}  // extern "C"
