// Host-side launchers of the step kernels (instantiated for dim 2 and 3 in step2d.cu and
// step3d.cu) and of the dimension-free scan utilities (scan.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

struct Params;
struct PState;
struct Scene;

// Caller-order copies of the state after a final-mode step (rows of x, v: dim floats; F, C:
// dim*dim floats), written by the fused kernel for the adjoint's recorded segments; all null
// when not recording (single simulations only).
struct Record {
  float *x, *v, *F, *C;
  float *Jp = nullptr;  // (may be null) Jp rows too
};

// The snow clamps a fused launch leaves for FP64 (mpm_step.cuh: snow_clamp_needs_fp64): the
// fused kernel appends the particle's slot, its F_hat and its Jp before the clamp, and keeps its
// FP32 result meanwhile; launch_snow_fix then recomputes those clamps in FP64, writes F and Jp
// and corrects the launch's P2G by the difference of the two stresses.  count is reset by the
// grid sweep that starts every step; cap >= the particles of one launch.  All null: no list
// (the small-scene kernels recompute in place).
struct SnowFix {
  int *count = nullptr;
  int cap = 0;
  int *slot = nullptr;
  float *Fh = nullptr;  // dim*dim per entry
  float *Jp = nullptr;
};

// P0: the one scene's parameters when block_scene is null (a single simulation).
template <int D> void launch_grid_sweep(float4 *G, float4 *V, uint8_t *flags, const Scene *scenes,
                                        const uint16_t *block_scene, const Params &P0,
                                        int total_blocks, int *work, int sms, cudaStream_t st,
                                        int *fix_count = nullptr);
// The FP64 snow clamps of the last fused launch (see SnowFix); scatter: that launch did the next
// step's P2G (not the G2P-only final step), whose accumulator G receives the correction.
template <int D> void launch_snow_fix(const PState &s, const Params &P0, const Scene *scenes,
                                      const SnowFix &fix, float4 *G, bool scatter, bool ref,
                                      const Record &rec, int sms, cudaStream_t st);
template <int D> void launch_discard_pending(float4 *G, uint8_t *flags, const Scene *scenes,
                                             const uint16_t *block_scene, int total_blocks, int sms,
                                             cudaStream_t st);
// err[2 s] collects scene s's errors of this call, err[2 s + next_slot] those of the P2G that
// follows the launch (next_slot 0: same call, 1: the next call).
template <int D> void launch_g2p2g(const PState &s, const Params &P0, const Scene *scenes, const uint16_t *block_scene,
                                   const float4 *V, float4 *G, uint8_t *flags, const int *blocks,
                                   const int *nactive, const int *bstart, const int *sparse, int *work,
                                   int *err, int next_slot, bool ref, int mode, int ctas, cudaStream_t st,
                                   const Record &rec = Record{}, const SnowFix &fix = SnowFix{},
                                   int item_threads = 0);
template <int D> int g2p2g_ctas_per_sm();
template <int D> int g2p_final_ctas_per_sm();
// The small-scene kernels' grid barrier: how many polls a waiting CTA makes before it gives up
// (about a second at the default), and how many arrivals beyond the launch's CTAs it waits for
// (0; a test sets 1, so that the wait runs out and the error path runs).
constexpr unsigned kBarrierSpinsDefault = 1u << 24;
struct BarrierTest {
  unsigned extra = 0;
  unsigned spins = kBarrierSpinsDefault;
};
// Small scenes: all `steps` steps of one scene in one cooperative launch (kSmallThreads-thread
// CTAs, `ctas` of them, all resident); bar = 2 zeroed unsigned.
template <int D> cudaError_t launch_small_steps(const PState &s, const Params &P, float4 *G, float4 *V,
                                               int steps, int *err, unsigned *bar, bool ref, int ctas,
                                               cudaStream_t st, BarrierTest bt = BarrierTest{});
template <int D> int small_ctas_per_sm(bool ref);
// The small-scene kernel launched as one thread-block cluster (the step's barriers are the
// cluster's hardware barrier): `ctas` <= small_cluster_max(ref, threads) CTAs of `threads`
// (<= kSmallClusterThreads[dim]) threads.
template <int D> cudaError_t launch_small_cluster(const PState &s, const Params &P, float4 *G,
                                                  float4 *V, int steps, int *err, unsigned *bar,
                                                  bool ref, int ctas, int threads, cudaStream_t st);
template <int D> int small_cluster_max(bool ref, int threads);
constexpr int kSmallClusterThreads2D = 640, kSmallClusterThreads3D = 512;
// The same for a batch: CTA c works on scene cta_scene[c]; scene s owns CTAs
// [group_first[s], group_first[s+1]) and the barrier bars[2s..2s+1] (zeroed).
template <int D> cudaError_t launch_small_batch(const PState &s, const Scene *scenes, const uint16_t *cta_scene,
                                               const int *group_first, float4 *G, float4 *V, uint8_t *flags,
                                               int steps, int *err, unsigned *bars, bool ref, int ctas,
                                               cudaStream_t st, BarrierTest bt = BarrierTest{});
template <int D> int small_batch_ctas_per_sm(bool ref);
constexpr int kSmallThreadsPerCta = 256;
constexpr uint8_t kFlagVNonzeroBit = 2;  // mpm_step.cuh's kVNonzero: V may be non-zero there
// g2p2g modes; kModeG2PFinal exists for single simulations only
enum : int { kModeStep = 0, kModeFinalStep = 1, kModeP2GOnly = 2, kModeG2PFinal = 3 };
template <int D> void launch_copy_vgrid(const float4 *V, int64_t nodes, float *vel, float *mass, cudaStream_t st);
template <int D> void launch_export_grid(const float4 *grid, const Params &P, float *vel, float *mass, cudaStream_t st);
// Caller rows [0, n) of the scene whose global ids (and slots) start at id_off <-> their
// slots: the export runs per caller row through inv (global id -> slot), the import per slot
// through id.  The import counts, into *moved (when non-null), the rows that left their
// slot's grid block.
template <int D> void launch_export_rows(const PState &s, const int *inv, int id_off, int n, float *x, float *v,
                                         float *F, float *C, float *Jp, cudaStream_t st);
template <int D> void launch_import_rows(const PState &s, int id_off, int n, const float *x,
                                         const float *v, const float *F, const float *C, const float *Jp,
                                         const Scene *scenes, const int *slot_block, int *moved,
                                         cudaStream_t st);
template <int D> void launch_block_keys(const PState &s, int n, const Scene *scenes, int *key, int *rank, int *count,
                                        cudaStream_t st);
// Also records inv[id] = new slot and slot_block[new slot] = its grid block.
template <int D> void launch_sort_move(const PState &src, const PState &dst, int n, const int *key, const int *rank, const int *bstart, const int4 *rounds, const int *count, bool move_vc, int *inv, int *slot_block, cudaStream_t st);
// The block sort's per-block round tables (block_tables_kernel in scan.cu): btotal[b] and
// rounds[b * kRoundTable + r] for the nblocks blocks of kCellsPerBlock cells.
constexpr int kCellsPerBlock = 64;  // Tiling<2>::CPB and Tiling<3>::CPB
constexpr int kRoundTable = 12;     // rounds with a table entry; later ranks count cell by cell
void launch_block_tables(const int *count, int nblocks, int *btotal, int4 *rounds, cudaStream_t st);
// Threads of the fused step's CTA; a single simulation's item steps a block's particles in
// passes of this many.
constexpr int kG2P2GThreads = 256;
// The non-empty blocks of the sort: those with at least sparse_max particles (all of them when
// sparse_max <= 0) go to list, the particle slots of the others, block by block, to sparse /
// nlist[1].  A listed block of more than kG2P2GThreads particles whose last pass would hold
// fewer than tail_max (0: none) also puts those last slots into sparse.  list (capacity
// nblocks) holds the blocks of more than kG2P2GThreads particles (after that rule) at its
// front (list[0 .. nlist[0])) and the others at its back (list[nblocks - 1 - k],
// k < nlist[2]); nlist[3] = nblocks.  nlist[0..2]
// must be zero on entry.
void launch_compact_blocks(const int *start, int nblocks, int cpb, int sparse_max, int tail_max,
                           int *list, int *nlist, int *sparse, cudaStream_t st);

// Counts material[] entries above NCLR_LIQUID into *out (host); synchronises `st`
// (scene_build.cu).
cudaError_t count_bad_materials(const uint8_t *mat, int64_t n, int *scratch, int *out, cudaStream_t st);
// lame[p] = (mu_0, lambda_0) of caller row id[p]'s E and nu (row p when id is null), for the
// n slots.
cudaError_t launch_set_lame(const int *id, int n, const float *E, const float *nu, float2 *lame,
                            cudaStream_t st);

// Reverse of one step of the scene's material P.model (adjoint.cu): adjoint of s_{t+1}
// (gx, gv, gF, gC, gJp; NULL = 0) -> adjoint of s_t (ox, ov, oF, oC, oJp; oJp may be NULL for
// jelly), mu_0 / lambda_0 adjoints added to gml[0..1].  States are caller-order rows (Jp: the
// state's plastic volume ratio, NULL = 1); V is the step's updated grid; VB (4 floats per
// node) must be zero on entry and is zero again on exit; GB holds nodes float4.  ev (may be
// null): four events recorded on `st` before adj_g2p, between the kernels and after adj_p2g
// (per-kernel timing).
// Per-particle moduli of a rollout, per row in the caller's order (both null: the scene's
// pair): lame[q] = (mu_0, lambda_0) of row q; grad[2q], grad[2q + 1] accumulate the adjoints of
// row q's mu_0 and lambda_0 over the reverse steps.
struct RowModuli {
  const float2 *lame = nullptr;
  double *grad = nullptr;
};
template <int D>
void launch_adjoint_step(int n, const float *x, const float *v, const float *F, const float *C,
                         const float *Jp, const float *Cn, const float *mass, const float *vol,
                         const float4 *V, const Params &P, bool ref, const float *gx,
                         const float *gv, const float *gF, const float *gC, const float *gJp,
                         float *ox, float *ov, float *oF, float *oC, float *oJp, float *VB,
                         float4 *GB, double *gml, RowModuli rm, int *err, cudaStream_t st,
                         cudaEvent_t *ev = nullptr);
// gE[q], gnu[q] from row q's accumulated mu_0 / lambda_0 adjoints (grad) and its E[q], nu[q],
// through mu_0 = E / (2 (1 + nu)), lambda_0 = E nu / ((1 + nu)(1 - 2 nu)).
cudaError_t launch_moduli_grads(int n, const float *E, const float *nu, const double *grad,
                                float *gE, float *gnu, cudaStream_t st);

// Exclusive prefix sum of count[0..n) into start[0..n]; tile_sums must hold
// scan_tiles(n) ints.  Three launches.
int64_t scan_tiles(int64_t n);
void launch_exclusive_scan(const int *count, int64_t n, int *start, int *tile_sums, cudaStream_t st);

// *out += number of grid nodes with mass > 0 (the .w lane of each node).
void launch_count_active(const float4 *grid, int64_t nodes, unsigned long long *out, cudaStream_t st);

}  // namespace mpm
