// Dimension-free helpers of the block sort: the per-block round tables, the exclusive prefix
// sum over the per-block particle counts of the counting sort, the compaction of the
// non-empty blocks and a count of grid nodes holding mass.  The scan:
// (1) per-tile totals, (2) one block scans the tile totals, (3) each tile scans its counts
// and adds its tile offset.  Tiles are 2048 counts (256 threads x 8), read as int4 pairs
// where aligned.
#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_launch.h"

namespace mpm {

namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ int warp_inclusive(int v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int u = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += u;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total in *total.
__device__ __forceinline__ int block_exclusive(int v, int *total) {
  __shared__ int warp_sums[kThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_inclusive(v);
  if (lane == 31) warp_sums[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int s = (lane < kThreads / 32) ? warp_sums[lane] : 0;
    s = warp_inclusive(s);
    if (lane < kThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  const int before = (wid > 0) ? warp_sums[wid - 1] : 0;
  *total = warp_sums[kThreads / 32 - 1];
  __syncthreads();
  return before + inc - v;
}

__global__ void __launch_bounds__(kThreads) tile_totals(const int *__restrict__ count, int64_t n,
                                                        int *__restrict__ tile_sums) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i)
    if (base + i < n) s += count[base + i];
  int total;
  block_exclusive(s, &total);
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kThreads) scan_totals(int *__restrict__ tile_sums, int64_t ntiles,
                                                        int *__restrict__ grand_total) {
  int carry = 0;
  for (int64_t b = 0; b < ntiles; b += kThreads) {
    const int64_t i = b + threadIdx.x;
    const int v = (i < ntiles) ? tile_sums[i] : 0;
    int total;
    const int ex = block_exclusive(v, &total);
    if (i < ntiles) tile_sums[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *grand_total = carry;
}

__global__ void __launch_bounds__(kThreads) tile_apply(const int *__restrict__ count, int64_t n,
                                                       const int *__restrict__ tile_sums,
                                                       int *__restrict__ start) {
  const int64_t base = (int64_t)blockIdx.x * kTile + (int64_t)threadIdx.x * kItems;
  int v[kItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    v[i] = (base + i < n) ? count[base + i] : 0;
    s += v[i];
  }
  int total;
  int run = block_exclusive(s, &total) + tile_sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kItems; ++i) {
    if (base + i < n) start[base + i] = run;
    run += v[i];
  }
}

// One warp per grid block of kCellsPerBlock cells: the block's particle total, and for every
// round r < min(largest cell count, kRoundTable) the entry {particles in rounds < r, the
// 64-bit mask of cells holding more than r particles}.  Particle r of cell c then sits at
// block start + entry.x + popc(mask & ((1 << c) - 1)) in the cell-by-cell-in-rounds order.
__global__ void __launch_bounds__(kThreads) block_tables_kernel(const int *__restrict__ count,
                                                                int nblocks,
                                                                int *__restrict__ btotal,
                                                                int4 *__restrict__ rounds) {
  static_assert(kCellsPerBlock == 64, "two cells per lane");
  const int b = (int)(((int64_t)blockIdx.x * kThreads + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (b >= nblocks) return;  // the whole warp
  const int *c = count + (int64_t)b * kCellsPerBlock;
  const int lo = c[lane], hi = c[32 + lane];
  int total = lo + hi, mx = max(lo, hi);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    total += __shfl_xor_sync(0xffffffffu, total, o);
    mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  if (lane == 0) btotal[b] = total;
  const int R = min(mx, kRoundTable);
  int before = 0;
  for (int r = 0; r < R; ++r) {
    const unsigned mlo = __ballot_sync(0xffffffffu, lo > r), mhi = __ballot_sync(0xffffffffu, hi > r);
    if (lane == 0) rounds[(int64_t)b * kRoundTable + r] = make_int4(before, (int)mlo, (int)mhi, 0);
    before += __popc(mlo) + __popc(mhi);
  }
}

__global__ void __launch_bounds__(kThreads) count_active_kernel(const float4 *__restrict__ grid,
                                                               int64_t nodes,
                                                               unsigned long long *out) {
  unsigned c = 0;
  for (int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x; i < nodes;
       i += (int64_t)gridDim.x * kThreads)
    c += grid[i].w > 0.0f ? 1u : 0u;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

// The non-empty blocks (start[b*cpb] < start[(b+1)*cpb]): those with at least sparse_max
// particles go to the block list, the particle slots of the thinner ones to the sparse list
// (stepped particle by particle), and so do the last np % kG2P2GThreads slots of a listed
// block of np > kG2P2GThreads particles when they are fewer than tail_max: the fused kernel
// would otherwise run a last pass of a few particles with the rest of the CTA waiting (the
// fused kernel applies the same rule).  Item order: blocks of more than kG2P2GThreads
// particles (after the tail rule) go to the front of the list, the others to its back, so the
// fused kernel's CTAs take the long items first and the launch ends on short ones (measured
// per fused launch, 1M particles: corrected snow 183 -> 169 us, exploding snow 707 -> 668,
// corrected jelly 162 -> 157, jelly 142-144 -> 142).  One atomic per warp and list for the
// append position, so the sparse slots stay in block order within each warp's run of 32
// blocks.
__global__ void compact_blocks_kernel(const int *__restrict__ start, int nblocks, int cpb,
                                      int sparse_max, int tail_max, int *__restrict__ list,
                                      int *__restrict__ nlist, int *__restrict__ sparse) {
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  int s0 = 0, np = 0;
  if (b < nblocks) {
    s0 = start[(int64_t)b * cpb];
    np = start[(int64_t)(b + 1) * cpb] - s0;
  }
  const bool thin = np > 0 && np < sparse_max;
  const bool act = np > 0 && !thin;
  const int tail = np % kG2P2GThreads;
  const bool cut = act && np > kG2P2GThreads && tail < tail_max;
  const bool multi = act && (cut ? np - tail : np) > kG2P2GThreads;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const unsigned mfront = __ballot_sync(0xffffffffu, multi);
  const unsigned mback = __ballot_sync(0xffffffffu, act && !multi);
  if (mfront | mback) {
    int front = 0, back = 0;
    if (lane == 0) {
      if (mfront) front = atomicAdd(nlist, __popc(mfront));
      if (mback) back = atomicAdd(nlist + 2, __popc(mback));
    }
    front = __shfl_sync(0xffffffffu, front, 0);
    back = __shfl_sync(0xffffffffu, back, 0);
    if (multi)
      list[front + __popc(mfront & below)] = b;
    else if (act)
      list[nblocks - 1 - (back + __popc(mback & below))] = b;
  }
  if (b == 0) nlist[3] = nblocks;
  const int cnt = thin ? np : (cut ? tail : 0);
  if (cut) s0 += np - tail;
  const int inc = warp_inclusive(cnt);
  const int tot = __shfl_sync(0xffffffffu, inc, 31);
  if (tot) {
    int base = 0;
    if (lane == 0) base = atomicAdd(nlist + 1, tot);
    base = __shfl_sync(0xffffffffu, base, 0) + inc - cnt;
    for (int i = 0; i < cnt; ++i) sparse[base + i] = s0 + i;
  }
}

}  // namespace

void launch_block_tables(const int *count, int nblocks, int *btotal, int4 *rounds, cudaStream_t st) {
  if (nblocks <= 0) return;
  const int64_t threads = (int64_t)nblocks * 32;
  block_tables_kernel<<<(unsigned)((threads + kThreads - 1) / kThreads), kThreads, 0, st>>>(
      count, nblocks, btotal, rounds);
}

void launch_compact_blocks(const int *start, int nblocks, int cpb, int sparse_max, int tail_max,
                           int *list, int *nlist, int *sparse, cudaStream_t st) {
  if (nblocks <= 0) return;
  compact_blocks_kernel<<<(unsigned)((nblocks + kThreads - 1) / kThreads), kThreads, 0, st>>>(
      start, nblocks, cpb, sparse_max, tail_max, list, nlist, sparse);
}

void launch_count_active(const float4 *grid, int64_t nodes, unsigned long long *out, cudaStream_t st) {
  if (nodes <= 0) return;
  int64_t blocks = (nodes + kThreads - 1) / kThreads;
  if (blocks > 152 * 8) blocks = 152 * 8;
  count_active_kernel<<<(unsigned)blocks, kThreads, 0, st>>>(grid, nodes, out);
}

int64_t scan_tiles(int64_t n) { return (n + kTile - 1) / kTile; }

void launch_exclusive_scan(const int *count, int64_t n, int *start, int *tile_sums, cudaStream_t st) {
  const int64_t nt = scan_tiles(n);
  if (nt == 0) return;
  tile_totals<<<(unsigned)nt, kThreads, 0, st>>>(count, n, tile_sums);
  scan_totals<<<1, kThreads, 0, st>>>(tile_sums, nt, start + n);
  tile_apply<<<(unsigned)nt, kThreads, 0, st>>>(count, n, tile_sums, start);
}

}  // namespace mpm
