// Host-side launchers of the step kernels (instantiated for dim 2 and 3 in step2d.cu and
// step3d.cu) and of the dimension-free scan (scan.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace mpm {

struct Params;
struct PState;

template <int D> void launch_prepare(const PState &s, const Params &P, float4 *pay, bool ref, cudaStream_t st);
template <int D> void launch_p2g(const float4 *pay, const Params &P, float4 *grid, int *err, int K, cudaStream_t st);
template <int D> void launch_g2p(const PState &s, const Params &P, const float4 *grid, float4 *pay, int *err, bool ref, cudaStream_t st);
template <int D> void launch_export_grid(const float4 *grid, const Params &P, float *vel, float *mass, cudaStream_t st);
template <int D> void launch_export_particles(const PState &s, int n, float *x, float *v, float *F, float *C, float *Jp, cudaStream_t st);
template <int D> void launch_import_particles(const PState &s, int n, const float *x, const float *v, const float *F, const float *C, const float *Jp, cudaStream_t st);
template <int D> void launch_sort_keys(const PState &s, const Params &P, int *key, int *rank, int *count, cudaStream_t st);
template <int D> void launch_sort_move(const PState &src, const PState &dst, int n, const float4 *pay_src, float4 *pay_dst, const int *key, const int *rank, const int *start, cudaStream_t st);

// Exclusive prefix sum of count[0..n) into start[0..n]; tile_sums must hold
// scan_tiles(n) ints.  Three launches.
int64_t scan_tiles(int64_t n);
void launch_exclusive_scan(const int *count, int64_t n, int *start, int *tile_sums, cudaStream_t st);

// *out += number of grid nodes with mass > 0 (the .w lane of each node).
void launch_count_active(const float4 *grid, int64_t nodes, unsigned long long *out, cudaStream_t st);

}  // namespace mpm
