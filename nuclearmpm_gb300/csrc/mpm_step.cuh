// Kernels of one MLS-MPM step and of the host<->device transfers, templated on the
// dimension; step2d.cu / step3d.cu instantiate them.
#pragma once

#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

// ---------------------------------------------------------------------------------------
// prepare_payload: the P2G input of each slot from the particle state (src/nclr.h:129,162:
// stress + APIC affine and m v), used after the state was uploaded or replaced.
// ---------------------------------------------------------------------------------------
template <int D, bool kRef>
__global__ void __launch_bounds__(256) prepare_payload_kernel(PState s, Params P,
                                                              float4 *__restrict__ pay) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int st = s.stride;
  float x[D], v[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    x[d] = s.x[(size_t)d * st + p];
    v[d] = s.v[(size_t)d * st + p];
  }
  const Mat<D> F = load_mat<D>(s.F, st, p);
  const Mat<D> C = load_mat<D>(s.C, st, p);
  const float Jp = s.Jp[p], m = s.mass[p], vol = s.vol[p];
  const int material = s.mat ? (int)s.mat[p] : P.model;
  const Mat<D> R = polar_R(F);
  const Mat<D> A = fused_affine<D>(F, R, C, Jp, m, vol, material, P);
  store_payload<D>(pay, p, x, m, v, A);
}

// ---------------------------------------------------------------------------------------
// P2G scatter (src/nclr.h:104-165).  Each thread takes K consecutive slots; slots are kept
// sorted by grid cell, so consecutive particles usually share the same 3^dim stencil.
// The thread accumulates its particles' contributions in registers while the cell stays
// the same and flushes them with one 16-byte vector reduction per node when it changes.
// ---------------------------------------------------------------------------------------
template <int D, int K>
__global__ void __launch_bounds__(128) p2g_kernel(const float4 *__restrict__ pay, Params P,
                                                  float4 *__restrict__ grid, int *err) {
  constexpr int S = (D == 3) ? 27 : 9;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int i0 = t * K;
  if (i0 >= P.n) return;
  const int i1 = min(i0 + K, P.n);
  float acc[S][4];
  int cb[D];
  int64_t cur = INT64_MIN;
  const float dx = P.dx;
  const int N = P.N;

  auto flush = [&]() {
    const int64_t f0 = flat_index<D>(cb, N);
    // 3D: node (i,j,k) of the stencil is f0 + i N^2 + j N + k
    const int64_t hi = (D == 3) ? f0 + 2 * (int64_t)N * N + 2 * N + 2 : f0 + 2 * (int64_t)N + 2;
    const bool inside = f0 >= 0 && hi < P.nodes;
#pragma unroll
    for (int o = 0; o < S; ++o) {
      const int oi = (D == 3) ? o / 9 : o / 3;
      const int oj = (D == 3) ? (o / 3) % 3 : o % 3;
      const int ok = (D == 3) ? o % 3 : 0;
      const int64_t f = (D == 3) ? f0 + ((int64_t)oi * N + oj) * N + ok : f0 + (int64_t)oi * N + oj;
      if (inside || (f >= 0 && f < P.nodes)) {
        red_add_v4(grid + f, acc[o][0], acc[o][1], acc[o][2], acc[o][3]);
      } else {
        atomicOr(err, kErrOutOfRange);
      }
    }
  };

  for (int i = i0; i < i1; ++i) {
    float x[D], mv[D], m;
    Mat<D> A;
    load_payload<D>(pay, i, x, m, mv, A);
    int base[D];
    float fx[D], w[3][D];
    stencil<D>(x, P.inv_dx, base, fx, w);
    const int64_t f = flat_index<D>(base, N);
    if (f != cur) {
      if (cur != INT64_MIN) flush();
#pragma unroll
      for (int o = 0; o < S; ++o) acc[o][0] = acc[o][1] = acc[o][2] = acc[o][3] = 0.0f;
      cur = f;
#pragma unroll
      for (int d = 0; d < D; ++d) cb[d] = base[d];
    }
#pragma unroll
    for (int o = 0; o < S; ++o) {
      const int oi = (D == 3) ? o / 9 : o / 3;
      const int oj = (D == 3) ? (o / 3) % 3 : o % 3;
      const int ok = (D == 3) ? o % 3 : 0;
      const int oo[3] = {oi, oj, ok};
      float dpos[D];
#pragma unroll
      for (int d = 0; d < D; ++d) dpos[d] = ((float)oo[d] - fx[d]) * dx;
      float weight = w[oi][0] * w[oj][1];
      if (D == 3) weight = weight * w[ok][D - 1];
#pragma unroll
      for (int r = 0; r < D; ++r) {
        float ad = A.a[r][0] * dpos[0];
#pragma unroll
        for (int c = 1; c < D; ++c) ad = ad + A.a[r][c] * dpos[c];
        acc[o][r] += weight * (mv[r] + ad);
      }
      acc[o][3] += weight * m;
    }
  }
  if (cur != INT64_MIN) flush();
}

// ---------------------------------------------------------------------------------------
// G2P (src/nclr.h:167-261) fused with the grid update (src/nclr.h:263-310) and with the
// next step's stress (src/nclr.h:313-337): gathers the 3^dim post-update node velocities,
// rebuilds v and the APIC C, advects x, updates F, applies the material's plasticity, and
// writes the new state plus the payload the next P2G reads.
// ---------------------------------------------------------------------------------------
template <int D, bool kRef>
__global__ void __launch_bounds__(128) g2p_kernel(PState s, Params P,
                                                  const float4 *__restrict__ grid,
                                                  float4 *__restrict__ pay, int *err) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  const int st = s.stride;
  const int N = P.N;
  float x[D];
#pragma unroll
  for (int d = 0; d < D; ++d) x[d] = s.x[(size_t)d * st + p];
  int base[D];
  float fx[D], w[3][D];
  stencil<D>(x, P.inv_dx, base, fx, w);
  const int64_t f0 = flat_index<D>(base, N);
  bool axes_inside = true;
#pragma unroll
  for (int d = 0; d < D; ++d) axes_inside &= base[d] >= 0 && base[d] + 2 < N;

  float v[D];
  Mat<D> C;
#pragma unroll
  for (int d = 0; d < D; ++d) v[d] = 0.0f;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) C.a[i][j] = 0.0f;

  constexpr int S = (D == 3) ? 27 : 9;
#pragma unroll
  for (int o = 0; o < S; ++o) {
    const int oi = (D == 3) ? o / 9 : o / 3;
    const int oj = (D == 3) ? (o / 3) % 3 : o % 3;
    const int ok = (D == 3) ? o % 3 : 0;
    const int oo[3] = {oi, oj, ok};
    const int64_t f = (D == 3) ? f0 + ((int64_t)oi * N + oj) * N + ok : f0 + (int64_t)oi * N + oj;
    float gv[D];
    if (f >= 0 && f < P.nodes) {
      int idx[D];
      if (axes_inside) {
#pragma unroll
        for (int d = 0; d < D; ++d) idx[d] = base[d] + oo[d];
      } else {
        unflatten<D>(f, N, idx);
      }
      float m;
      grid_update<D>(__ldg(grid + f), idx, P, gv, m);
    } else {
      atomicOr(err, kErrOutOfRange);
#pragma unroll
      for (int d = 0; d < D; ++d) gv[d] = 0.0f;
    }
    float weight = w[oi][0] * w[oj][1];
    if (D == 3) weight = weight * w[ok][D - 1];
    float wgv[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      wgv[d] = weight * gv[d];
      v[d] += wgv[d];
    }
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) C.a[i][j] += (P.cscale * wgv[i]) * ((float)oo[j] - fx[j]);
  }

#pragma unroll
  for (int d = 0; d < D; ++d) x[d] += P.dt * v[d];
  Mat<D> M;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M.a[i][j] = diag_one<D, kRef>(i, j) + P.dt * C.a[i][j];
  const Mat<D> F = load_mat<D>(s.F, st, p);
  Mat<D> Fh = mat_mul<D>(M, F);
  float Jp = s.Jp[p];
  const int material = s.mat ? (int)s.mat[p] : P.model;
  Mat<D> R;
  if (material == kJelly) {
    R = polar_R(Fh);
  } else {
    Mat<D> U, V;
    float sig[D];
    if constexpr (D == 3) {
      svd3(Fh, U, sig, V);
    } else {
      svd2<kRef>(Fh, U, sig, V);
    }
    if (material == kSnow) {
#pragma unroll
      for (int d = 0; d < D; ++d) sig[d] = clampf_(sig[d], 1.0f - 2.5e-2f, 1.0f + 4.5e-3f);
      const float old_J = det(Fh);
      Fh = usv<D>(U, sig, V);
      Jp = clampf_(Jp * old_J / det(Fh), 0.6f, 20.0f);
      if constexpr (D == 3) {
        R = uvt<3>(U, V);  // the clamped sigma are positive: F = (U V^T)(V S V^T)
      } else {
        R = polar_rotation(Fh);
      }
    } else {  // liquid: J = prod sigma accumulated in double (src/nclr.h:253-257)
      double J = 1.0;
#pragma unroll
      for (int d = 0; d < D; ++d) J *= (double)sig[d];
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) Fh.a[i][j] = diag_one<D, kRef>(i, j);
      Fh.a[0][0] = (float)J;
      R = polar_R(Fh);
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) {
    s.x[(size_t)d * st + p] = x[d];
    s.v[(size_t)d * st + p] = v[d];
  }
  store_mat<D>(s.F, st, p, Fh);
  store_mat<D>(s.C, st, p, C);
  s.Jp[p] = Jp;
  const float m = s.mass[p], vol = s.vol[p];
  const Mat<D> A = fused_affine<D>(Fh, R, C, Jp, m, vol, material, P);
  store_payload<D>(pay, p, x, m, v, A);
}

// ---------------------------------------------------------------------------------------
// grid() export (src/nclr.h:87): the post-update grid in the reference's node order.
// ---------------------------------------------------------------------------------------
template <int D>
__global__ void export_grid_kernel(const float4 *__restrict__ grid, Params P,
                                   float *__restrict__ vel, float *__restrict__ mass) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= P.nodes) return;
  int idx[D];
  unflatten<D>(f, P.N, idx);
  float v[D], m;
  grid_update<D>(grid[f], idx, P, v, m);
#pragma unroll
  for (int d = 0; d < D; ++d) vel[f * D + d] = v[d];
  mass[f] = m;
}

// particles() export: slot-major SoA -> caller's order, particle-major rows.
template <int D>
__global__ void export_particles_kernel(PState s, int n, float *__restrict__ x,
                                        float *__restrict__ v, float *__restrict__ F,
                                        float *__restrict__ C, float *__restrict__ Jp) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int st = s.stride;
  const int q = s.id[p];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (x) x[(size_t)q * D + d] = s.x[(size_t)d * st + p];
    if (v) v[(size_t)q * D + d] = s.v[(size_t)d * st + p];
  }
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    if (F) F[(size_t)q * D * D + c] = s.F[(size_t)c * st + p];
    if (C) C[(size_t)q * D * D + c] = s.C[(size_t)c * st + p];
  }
  if (Jp) Jp[q] = s.Jp[p];
}

// Upload: caller's rows -> SoA slots.  Slot p takes caller particle id[p] (the current
// permutation is kept, so a partial update leaves the other fields in place).
template <int D>
__global__ void import_particles_kernel(PState s, int n, const float *__restrict__ x,
                                        const float *__restrict__ v, const float *__restrict__ F,
                                        const float *__restrict__ C,
                                        const float *__restrict__ Jp) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int st = s.stride;
  const int q = s.id[p];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    if (x) s.x[(size_t)d * st + p] = x[(size_t)q * D + d];
    if (v) s.v[(size_t)d * st + p] = v[(size_t)q * D + d];
  }
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    if (F) s.F[(size_t)c * st + p] = F[(size_t)q * D * D + c];
    if (C) s.C[(size_t)c * st + p] = C[(size_t)q * D * D + c];
  }
  if (Jp) s.Jp[p] = Jp[q];
}

// ---------------------------------------------------------------------------------------
// Sorting slots by grid cell (a one-digit counting sort over the (res+1)^dim cell keys):
// keys + ranks, exclusive scan of the per-cell counts, then every field moves to
// start[key] + rank in the other buffer.
// ---------------------------------------------------------------------------------------
template <int D>
__global__ void sort_keys_kernel(const float *__restrict__ xs, int stride, Params P,
                                 int *__restrict__ key, int *__restrict__ rank,
                                 int *__restrict__ count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= P.n) return;
  int b[D];
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int bd = __float2int_rz(xs[(size_t)d * stride + p] * P.inv_dx - 0.5f);
    b[d] = min(max(bd, 0), P.N - 1);
  }
  const int k = (int)flat_index<D>(b, P.N);
  key[p] = k;
  rank[p] = atomicAdd(count + k, 1);
}

template <int D>
__global__ void sort_move_kernel(PState src, PState dst, int n, const float4 *__restrict__ pay_src,
                                 float4 *__restrict__ pay_dst, const int *__restrict__ key,
                                 const int *__restrict__ rank, const int *__restrict__ start) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int q = start[key[p]] + rank[p];
  const int ss = src.stride, ds = dst.stride;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    dst.x[(size_t)d * ds + q] = src.x[(size_t)d * ss + p];
    dst.v[(size_t)d * ds + q] = src.v[(size_t)d * ss + p];
  }
#pragma unroll
  for (int c = 0; c < D * D; ++c) {
    dst.F[(size_t)c * ds + q] = src.F[(size_t)c * ss + p];
    dst.C[(size_t)c * ds + q] = src.C[(size_t)c * ss + p];
  }
  dst.Jp[q] = src.Jp[p];
  dst.mass[q] = src.mass[p];
  dst.vol[q] = src.vol[p];
  dst.id[q] = src.id[p];
  if (src.mat) dst.mat[q] = src.mat[p];
  constexpr int R = PayloadRecs<D>::value;
#pragma unroll
  for (int r = 0; r < R; ++r) pay_dst[(size_t)q * R + r] = pay_src[(size_t)p * R + r];
}

// ---------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------
inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

template <int D>
void launch_prepare(const PState &s, const Params &P, float4 *pay, bool ref, cudaStream_t st) {
  if (P.n == 0) return;
  if (ref)
    prepare_payload_kernel<D, true><<<blocks_for(P.n, 256), 256, 0, st>>>(s, P, pay);
  else
    prepare_payload_kernel<D, false><<<blocks_for(P.n, 256), 256, 0, st>>>(s, P, pay);
}

template <int D>
void launch_p2g(const float4 *pay, const Params &P, float4 *grid, int *err, int K, cudaStream_t st) {
  if (P.n == 0) return;
  const int threads = 128;
  switch (K) {
    case 4: p2g_kernel<D, 4><<<blocks_for((P.n + 3) / 4, threads), threads, 0, st>>>(pay, P, grid, err); break;
    case 16: p2g_kernel<D, 16><<<blocks_for((P.n + 15) / 16, threads), threads, 0, st>>>(pay, P, grid, err); break;
    default: p2g_kernel<D, 8><<<blocks_for((P.n + 7) / 8, threads), threads, 0, st>>>(pay, P, grid, err); break;
  }
}

template <int D>
void launch_g2p(const PState &s, const Params &P, const float4 *grid, float4 *pay, int *err,
                bool ref, cudaStream_t st) {
  if (P.n == 0) return;
  if (ref)
    g2p_kernel<D, true><<<blocks_for(P.n, 128), 128, 0, st>>>(s, P, grid, pay, err);
  else
    g2p_kernel<D, false><<<blocks_for(P.n, 128), 128, 0, st>>>(s, P, grid, pay, err);
}

template <int D>
void launch_export_grid(const float4 *grid, const Params &P, float *vel, float *mass, cudaStream_t st) {
  export_grid_kernel<D><<<blocks_for(P.nodes, 256), 256, 0, st>>>(grid, P, vel, mass);
}

template <int D>
void launch_export_particles(const PState &s, int n, float *x, float *v, float *F, float *C,
                             float *Jp, cudaStream_t st) {
  if (n == 0) return;
  export_particles_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(s, n, x, v, F, C, Jp);
}

template <int D>
void launch_import_particles(const PState &s, int n, const float *x, const float *v,
                             const float *F, const float *C, const float *Jp, cudaStream_t st) {
  if (n == 0) return;
  import_particles_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(s, n, x, v, F, C, Jp);
}

template <int D>
void launch_sort_keys(const PState &s, const Params &P, int *key, int *rank, int *count, cudaStream_t st) {
  if (P.n == 0) return;
  sort_keys_kernel<D><<<blocks_for(P.n, 256), 256, 0, st>>>(s.x, s.stride, P, key, rank, count);
}

template <int D>
void launch_sort_move(const PState &src, const PState &dst, int n, const float4 *pay_src,
                      float4 *pay_dst, const int *key, const int *rank, const int *start,
                      cudaStream_t st) {
  if (n == 0) return;
  sort_move_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(src, dst, n, pay_src, pay_dst, key, rank, start);
}

#define MPM_INSTANTIATE(D)                                                                      \
  template void launch_prepare<D>(const PState &, const Params &, float4 *, bool, cudaStream_t); \
  template void launch_p2g<D>(const float4 *, const Params &, float4 *, int *, int, cudaStream_t); \
  template void launch_g2p<D>(const PState &, const Params &, const float4 *, float4 *, int *,   \
                              bool, cudaStream_t);                                              \
  template void launch_export_grid<D>(const float4 *, const Params &, float *, float *,         \
                                      cudaStream_t);                                            \
  template void launch_export_particles<D>(const PState &, int, float *, float *, float *,      \
                                           float *, float *, cudaStream_t);                     \
  template void launch_import_particles<D>(const PState &, int, const float *, const float *,   \
                                           const float *, const float *, const float *,         \
                                           cudaStream_t);                                       \
  template void launch_sort_keys<D>(const PState &, const Params &, int *, int *, int *,        \
                                    cudaStream_t);                                              \
  template void launch_sort_move<D>(const PState &, const PState &, int, const float4 *,        \
                                    float4 *, const int *, const int *, const int *, cudaStream_t);

}  // namespace mpm
