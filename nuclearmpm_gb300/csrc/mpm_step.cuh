// Kernels of one MLS-MPM step and of the host<->device transfers, templated on the
// dimension; step2d.cu / step3d.cu instantiate them.
//
// Step k (the reference's advance(): p2g, grid_op, g2p; src/nclr.h:80-84) runs as
//   grid_sweep:  V = grid_op(G) (normalise, gravity, clamp, sticky boundary), G = 0
//   g2p2g:       per block of particles: G2P of step k from a shared-memory tile of V,
//                F/C/Jp update, then the P2G of step k+1 from the updated particle into a
//                shared-memory tile of G, flushed once per block with vector reductions.
// The P2G of the first step after an upload is g2p2g in its P2G-only mode.
#pragma once

#include <algorithm>
#include <type_traits>
#include <utility>

#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

// Programmatic dependent launch: a kernel launched by launch_overlapped may start while the
// kernel before it in the stream drains.  wait_prior_grid() holds it until that kernel has
// finished and its writes are visible (a no-op for an ordinary launch), and
// allow_next_grid() lets the kernel after it launch once every CTA of this one has run it.
// Used for the grid sweeps and every fused launch: 3D jelly 164 -> 159 us per step in CUDA
// graphs, the 256-scene 2D batch 2-4% faster.  The FP64 snow fix-up launches as before: with
// it overlapped too, the scenes that have fix-ups ran 5-13% slower (the next kernel's CTAs
// wait on SMs that the FP64-bound fix-up runs on).
__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void allow_next_grid() { asm volatile("griddepcontrol.launch_dependents;"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_overlapped(void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem,
                              cudaStream_t st, Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// Threads that work on one item of the fused kernel (a grid block, or a chunk of thin-block
// particles): the whole CTA, except in 2D batches.  There the tiles are small (2.3 KB), and a
// block of a few hundred particles runs in passes of 128, with each half of the CTA on its
// own item, tiles and barrier.  That replaces a 256-thread pass and a mostly idle second one
// (measured on 256 mixed scenes: 1.50-1.58e10 particle-steps/s against 1.37e10; one warp per
// item measured 3x slower, and the half-CTA items slow a single 2D simulation's tile path).
// kItem (batches): the threads per item chosen instead (128 or 256; 0 = the default above),
// a knob of the autotuner.
template <int D, bool kBatch, int kItem = 0>
__host__ __device__ constexpr int g2p2g_group() {
  return kItem ? kItem : ((D == 2 && kBatch) ? kG2P2GThreads / 2 : kG2P2GThreads);
}

// 0 <= v <= hi, as one unsigned compare that no large v (a saturated float-to-int conversion
// of a huge position) can overflow into passing.
__device__ __forceinline__ bool in_range(int v, int hi) { return (unsigned)v <= (unsigned)hi; }

template <int D>
__device__ __forceinline__ void stencil_offset(int o, int &oi, int &oj, int &ok) {
  oi = (D == 3) ? o / 9 : o / 3;
  oj = (D == 3) ? (o / 3) % 3 : o % 3;
  ok = (D == 3) ? o % 3 : 0;
}

// Flat index of stencil node o relative to the node of flat index f0 (the reference's index
// arithmetic, src/nclr.h:141-142,152: per-axis offsets folded into one flat index).
template <int D>
__device__ __forceinline__ int64_t stencil_flat(int64_t f0, int o, int N) {
  int oi, oj, ok;
  stencil_offset<D>(o, oi, oj, ok);
  return (D == 3) ? f0 + ((int64_t)oi * N + oj) * N + ok : f0 + (int64_t)oi * N + oj;
}

// Shared-memory index of tile-local node (i, j, k).
template <int D>
__device__ __forceinline__ int tile_index(int i, int j, int k) {
  using Tl = Tiling<D>;
  if (D == 3) return i * Tl::SX + j * Tl::SY + k;
  return i * Tl::SX + j;
}

template <int D>
__device__ __forceinline__ int tile_offset(int o) {
  int oi, oj, ok;
  stencil_offset<D>(o, oi, oj, ok);
  return tile_index<D>(oi, oj, ok);
}

// The reference's compute_fused_momentum (src/nclr.h:160-165) gives node o
//   weight_o * (m v + A dpos_o) and weight_o * m,   dpos_o = (o - fx) dx.
// p2g_terms rewrites a particle's m v and A once into q0 = m v - A fx dx (the bracket at
// o = 0) and A dx, so that a node's bracket is q0 + sum_d o_d (A dx)[:, d] with constant o_d:
// a few adds per node instead of a matrix-vector product (the two differ only in rounding).
template <int D>
__device__ __forceinline__ void p2g_terms(const float fx[D], float dx, float mv[D], Mat<D> &A) {
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float afx = A.a[r][0] * fx[0];
#pragma unroll
    for (int k = 1; k < D; ++k) afx += A.a[r][k] * fx[k];
    mv[r] -= afx * dx;  // q0
#pragma unroll
    for (int k = 0; k < D; ++k) A.a[r][k] *= dx;  // A dx
  }
}

// One node's contribution from the terms of p2g_terms: c[0..D) the momentum, c[3] the mass.
template <int D>
__device__ __forceinline__ void p2g_contrib(int o, const float w[3][D], const float q0[D], float m,
                                            const Mat<D> &Adx, float c[4]) {
  int oi, oj, ok;
  stencil_offset<D>(o, oi, oj, ok);
  const int oo[3] = {oi, oj, ok};
  float weight = w[oi][0] * w[oj][1];
  if (D == 3) weight = weight * w[ok][D - 1];
  c[2] = 0.0f;
#pragma unroll
  for (int r = 0; r < D; ++r) {
    float q = q0[r];
#pragma unroll
    for (int k = 0; k < D; ++k) {
      if (oo[k] == 1) q += Adx.a[r][k];
      if (oo[k] == 2) q += 2.0f * Adx.a[r][k];
    }
    c[r] = weight * q;
  }
  c[3] = weight * m;
}

// The G2P gather (src/nclr.h:197-225) over the 3^dim stencil nodes:
//   v += sum_o W_o g_o,   C += sum_o W_o g_o (o - fx)^T,   W_o = prod_d w[o_d][d],
// factored by axis -- sums over the last axis first, then the middle one, then the first --
// which is the same algebra in about half the multiply-adds of the node-by-node form (the
// two differ only in rounding).  load(o) returns node o's {v, m}; the caller scales C by
// 4 inv_dx once at the end (the reference scales every term).
template <int D, class Load>
__device__ __forceinline__ void g2p_gather(const Load &load, const float fx[D],
                                           const float w[3][D], float v[D], Mat<D> &C) {
  float wl[3], wld[3];  // last axis: weight, and weight times the node's distance
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    wl[k] = w[k][D - 1];
    wld[k] = w[k][D - 1] * ((float)k - fx[D - 1]);
  }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    float a[3] = {0.0f, 0.0f, 0.0f}, bl[3] = {0.0f, 0.0f, 0.0f}, bm[3] = {0.0f, 0.0f, 0.0f};
    if constexpr (D == 3) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        float aj[3] = {0.0f, 0.0f, 0.0f}, bj[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float4 g = load(i * 9 + j * 3 + k);
          const float gv[3] = {g.x, g.y, g.z};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            aj[c] += wl[k] * gv[c];
            bj[c] += wld[k] * gv[c];
          }
        }
        const float wm = w[j][1], wmd = w[j][1] * ((float)j - fx[1]);
#pragma unroll
        for (int c = 0; c < 3; ++c) {
          a[c] += wm * aj[c];
          bm[c] += wmd * aj[c];
          bl[c] += wm * bj[c];
        }
      }
    } else {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float4 g = load(i * 3 + j);
        const float gv[2] = {g.x, g.y};
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          a[c] += wl[j] * gv[c];
          bl[c] += wld[j] * gv[c];
        }
      }
    }
    const float wf = w[i][0], wfd = w[i][0] * ((float)i - fx[0]);
#pragma unroll
    for (int c = 0; c < D; ++c) {
      v[c] += wf * a[c];
      C.a[c][0] += wfd * a[c];
      if constexpr (D == 3) C.a[c][1] += wf * bm[c];
      C.a[c][D - 1] += wf * bl[c];
    }
  }
}

template <int D>
__device__ __forceinline__ void scale_mat(Mat<D> &C, float c) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) C.a[i][j] *= c;
}

// FP64 threshold of the snow clamp (see snow_clamp_needs_fp64): the FP32 clamp's own error
// measured about 2e-7 per unit of this gain, so below 50 it stays within about 1e-5.
constexpr float kClampFP64Gain = 50.0f;

// Whether the snow clamp of F_hat (FP32 signed singular values sig, decreasing in magnitude)
// must be recomputed in FP64.  With det F_hat < 0 the last singular value s_l is negative,
// and the clamp lifts it to a positive value: the clamped F then depends on F_hat through the
// divided difference (f(s_p) + f(s_l)) / (s_p + s_l) of the clamp f over the last pair, which
// grows without bound as |s_l| approaches s_p (the clamped F is discontinuous at |s_l| = s_p,
// where the SVD's choice of the vector that carries the sign flips).  FP32 rounding of the SVD
// (about eps s_1) is amplified by that factor; where the gain f s_1 / (s_p + s_l) passes
// kClampFP64Gain the clamp is recomputed in FP64.  With s_l >= 0 the map is 1-Lipschitz in
// F_hat and FP32 suffices.
template <int D, bool kRef>
__device__ __forceinline__ bool snow_clamp_needs_fp64(const float sig[D]) {
  if constexpr (D == 2 && kRef) return false;  // that 2D SVD keeps sigma >= 0 (no sign fix)
  const float sl = sig[D - 1], sp = sig[D - 2];
  if (!(sl < 0.0f)) return false;
  const float f = clampf_(sp, kSnowLo, kSnowHi) + clampf_(sl, kSnowLo, kSnowHi);
  return f * sig[0] > kClampFP64Gain * (sp + sl);
}

// The snow clamp and Jp update of src/nclr.h:237-250 in FP64 from the FP32 F_hat (exact in
// double): SVD, clamp, F = U clamp(S) V^T, Jp = clamp(Jp det F_hat / det F, 0.6, 20), and the
// polar rotation of the clamped F (3D: U V^T).  V0: the FP32 right singular vectors, where the
// 3D Jacobi sweeps start.  Not inlined: it runs for a few particles, and its doubles stay out
// of the calling kernel's register budget.
template <int D, bool kRef>
__device__ __noinline__ void snow_clamp_fp64(const Mat<D> *Fh_in, const Mat<D> *V0, float *Jp,
                                             Mat<D> *F_out, Mat<D> *R_out) {
  double A[D][D], U[D][D], V[D][D], sg[D];
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) A[i][j] = (double)Fh_in->a[i][j];
  if constexpr (D == 3) {
    double W[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) W[i][j] = (double)V0->a[i][j];
    detail::svd3_t<true, double>(A, U, sg, V, W);
  } else {
    svd2_t<kRef, double>(A, U, sg, V);
  }
  double Fn[D][D];
#pragma unroll
  for (int d = 0; d < D; ++d) sg[d] = fmin(fmax(sg[d], (double)kSnowLo), (double)kSnowHi);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k < D; ++k) v += U[i][k] * sg[k] * V[j][k];
      Fn[i][j] = v;
    }
  double old_J, new_J;
  if constexpr (D == 3) {
    old_J = A[0][0] * (A[1][1] * A[2][2] - A[1][2] * A[2][1]) -
            A[0][1] * (A[1][0] * A[2][2] - A[1][2] * A[2][0]) +
            A[0][2] * (A[1][0] * A[2][1] - A[1][1] * A[2][0]);
    new_J = Fn[0][0] * (Fn[1][1] * Fn[2][2] - Fn[1][2] * Fn[2][1]) -
            Fn[0][1] * (Fn[1][0] * Fn[2][2] - Fn[1][2] * Fn[2][0]) +
            Fn[0][2] * (Fn[1][0] * Fn[2][1] - Fn[1][1] * Fn[2][0]);
  } else {
    old_J = A[0][0] * A[1][1] - A[0][1] * A[1][0];
    new_J = Fn[0][0] * Fn[1][1] - Fn[0][1] * Fn[1][0];
  }
  *Jp = (float)fmin(fmax((double)*Jp * old_J / new_J, 0.6), 20.0);
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) F_out->a[i][j] = (float)Fn[i][j];
  if constexpr (D == 3) {
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j)
        R_out->a[i][j] = (float)(U[i][0] * V[j][0] + U[i][1] * V[j][1] + U[i][2] * V[j][2]);
  } else {
    *R_out = polar_rotation(*F_out);
  }
}

// The FP32 snow clamp (src/nclr.h:237-250) of F_hat = U S V^T: F_hat becomes U clamp(S) V^T,
// Jp is updated, and R receives the polar rotation of the result (3D: U V^T; 2D when need_R).
template <int D>
__device__ __forceinline__ void snow_clamp_fp32(const Mat<D> &U, float sig[D], const Mat<D> &Vm,
                                                Mat<D> &Fh, float &Jp, Mat<D> &R, bool need_R) {
#pragma unroll
  for (int d = 0; d < D; ++d) sig[d] = clampf_(sig[d], kSnowLo, kSnowHi);
  const float old_J = det(Fh);
  Fh = usv<D>(U, sig, Vm);
  Jp = clampf_(Jp * old_J / det(Fh), 0.6f, 20.0f);
  if constexpr (D == 3) {
    R = uvt<3>(U, Vm);  // the clamped sigma are positive: F = (U V^T)(V S V^T)
  } else {
    if (need_R) R = polar_rotation(Fh);
  }
}

// The F update and plasticity of G2P (src/nclr.h:228-259) from the gathered C; returns the
// rotation R of the updated F (the polar factor the next step's corotated stress needs; with
// need_R false -- the neo-Hookean stress -- whatever is at hand).  A snow clamp that needs FP64
// is, with kDefer (the fused kernel), appended to `fix` -- the FP64 fix-up launch that follows
// redoes it, and this launch carries on with the FP32 result -- and otherwise recomputed in
// place (the small-scene kernels).
template <int D, bool kRef, bool kDefer = false>
__device__ __forceinline__ Mat<D> update_F(const Mat<D> &C, Mat<D> &F, float &Jp, int material,
                                           float dt, bool need_R = true,
                                           const SnowFix *fix = nullptr, int slot = 0) {
  Mat<D> M;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M.a[i][j] = diag_one<D, kRef>(i, j) + dt * C.a[i][j];
  Mat<D> Fh = mat_mul<D>(M, F);
  Mat<D> R = Fh;
  // jelly and liquid take the polar rotation of their new F from one call after the branch
  // (one inlined SVD for both in the kernels that read the material per particle)
  bool polar = false;
  if (material == kJelly) {
    polar = need_R;
  } else if (material == kLiquid) {
    // src/nclr.h:253-257: F = diag(1) with F_00 = J = prod sigma.  The signed SVD's product
    // is det F_hat (U, V rotations; |det F_hat| under the 2D reference physics, whose SVD
    // keeps sigma >= 0), taken here from the determinant: no SVD, and no error from the
    // singular values' rounding where F_hat is nearly singular (the reference physics' 3D
    // diag(1, 1, 0) makes its third row O(dt C)).
    float J = det(Fh);
    if (D == 2 && kRef) J = fabsf(J);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) Fh.a[i][j] = diag_one<D, kRef>(i, j);
    Fh.a[0][0] = J;
    R = Fh;
    polar = need_R;
  } else {
    Mat<D> U, Vm;
    float sig[D];
    if constexpr (D == 3) {
      svd3(Fh, U, sig, Vm);
    } else {
      svd2<kRef>(Fh, U, sig, Vm);
    }
    const bool fp64 = material == kSnow && snow_clamp_needs_fp64<D, kRef>(sig);
    if (!kDefer && fp64) {
      const Mat<D> Fh_in = Fh;
      snow_clamp_fp64<D, kRef>(&Fh_in, &Vm, &Jp, &Fh, &R);
    } else if (material == kSnow) {
      if (kDefer && fp64 && fix) {  // for the fix-up launch: slot, F_hat and Jp before the clamp
        const int i = atomicAdd(fix->count, 1);
        if (i < fix->cap) {
          fix->slot[i] = slot;
#pragma unroll
          for (int a = 0; a < D; ++a)
#pragma unroll
            for (int b = 0; b < D; ++b) fix->Fh[((size_t)i * D + a) * D + b] = Fh.a[a][b];
          fix->Jp[i] = Jp;
        }
      }
      snow_clamp_fp32<D>(U, sig, Vm, Fh, Jp, R, need_R);
    }
  }
  if (polar) R = polar_R(Fh);
  F = Fh;
  return R;
}

// Grid-block activity flags (one byte per block of BS^dim nodes, the same blocks as the
// particle blocks): bit 0 = the pending P2G accumulator G has contributions there, bit 1 = V
// (the last step's grid) may be non-zero there.  Writers of G set bit 0 with a plain
// read-modify-write (every writer stores the same value, and bit 1 only changes in the
// sweep); the sweep visits only flagged blocks.
enum : uint8_t { kPending = 1, kVNonzero = 2 };

// Marks the blocks the stencil at base[] adds to (slow paths).  A stencil whose per-axis
// index leaves the grid wraps into another row (the reference's flat indexing): then every
// node's block is marked from its flat index, else the <= 2 blocks per axis.
template <int D>
__device__ __forceinline__ void mark_node(uint8_t *flags, int64_t f, const Params &P);

template <int D>
__device__ void mark_stencil(uint8_t *flags, const int base[D], const Params &P) {
  constexpr int BS = Tiling<D>::BS;
  bool wraps = false;
#pragma unroll
  for (int d = 0; d < D; ++d) wraps |= base[d] < 0 || base[d] + 2 >= P.N;
  if (wraps) {
    const int64_t f0 = flat_index<D>(base, P.N);
    constexpr int S = (D == 3) ? 27 : 9;
    for (int o = 0; o < S; ++o) {
      int oi = (D == 3) ? o / 9 : o / 3, oj = (D == 3) ? (o / 3) % 3 : o % 3, ok = (D == 3) ? o % 3 : 0;
      const int64_t f = (D == 3) ? f0 + ((int64_t)oi * P.N + oj) * P.N + ok : f0 + (int64_t)oi * P.N + oj;
      if (f >= 0 && f < P.nodes) mark_node<D>(flags, f, P);
    }
    return;
  }
  const int i0 = base[0] / BS, i1 = (base[0] + 2) / BS;
  const int j0 = base[1] / BS, j1 = (base[1] + 2) / BS;
  const int k0 = base[D - 1] / BS, k1 = (base[D - 1] + 2) / BS;
  for (int i = i0; i <= i1; ++i)
    for (int j = j0; j <= j1; ++j) {
      if constexpr (D == 2) {
        flags[i * P.nb + j] |= kPending;
      } else {
        for (int k = k0; k <= k1; ++k) flags[(i * P.nb + j) * P.nb + k] |= kPending;
      }
    }
}

// Marks the block of node f.
template <int D>
__device__ __forceinline__ void mark_node(uint8_t *flags, int64_t f, const Params &P) {
  constexpr int BS = Tiling<D>::BS;
  int idx[D];
  unflatten<D>(f, P.N, idx);
  int blk = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) blk = blk * P.nb + idx[d] / BS;
  flags[blk] |= kPending;
}

// ---------------------------------------------------------------------------------------
// grid_sweep: grid_op (src/nclr.h:263-310) on the flagged blocks: V = update(G), G = 0, and
// the flags roll over (pending -> V non-zero).  Blocks never flagged hold V = 0 = update(0)
// (a massless node's velocity is zero and stays zero through the boundary rule).  Eight lanes
// per block (eight nodes each), four blocks per warp at a time; also resets the g2p2g work
// counter.
// ---------------------------------------------------------------------------------------
// Scene of global block gb, and the block's first node per axis inside that scene.
template <int D>
__device__ __forceinline__ int block_origin(int gb, const Scene *scenes,
                                            const uint16_t *block_scene, int bc[D]) {
  const int sid = block_scene ? (int)block_scene[gb] : 0;
  int r = gb - scenes[sid].block_off;
  const int nb = scenes[sid].P.nb;
#pragma unroll
  for (int d = D - 1; d >= 0; --d) {
    bc[d] = (r % nb) * Tiling<D>::BS;
    r /= nb;
  }
  return sid;
}

// kBatch: the scene of each block from the scene table; otherwise the one scene's parameters
// come by value (no dependent loads before the nodes').
template <int D, bool kBatch>
__global__ void __launch_bounds__(256) grid_sweep_kernel(float4 *__restrict__ G,
                                                         float4 *__restrict__ V,
                                                         uint8_t *__restrict__ flags,
                                                         const Scene *__restrict__ scenes,
                                                         const uint16_t *__restrict__ block_scene,
                                                         Params P0, int total_blocks,
                                                         int *__restrict__ work,
                                                         int *__restrict__ fix_count) {
  constexpr int BS = Tiling<D>::BS;
  constexpr int BN = (D == 3) ? BS * BS * BS : BS * BS;  // nodes per block
  constexpr int kLanes = 8, kPer = BN / kLanes;          // lanes per block, nodes per lane
  static_assert(BN % kLanes == 0, "whole nodes per lane");
  wait_prior_grid();  // the fused launch before it wrote G and the flags
  allow_next_grid();
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    *work = 0;
    if (fix_count) *fix_count = 0;  // the FP64 snow list of the step that follows
  }
  const int lane = threadIdx.x & 31, sub = lane / kLanes, l8 = lane % kLanes;
  const int warps = gridDim.x * (blockDim.x >> 5);
  const int wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  // This warp's blocks are wid, wid + warps, ...; their flags are read 32 at a time (one per
  // lane) and only the flagged ones are visited, four at a time (the sub-th lowest flagged
  // block goes to lanes 8 sub .. 8 sub + 7), so neither the flag loads nor the blocks chain
  // one after another.
  for (int k0 = 0; wid + k0 * warps < total_blocks; k0 += 32) {
    const int mine = wid + (k0 + lane) * warps;
    const uint8_t fl_l = mine < total_blocks ? flags[mine] : 0;
    unsigned todo = __ballot_sync(0xffffffffu, fl_l != 0);
    while (todo) {
      unsigned pick = todo;
      for (int i = 0; i < sub; ++i) pick &= pick - 1;  // drop the sub lowest
      const int k = pick ? __ffs(pick) - 1 : -1;
#pragma unroll
      for (int i = 0; i < 32 / kLanes; ++i) todo &= todo - 1;
      const uint8_t fl = __shfl_sync(0xffffffffu, fl_l, k < 0 ? 0 : k);
      if (k < 0) continue;
      const int gb = wid + (k0 + k) * warps;
      int bc[D];
      const int sid = kBatch ? block_origin<D>(gb, scenes, block_scene, bc) : 0;
      if constexpr (!kBatch) {
        int r = gb;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          bc[d] = (r % P0.nb) * BS;
          r /= P0.nb;
        }
      }
      const Params &P = kBatch ? scenes[sid].P : P0;
      const int64_t off = kBatch ? scenes[sid].node_off : 0;
      float4 *Gs = G + off;
      float4 *Vs = V + off;
      int f[kPer];  // node within the scene (res <= 1024: below 2^31)
      float4 g[kPer];
#pragma unroll
      for (int j = 0; j < kPer; ++j) {  // every load first
        const int t = l8 + kLanes * j;
        int idx[D];
        bool in = true;
        int r = t;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          idx[d] = bc[d] + r % BS;
          r /= BS;
          in &= idx[d] < P.N;
        }
        f[j] = in ? (int)flat_index<D>(idx, P.N) : -1;
        g[j] = in ? Gs[f[j]] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
#pragma unroll
      for (int j = 0; j < kPer; ++j) {
        if (f[j] < 0) continue;
        const int t = l8 + kLanes * j;
        int idx[D];
        int r = t;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          idx[d] = bc[d] + r % BS;
          r /= BS;
        }
        float v[D], m;
        grid_update<D>(g[j], idx, P, v, m);
        Vs[f[j]] = make_float4(v[0], v[1], D == 3 ? v[D - 1] : 0.0f, m);
        Gs[f[j]] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
      if (l8 == 0) flags[gb] = (fl & kPending) ? kVNonzero : 0;
    }
  }
}

// Drops the pending accumulation (after the particle state was replaced): G = 0 on the
// pending blocks, pending flags cleared; V and its flags stay (they are grid()).
template <int D>
__global__ void __launch_bounds__(256) discard_pending_kernel(float4 *__restrict__ G,
                                                              uint8_t *__restrict__ flags,
                                                              const Scene *__restrict__ scenes,
                                                              const uint16_t *__restrict__ block_scene,
                                                              int total_blocks) {
  constexpr int BS = Tiling<D>::BS;
  constexpr int BN = (D == 3) ? BS * BS * BS : BS * BS;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  for (int gb = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); gb < total_blocks;
       gb += warps) {
    const uint8_t fl = flags[gb];
    if (!(fl & kPending)) continue;
    int bc[D];
    const int sid = block_origin<D>(gb, scenes, block_scene, bc);
    const int N = scenes[sid].P.N;
    float4 *Gs = G + scenes[sid].node_off;
    for (int t = lane; t < BN; t += 32) {
      int idx[D];
      bool in = true;
      int r = t;
#pragma unroll
      for (int d = D - 1; d >= 0; --d) {
        idx[d] = bc[d] + r % BS;
        r /= BS;
        in &= idx[d] < N;
      }
      if (in) Gs[flat_index<D>(idx, N)] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if (lane == 0) flags[gb] = fl & (uint8_t)~kPending;
  }
}

// ---------------------------------------------------------------------------------------
// g2p2g: persistent CTAs take blocks of particles from the active-block list.  For each
// block: stage the (BS+4)^dim node tile of V around it, run G2P for its particles (those
// sorted into it; a particle that has since drifted out of the tile, or whose stencil leaves
// the grid on some axis, reads V in global memory with the reference's flat-index arithmetic),
// update F/C/Jp, compute the next stress and scatter the next P2G into a shared-memory tile
// of G (again with a global fallback), then flush the tile with one vector reduction per
// touched node.
// ---------------------------------------------------------------------------------------
// kMode: kStep (G2P + next P2G), kFinalStep (also writes v and C), kP2GOnly (the P2G of the
// coming step from the stored state, after an upload; the particles are sorted already),
// kG2PFinal (the final step without the next P2G: for callers that replace the state before
// the next step, whose pending P2G would be thrown away; no G tiles, no polar rotation).
enum : int { kStep = kModeStep, kFinalStep = kModeFinalStep, kP2GOnly = kModeP2GOnly,
             kG2PFinal = kModeG2PFinal };

// kBatch: several scenes (per-block parameters from the scene table, staged in shared memory)
// or one (its parameters are a kernel argument: constant-bank operands, no registers).
template <int D, bool kRef, int kMode, bool kBatch, int kMat = -1, int kItem = 0>
// 3D: two CTAs per SM (the tiles take 106 KB of shared memory each), three for the G2P-only
// step (one 12 KB tile); 2D: four, which keeps the 2D kernel within 64 registers without
// spills.  kMat >= 0 fixes every particle's material at compile time (a single simulation
// without per-particle materials): the other materials' branches drop out of the code.
__global__ void __launch_bounds__(kG2P2GThreads, D == 3 ? (kMode == kG2PFinal ? 3 : 2) : 4)
g2p2g_kernel(
    PState s, Params P0, const Scene *__restrict__ scenes, const uint16_t *__restrict__ block_scene,
    const float4 *__restrict__ Vall, float4 *__restrict__ Gall, uint8_t *__restrict__ flags_all,
    const int *__restrict__ blocks, const int *__restrict__ nactive,
    const int *__restrict__ bstart, const int *__restrict__ sparse, int *__restrict__ work,
    int *__restrict__ err, int next_slot, Record rec, SnowFix fix) {
  using Tl = Tiling<D>;
  constexpr int T = Tl::T, NODES = Tl::NODES, BS = Tl::BS, GS = Tl::SIZE;
  constexpr int S = (D == 3) ? 27 : 9;
  constexpr int kGroup = g2p2g_group<D, kBatch, kItem>();  // threads per item
  constexpr int kGroups = kG2P2GThreads / kGroup;  // items in flight per CTA
  constexpr int kWarps = kGroup / 32;              // warps per item, each with its G tile
  constexpr int kTiles = (kMode == kG2PFinal) ? 1 : 1 + kWarps;  // tiles per group
  static_assert(kBatch || kGroup == kG2P2GThreads, "the tail rule counts passes of the CTA");
  wait_prior_grid();  // the sweep before it wrote V, the flags and the item counter
  allow_next_grid();
  extern __shared__ float4 smem[];
  const int grp = threadIdx.x / kGroup, gtid = threadIdx.x % kGroup;
  float4 *vt = smem + grp * kTiles * GS;  // the group's V tile
  float4 *gt = vt + GS;                   // its kWarps private G tiles: [warp][SIZE]
  __shared__ int s_items[kGroups];
  __shared__ Params sPs[kGroups];  // each item's scene (shared: keeps registers for the math)
  __shared__ int64_t s_node_offs[kGroups];
  __shared__ int s_block_offs[kGroups];
  int &s_item = s_items[grp];
  Params &sP = sPs[grp];
  int64_t &s_node_off = s_node_offs[grp];
  int &s_block_off = s_block_offs[grp];
  // the barrier of one item's threads (a named barrier per group when the CTA has several)
  auto group_sync = [grp] {
    if constexpr (kGroups == 1)
      __syncthreads();
    else
      asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "n"(kGroup) : "memory");
  };
  const int st = s.stride;
  // work items: the dense blocks of the list, then chunks of kG2P2GThreads particles of the
  // sparse blocks (single simulations only; see compact_blocks_kernel)
  // the block list: nactive[0] blocks of more than one pass at its front, nactive[2] others at
  // its back (capacity nactive[3]; compact_blocks_kernel), taken in that order
  const int nfront = nactive[0], lcap = nactive[3];
  const int nact = nfront + nactive[2];
  auto block_at = [&](int it) { return blocks[it < nfront ? it : lcap - 1 - (it - nfront)]; };
  const int nsp = kBatch ? 0 : nactive[1];
  const int nitems = nact + (nsp + kGroup - 1) / kGroup;
  const int lane = threadIdx.x & 31;
  float4 *mytile = gt + (gtid >> 5) * GS;
  // The G tiles start clear and every item's flush clears what it read, so they are clear
  // again at the start of the next item (padding entries are never written).
  if constexpr (kMode != kG2PFinal)
    for (int t = gtid; t < kWarps * GS; t += kGroup) gt[t] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);

  // Single simulations: thread 0 claims item k+1 right after item k's particle loop, so the
  // claim's latency overlaps item k's flush, and publishes it in s_item after its own share
  // of the flush (everyone read s_item for item k before the tile-load barrier): three
  // barriers per item (measured up to 4% faster than claiming at the top; within noise on
  // the dense jelly scene).
  // Batches claim at the top, behind a barrier, as their per-item parameters sit in shared
  // memory that the flush still reads.
  int nx_it = 0;
  if (!kBatch && gtid == 0) s_item = atomicAdd(work, 1);
  for (;;) {
    if constexpr (kBatch) group_sync();
    if (kBatch && gtid == 0) {  // the next block of the list, and its scene
      const int it = atomicAdd(work, 1);
      s_item = it;
      if (kBatch && it < nact) {
        const int sid0 = (int)block_scene[block_at(it)];
        sP = scenes[sid0].P;
        s_node_off = scenes[sid0].node_off;
        s_block_off = scenes[sid0].block_off;
      }
    }
    group_sync();
    const int item = s_item;
    if (item >= nitems) return;
    // a sparse chunk: particles of blocks too thin for the tile to pay, one per thread,
    // gathered from V and scattered into G directly (CTA-uniform)
    const bool chunk = !kBatch && item >= nact;
    const int gb = chunk ? 0 : block_at(item);  // global block (scene-major)
    const int sid = kBatch ? (int)block_scene[gb] : 0;
    const Params &P = kBatch ? sP : P0;
    const int64_t node_off = kBatch ? s_node_off : 0;
    const int block_off = kBatch ? s_block_off : 0;
    const int N = P.N;
    int org[D];
    {
      int r = gb - block_off;
#pragma unroll
      for (int d = D - 1; d >= 0; --d) {
        org[d] = (r % P.nb) * BS - 1;
        r /= P.nb;
      }
    }
    const float4 *__restrict__ V = Vall + node_off;
    float4 *__restrict__ G = Gall + node_off;
    uint8_t *__restrict__ flags = flags_all + block_off;
    const int b = gb - block_off;
    int *err_now = err + 2 * sid, *err_next = err + 2 * sid + next_slot;
    // The block's particles, stored cell by cell in rounds (see sort_move_kernel), or a chunk's.
    const int c0 = (item - nact) * kGroup;
    const int p0 = chunk ? 0 : bstart[gb];
    int np = chunk ? min(kGroup, nsp - c0) : bstart[gb + 1] - p0;
    // A single simulation's block whose last pass would hold fewer than P.tail_max particles
    // left them to the chunks (compact_blocks_kernel): its item runs whole passes only.
    if (!kBatch && !chunk && np > kGroup && np % kGroup < P.tail_max) np -= np % kGroup;
    // A batch's thin block (fewer than P.thin_max particles) skips the tiles like a chunk:
    // gathered from V and scattered into G directly (CTA-uniform).
    const bool direct = chunk || (kBatch && np < P.thin_max);
    if (kMode != kP2GOnly && !direct) {
      for (int t = gtid; t < NODES; t += kGroup) {
        int g[D], l[3] = {0, 0, 0};
        bool in = true;
        int r = t;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          l[d] = r % T;
          g[d] = org[d] + l[d];
          r /= T;
          in &= g[d] >= 0 && g[d] < N;
        }
        vt[tile_index<D>(l[0], l[1], l[2])] =
            in ? __ldg(V + flat_index<D>(g, N)) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    }
    group_sync();

    // One particle per thread in slot order.  Every lane of a warp runs the same number of
    // iterations (the warp-wide steps below need them all).
    for (int j0 = 0; j0 < np; j0 += kGroup) {
      const int j = j0 + gtid;
      const bool valid = j < np;
      const int p = chunk ? (valid ? sparse[c0 + j] : 0) : p0 + j;
      // what the particle contributes to the next P2G
      bool fast_s = false;
      int tb_s = 0;
      float fx_s[D], w_s[3][D], mv[D], m = 0.0f;
      Mat<D> A;
      if (valid) {
        float x[D];
        Mat<D> F, C, R;
        float v[D], Jp;
        const int material = kMat >= 0 ? kMat : (s.mat ? (int)s.mat[p] : P.model);
        int base[D], lb[3] = {0, 0, 0};
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] = s.x[(size_t)d * st + p];
        if (kMode == kP2GOnly) {
#pragma unroll
          for (int d = 0; d < D; ++d) v[d] = s.v[(size_t)d * st + p];
          F = load_mat<D>(s.F, st, p);
          C = load_mat<D>(s.C, st, p);
          Jp = s.Jp[p];
          R = stress_R<D>(F, P, material);
        } else {
        // F and Jp are not needed before the gather has finished; loading them first lets
        // their global-memory latency overlap it (measured 3% off the 3D step)
        F = load_mat<D>(s.F, st, p);
        Jp = s.Jp[p];
        // ---- G2P of this step ----
        float fx[D], w[3][D];
        stencil<D>(x, P.inv_dx, base, fx, w);
        bool fast = !direct;
#pragma unroll
        for (int d = 0; d < D; ++d) {
          lb[d] = base[d] - org[d];
          fast &= in_range(lb[d], T - 3) && in_range(base[d], N - 3);
        }
        const int tb = tile_index<D>(lb[0], lb[1], lb[2]);
#pragma unroll
        for (int d = 0; d < D; ++d) v[d] = 0.0f;
#pragma unroll
        for (int i = 0; i < D; ++i)
#pragma unroll
          for (int jj = 0; jj < D; ++jj) C.a[i][jj] = 0.0f;
        if (fast) {
          g2p_gather<D>([&](int o) { return vt[tb + tile_offset<D>(o)]; }, fx, w, v, C);
        } else {  // outside the tile: straight from V, each node range-checked
          const int64_t f0 = flat_index<D>(base, N);
          g2p_gather<D>(
              [&](int o) {
                const int64_t f = stencil_flat<D>(f0, o, N);
                if (f >= 0 && f < P.nodes) return __ldg(V + f);
                atomicOr(err_now, kErrOutOfRange);
                return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
              },
              fx, w, v, C);
        }
        scale_mat<D>(C, P.cscale);
#pragma unroll
        for (int d = 0; d < D; ++d) x[d] += P.dt * v[d];  // advection, src/nclr.h:229
        R = update_F<D, kRef, true>(C, F, Jp, material, P.dt,
                                    kMode != kG2PFinal && P.stress == kCorotated,
                                    fix.count ? &fix : nullptr, p);
#pragma unroll
        for (int d = 0; d < D; ++d) s.x[(size_t)d * st + p] = x[d];
        store_mat<D>(s.F, st, p, F);
        s.Jp[p] = Jp;
        if (kMode == kFinalStep || kMode == kG2PFinal) {
#pragma unroll
          for (int d = 0; d < D; ++d) s.v[(size_t)d * st + p] = v[d];
          store_mat<D>(s.C, st, p, C);
          if (!kBatch && rec.x) {  // the recorded state, in the caller's order
            const size_t q = (size_t)s.id[p];
#pragma unroll
            for (int d = 0; d < D; ++d) {
              rec.x[q * D + d] = x[d];
              rec.v[q * D + d] = v[d];
            }
#pragma unroll
            for (int i = 0; i < D; ++i)
#pragma unroll
              for (int jj = 0; jj < D; ++jj) {
                rec.F[(q * D + i) * D + jj] = F.a[i][jj];
                rec.C[(q * D + i) * D + jj] = C.a[i][jj];
              }
            if (rec.Jp) rec.Jp[q] = Jp;
          }
        }
        }

        if constexpr (kMode != kG2PFinal) {
          // ---- P2G of the next step: stress, stencil ----
          m = s.mass[p];
          A = fused_affine<D>(F, R, C, Jp, m, s.vol[p], material, lame0(s, p, P), P);
          int *err_p2g = (kMode == kP2GOnly) ? err_now : err_next;
#pragma unroll
          for (int d = 0; d < D; ++d) mv[d] = v[d] * m;
          stencil<D>(x, P.inv_dx, base, fx_s, w_s);
          p2g_terms<D>(fx_s, P.dx, mv, A);  // mv, A now hold q0 and A dx
          fast_s = !direct;
#pragma unroll
          for (int d = 0; d < D; ++d) {
            lb[d] = base[d] - org[d];
            fast_s &= in_range(lb[d], T - 3) && in_range(base[d], N - 3);
          }
          tb_s = tile_index<D>(lb[0], lb[1], lb[2]);
          if (!fast_s) {  // outside the tile: straight to G
            const int64_t f0 = flat_index<D>(base, N);
#pragma unroll
            for (int o = 0; o < S; ++o) {
              const int64_t f = stencil_flat<D>(f0, o, N);
              if (f < 0 || f >= P.nodes) {
                atomicOr(err_p2g, kErrOutOfRange);
                continue;
              }
              float c[4];
              p2g_contrib<D>(o, w_s, mv, m, A, c);
              red_add_v4(G + f, c[0], c[1], c[2], c[3]);
            }
            mark_stencil<D>(flags, base, P);
          }
        }
      }
      // ---- P2G into this warp's tile, with plain read-modify-writes (one tile per item with
      // shared-memory FP32 atomics measured 2.5x slower, even at 3-4 CTAs per SM): the first
      // lane of each stencil base in the warp writes the tile, so every such lane writes a
      // different node for each stencil offset; __syncwarp orders the offsets.  A lane whose
      // base an earlier lane of the warp has (particles that drifted since the sort, or a
      // warp that spans two rounds of the slot order) adds its 27 (or 9) contributions straight
      // into G with vector reductions instead: no second pass of the dependent
      // read-modify-write chain for the whole warp, and its nodes lie in the blocks this item
      // flags anyway.  Measured against a second pass per repeated base: fused launch on the
      // 1M jelly scene 142 -> 126.5 us (reference physics), 153 -> 137 us (corrected),
      // corrected snow 170 -> 155 us, liquid + snow 1.27 -> 1.22 ms, the 256-scene 2D batch
      // 1.72-1.74e10 -> 1.94-1.97e10 particle-steps/s.
      if (direct || kMode == kG2PFinal) continue;  // nothing for the tile
      const bool tile_lane = valid && fast_s;
      const int key = tile_lane ? tb_s : -1 - lane;
      const unsigned same = __match_any_sync(0xffffffffu, key);
      const int rank = __popc(same & ((1u << lane) - 1u));
      {
        const bool act = tile_lane && rank == 0;
#pragma unroll
        for (int o = 0; o < S; ++o) {
          if (act) {
            float c[4];
            p2g_contrib<D>(o, w_s, mv, m, A, c);
            const int ti = tb_s + tile_offset<D>(o);
            float4 a = mytile[ti];
            a.x += c[0];
            a.y += c[1];
            a.z += c[2];
            a.w += c[3];
            mytile[ti] = a;
          }
          __syncwarp();
        }
      }
      if (tile_lane && rank > 0) {  // a base an earlier lane of the warp has: straight to G
        // (its base node from the tile index: lb = base - org per axis)
        int g[D];
        {
          int r = tb_s;
          if constexpr (D == 3) {
            g[0] = org[0] + r / Tl::SX;
            r %= Tl::SX;
            g[1] = org[1] + r / Tl::SY;
            g[2] = org[2] + r % Tl::SY;
          } else {
            g[0] = org[0] + r / Tl::SX;
            g[1] = org[1] + r % Tl::SX;
          }
        }
        const int64_t f0 = flat_index<D>(g, N);
#pragma unroll
        for (int o = 0; o < S; ++o) {
          float c[4];
          p2g_contrib<D>(o, w_s, mv, m, A, c);
          red_add_v4(G + stencil_flat<D>(f0, o, N), c[0], c[1], c[2], c[3]);
        }
      }
    }
    if (!kBatch && gtid == 0) nx_it = atomicAdd(work, 1);  // the next item (see above)
    if (direct || kMode == kG2PFinal) {  // its P2G went straight to G (and the flags)
      if (!kBatch && gtid == 0) s_item = nx_it;
      continue;
    }
    group_sync();

    for (int t = gtid; t < NODES; t += kGroup) {
      int g[D], l[3] = {0, 0, 0};
      bool in = true;
      int r = t;
#pragma unroll
      for (int d = D - 1; d >= 0; --d) {
        l[d] = r % T;
        g[d] = org[d] + l[d];
        r /= T;
        in &= g[d] >= 0 && g[d] < N;
      }
      const int ti = tile_index<D>(l[0], l[1], l[2]);
      float a[4] = {0.0f, 0.0f, 0.0f, 0.0f};
      bool touched = false;
#pragma unroll
      for (int wi = 0; wi < kWarps; ++wi) {
        const float4 g4 = gt[wi * GS + ti];
        a[0] += g4.x;
        a[1] += g4.y;
        a[2] += g4.z;
        a[3] += g4.w;
        touched |= g4.x != 0.0f || g4.y != 0.0f || g4.z != 0.0f || g4.w != 0.0f;
      }
      if (!touched) continue;
#pragma unroll
      for (int wi = 0; wi < kWarps; ++wi) gt[wi * GS + ti] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (a[0] == 0.0f && a[1] == 0.0f && a[2] == 0.0f && a[3] == 0.0f) continue;
      if (in) red_add_v4(G + flat_index<D>(g, N), a[0], a[1], a[2], a[3]);
    }
    // the tile spans node blocks b-1 .. b+1 on every axis
    if (gtid < ((D == 3) ? 27 : 9)) {
      int nbc[3] = {0, 0, 0}, r = b;
#pragma unroll
      for (int d = D - 1; d >= 0; --d) {
        nbc[d] = r % P.nb;
        r /= P.nb;
      }
      const int t = gtid;
      const int di = (D == 3) ? t / 9 - 1 : t / 3 - 1, dj = (D == 3) ? (t / 3) % 3 - 1 : t % 3 - 1;
      const int dk = (D == 3) ? t % 3 - 1 : 0;
      const int bi = nbc[0] + di, bj = nbc[1] + dj, bk = nbc[D - 1] + dk;
      if (bi >= 0 && bi < P.nb && bj >= 0 && bj < P.nb && (D == 2 || (bk >= 0 && bk < P.nb)))
        flags[(D == 3) ? (bi * P.nb + bj) * P.nb + bk : bi * P.nb + bj] |= kPending;
    }
    if (!kBatch && gtid == 0) s_item = nx_it;
  }
}

// Dynamic shared memory of g2p2g: per item group, the V tile plus one G tile per warp (the V
// tile alone for kG2PFinal, which has no P2G and runs single simulations only).
template <int D, bool kBatch, int kItem = 0>
constexpr size_t g2p2g_smem_bytes() {
  return sizeof(float4) * Tiling<D>::SIZE * (kG2P2GThreads / g2p2g_group<D, kBatch, kItem>()) *
         (1 + g2p2g_group<D, kBatch, kItem>() / 32);
}
template <int D>
constexpr size_t g2p_final_smem_bytes() {
  return sizeof(float4) * Tiling<D>::SIZE;
}

// ---------------------------------------------------------------------------------------
// grid() export (src/nclr.h:87): V is already the post-update grid; copy it out.
// ---------------------------------------------------------------------------------------
template <int D>
__global__ void copy_vgrid_kernel(const float4 *__restrict__ V, int64_t nodes,
                                  float *__restrict__ vel, float *__restrict__ mass) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= nodes) return;
  const float4 g = V[f];
  vel[f * D] = g.x;
  vel[f * D + 1] = g.y;
  if (D == 3) vel[f * D + D - 1] = g.z;
  mass[f] = g.w;
}

// grid() of an accumulation grid: applies the grid update on the way out.
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

// Grid block (global, scene-major) and cell within it of a position: the sort key of
// block_keys_kernel (stencil base clamped into the grid, as the sort needs a bucket even for a
// particle that is about to raise the out-of-range error).
template <int D>
__device__ __forceinline__ void block_of(const float x[D], const Params &P, int block_off, int &kb,
                                         int &kc) {
  constexpr int BS = Tiling<D>::BS;
  kb = 0;
  kc = 0;
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const int bd = min(max(__float2int_rz(x[d] * P.inv_dx - 0.5f), 0), P.N - 1);
    kb = kb * P.nb + bd / BS;
    kc = kc * BS + bd % BS;
  }
  kb += block_off;
}

// particles() export, one thread per caller row: row q of the scene whose rows start at
// global id id_off lives in slot inv[id_off + q].  Rows are written in order (coalesced on the
// caller's side, which may be mapped host memory); slots are read where the sort put them.
template <int D>
__global__ void export_rows_kernel(PState s, const int *__restrict__ inv, int id_off, int n,
                                   float *__restrict__ x, float *__restrict__ v,
                                   float *__restrict__ F, float *__restrict__ C,
                                   float *__restrict__ Jp) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  const int p = inv[id_off + q];
  const int st = s.stride;
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

// Upload, one thread per slot of the scene (slots [id_off, id_off + n); slot p takes caller
// row id[p] - id_off, so the slot-major writes stay coalesced and a partial update leaves the
// other fields in place).  With `moved`, counts the rows whose new position lies in another
// grid block than the one their slot was sorted into (slot_block, from the last sort): zero
// means the block lists still describe the particles and no re-sort is needed.
template <int D>
__global__ void import_rows_kernel(PState s, int id_off, int n, const float *__restrict__ x,
                                   const float *__restrict__ v, const float *__restrict__ F,
                                   const float *__restrict__ C, const float *__restrict__ Jp,
                                   const Scene *__restrict__ scenes,
                                   const int *__restrict__ slot_block, int *moved) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool off_block = false;
  if (i < n) {
    const int p = id_off + i;
    const int q = s.id[p] - id_off;
    const int st = s.stride;
    float xp[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      if (x) {
        xp[d] = x[(size_t)q * D + d];
        s.x[(size_t)d * st + p] = xp[d];
      }
      if (v) s.v[(size_t)d * st + p] = v[(size_t)q * D + d];
    }
#pragma unroll
    for (int c = 0; c < D * D; ++c) {
      if (F) s.F[(size_t)c * st + p] = F[(size_t)q * D * D + c];
      if (C) s.C[(size_t)c * st + p] = C[(size_t)q * D * D + c];
    }
    if (Jp) s.Jp[p] = Jp[q];
    if (moved && x) {
      const Scene &sc = scenes[s.scene ? (int)s.scene[p] : 0];
      int kb, kc;
      block_of<D>(xp, sc.P, sc.block_off, kb, kc);
      off_block = kb != slot_block[p];
    }
  }
  if (moved) {  // one atomic per warp (every lane reaches this point)
    const unsigned b = __ballot_sync(0xffffffffu, off_block);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(moved, __popc(b));
  }
}

// ---------------------------------------------------------------------------------------
// Sorting slots by grid block and, inside a block, by cell (a one-digit counting sort over
// nb^dim * cells-per-block keys): keys + ranks, exclusive scan of the counts, the list of
// non-empty blocks, then the
// fields the step reads (x, F, Jp, mass, volume, id, material) move to start[key] + rank in
// the other buffer (and the per-particle moduli, when set).  v and C do not move: they are rewritten by the last step of every
// advance() call before anyone reads them.
// ---------------------------------------------------------------------------------------
template <int D>
__global__ void block_keys_kernel(const float *__restrict__ xs, const uint16_t *__restrict__ pscene,
                                  int stride, int n, const Scene *__restrict__ scenes,
                                  int *__restrict__ key, int *__restrict__ rank,
                                  int *__restrict__ count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int sid = pscene ? (int)pscene[p] : 0;
  float x[D];
#pragma unroll
  for (int d = 0; d < D; ++d) x[d] = xs[(size_t)d * stride + p];
  int kb, kc;
  block_of<D>(x, scenes[sid].P, scenes[sid].block_off, kb, kc);
  const int k = kb * Tiling<D>::CPB + kc;  // block-major, then cell
  key[p] = k;
  rank[p] = atomicAdd(count + k, 1);
}

// Destination of a particle inside its block: the block's particles are stored cell by cell
// in rounds -- the first particle of every non-empty cell (cells in x-major order), then the
// second of every cell that has two, and so on -- so consecutive slots lie in different,
// neighbouring cells.  Particle `rank` of cell c goes to
//   bstart[block] + sum_c' min(count[c'], rank) + #{c' < c : count[c'] > rank},
// which the block's round table holds for ranks below kRoundTable (block_tables_kernel);
// later ranks count cell by cell.
template <int D>
__global__ void sort_move_kernel(PState src, PState dst, int n, const int *__restrict__ key,
                                 const int *__restrict__ rank, const int *__restrict__ bstart,
                                 const int4 *__restrict__ rounds, const int *__restrict__ count,
                                 int move_vc, int *__restrict__ inv, int *__restrict__ slot_block) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  constexpr int CPB = Tiling<D>::CPB;
  static_assert(CPB == kCellsPerBlock, "the round tables assume 64 cells per block");
  const int k = key[p], r = rank[p];
  const int blk = k / CPB, c = k % CPB;
  int q = __ldg(bstart + blk);
  if (r < kRoundTable) {
    const int4 t = __ldg(rounds + (int64_t)blk * kRoundTable + r);
    const unsigned long long m = ((unsigned long long)(unsigned)t.z << 32) | (unsigned)t.y;
    q += t.x + __popcll(m & ((1ull << c) - 1ull));
  } else {
    const int b0 = blk * CPB;
    for (int cc = 0; cc < CPB; ++cc) {
      const int m = __ldg(count + b0 + cc);
      q += min(m, r) + ((cc < c && m > r) ? 1 : 0);
    }
  }
  const int ss = src.stride, ds = dst.stride;
#pragma unroll
  for (int d = 0; d < D; ++d) dst.x[(size_t)d * ds + q] = src.x[(size_t)d * ss + p];
#pragma unroll
  for (int cmp = 0; cmp < D * D; ++cmp) dst.F[(size_t)cmp * ds + q] = src.F[(size_t)cmp * ss + p];
  dst.Jp[q] = src.Jp[p];
  dst.mass[q] = src.mass[p];
  dst.vol[q] = src.vol[p];
  const int id = src.id[p];
  dst.id[q] = id;
  inv[id] = q;                     // caller row -> slot
  slot_block[q] = blk;             // the block this slot now belongs to
  if (src.mat) dst.mat[q] = src.mat[p];
  if (src.lame) dst.lame[q] = src.lame[p];
  if (src.scene) dst.scene[q] = src.scene[p];
  if (move_vc) {  // the next P2G reads v and C (right after an upload)
#pragma unroll
    for (int d = 0; d < D; ++d) dst.v[(size_t)d * ds + q] = src.v[(size_t)d * ss + p];
#pragma unroll
    for (int cmp = 0; cmp < D * D; ++cmp) dst.C[(size_t)cmp * ds + q] = src.C[(size_t)cmp * ss + p];
  }
}

// ---------------------------------------------------------------------------------------
// Small scenes: all k steps in one cooperative launch, in the reference's order -- p2g,
// grid_op, g2p (src/nclr.h:80-84) -- one particle per thread straight from global memory
// (the grid of a small scene stays in L2), with a grid-wide barrier after the P2G and after
// the grid update.  A thread keeps the same particles in every phase, so only V and G
// cross threads; they are read through L2 (__ldcg), since other SMs rewrite them during
// the launch.  Replaces 2 launches per step (whose fixed cost dominates a scene of a few
// thousand particles) by one per advance() call.
// ---------------------------------------------------------------------------------------
constexpr int kSmallThreads = 256;

// Barrier of `ctas` CTAs of a cooperative launch (every CTA is resident): bar[0] counts
// arrivals, bar[1] is the generation.  A wait that runs out (`spins` polls of ~64 ns; the
// default kBarrierSpinsDefault is about a second) sets kErrBarrier and every CTA returns false
// (and leaves the kernel); nothing waits without a bound.
__device__ __forceinline__ bool grid_barrier(unsigned *bar, int *err, unsigned ctas,
                                             unsigned spin_limit) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned *gen = bar + 1;
    const unsigned g = *gen;
    __threadfence();  // this CTA's writes before its arrival
    int ok = 1;
    if (atomicAdd(bar, 1u) + 1u == ctas) {
      atomicExch(bar, 0u);  // reset for the next barrier, before the release
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned spins = 0;
      while (*gen == g) {
        if (++spins > spin_limit) {
          atomicOr(err, kErrBarrier);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok && !(*(volatile int *)err & kErrBarrier);
  }
  __syncthreads();
  return s_ok != 0;
}

// The hardware barrier of a thread-block cluster, with release/acquire at cluster scope: every
// CTA's global writes before it (the P2G reductions, V) are visible to every CTA after it.
__device__ __forceinline__ void cluster_barrier() {
  asm volatile(
      "barrier.cluster.arrive.release.aligned;\n\t"
      "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Threads per CTA of the small-scene kernel launched as one cluster (registers allow these
// without spills: up to 80 a thread in 2D, 127 in 3D).
template <int D>
constexpr int small_cluster_threads() {
  return D == 3 ? 512 : 640;
}
static_assert(small_cluster_threads<2>() == kSmallClusterThreads2D &&
                  small_cluster_threads<3>() == kSmallClusterThreads3D,
              "the host sizes cluster launches by these");

// kCluster: the launch is a single thread-block cluster (every CTA resident on one GPC) and
// the step's two barriers are the cluster's hardware barrier; otherwise a cooperative launch
// with the bounded grid barrier above.
template <int D, bool kRef, bool kCluster = false>
__global__ void __launch_bounds__(kCluster ? small_cluster_threads<D>() : kSmallThreads)
small_steps_kernel(PState s, Params P, float4 *__restrict__ G, float4 *__restrict__ V, int steps,
                   int *err, unsigned *bar, BarrierTest bt) {
  constexpr int S = (D == 3) ? 27 : 9;
  const int stride = gridDim.x * blockDim.x;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int st = s.stride, N = P.N;
  // P2G of one particle into G from its state (x, v, F, C, Jp) and the rotation R of its F
  auto p2g_one = [&](int p, const float x[D], const float v[D], const Mat<D> &F, const Mat<D> &C,
                     float Jp, const Mat<D> &R, int material) {
    float mv[D], fx[D], w[3][D];
    int base[D];
    const float m = s.mass[p];
    Mat<D> A = fused_affine<D>(F, R, C, Jp, m, s.vol[p], material, lame0(s, p, P), P);
#pragma unroll
    for (int d = 0; d < D; ++d) mv[d] = v[d] * m;
    stencil<D>(x, P.inv_dx, base, fx, w);
    p2g_terms<D>(fx, P.dx, mv, A);
    const int64_t f0 = flat_index<D>(base, N);
#pragma unroll
    for (int o = 0; o < S; ++o) {
      const int64_t f = stencil_flat<D>(f0, o, N);
      if (f < 0 || f >= P.nodes) {
        atomicOr(err, kErrOutOfRange);
        continue;
      }
      float c[4];
      p2g_contrib<D>(o, w, mv, m, A, c);
      red_add_v4(G + f, c[0], c[1], c[2], c[3]);
    }
  };
  // G2P of one particle (src/nclr.h:167-261): gathers v and C from V, advects x, updates F
  // and Jp; returns the rotation of the new F when need_R (see update_F)
  auto g2p_one = [&](float x[D], float v[D], Mat<D> &F, Mat<D> &C, float &Jp, int material,
                     bool need_R) {
    float fx[D], w[3][D];
    int base[D];
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = 0.0f;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) C.a[i][j] = 0.0f;
    stencil<D>(x, P.inv_dx, base, fx, w);
    const int64_t f0 = flat_index<D>(base, N);
    g2p_gather<D>(
        [&](int o) {
          const int64_t f = stencil_flat<D>(f0, o, N);
          if (f >= 0 && f < P.nodes) return __ldcg(V + f);
          atomicOr(err, kErrOutOfRange);
          return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        },
        fx, w, v, C);
    scale_mat<D>(C, P.cscale);
#pragma unroll
    for (int d = 0; d < D; ++d) x[d] += P.dt * v[d];
    return update_F<D, kRef>(C, F, Jp, material, P.dt, need_R);
  };
  if (steps <= 0) return;
  // With at most one particle per thread (thread tid owns particle tid), the particle's state
  // stays in registers for the whole call: read once here, written once after the last step
  // (README scene 6.89 -> 6.64 us per step, a 22k-particle 3D block 18.5 -> 18.0 us).
  const bool resident = P.n <= stride;
  const bool mine = resident && tid < P.n;
  float rx[D], rv[D], rJp = 0.0f;
  Mat<D> rF, rC;
  int rmat = P.model;
  if (mine) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      rx[d] = s.x[(size_t)d * st + tid];
      rv[d] = s.v[(size_t)d * st + tid];
    }
    rF = load_mat<D>(s.F, st, tid);
    rC = load_mat<D>(s.C, st, tid);
    rJp = s.Jp[tid];
    rmat = s.mat ? (int)s.mat[tid] : P.model;
  }
  // ---- p2g of the first step (src/nclr.h:104-165) from the stored state ----
  if (resident) {
    if (mine) p2g_one(tid, rx, rv, rF, rC, rJp, stress_R<D>(rF, P, rmat), rmat);
  } else {
    for (int p = tid; p < P.n; p += stride) {
      float x[D], v[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        x[d] = s.x[(size_t)d * st + p];
        v[d] = s.v[(size_t)d * st + p];
      }
      const Mat<D> F = load_mat<D>(s.F, st, p), C = load_mat<D>(s.C, st, p);
      const int material = s.mat ? (int)s.mat[p] : P.model;
      p2g_one(p, x, v, F, C, s.Jp[p], stress_R<D>(F, P, material), material);
    }
  }
  for (int step = 0; step < steps; ++step) {
    if constexpr (kCluster) cluster_barrier();
    else if (!grid_barrier(bar, err, gridDim.x + bt.extra, bt.spins)) return;
    // ---- grid_op (src/nclr.h:263-310): V = op(G), and G cleared for the next p2g ----
    for (int64_t i = tid; i < P.nodes; i += stride) {
      int idx[D];
      unflatten<D>(i, N, idx);
      float v[D], m;
      grid_update<D>(__ldcg(G + i), idx, P, v, m);
      V[i] = make_float4(v[0], v[1], D == 3 ? v[D - 1] : 0.0f, m);
      G[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    if constexpr (kCluster) cluster_barrier();
    else if (!grid_barrier(bar, err, gridDim.x + bt.extra, bt.spins)) return;
    // ---- g2p, then the next step's p2g of the same particle from its new state in
    // registers (each thread keeps its particles from step to step, so no barrier is needed
    // between the two; G was cleared above), with the stress rotation from the F update's own
    // decomposition.  Measured against a separate p2g pass at the top of each step: the
    // README scene 7.25 -> 6.86 us per step, a 22k-particle 3D jelly block 18.7 -> 18.4 us ----
    const bool next = step + 1 < steps;
    const bool need_R = next && P.stress == kCorotated;
    if (resident) {
      if (mine) {
        const Mat<D> R = g2p_one(rx, rv, rF, rC, rJp, rmat, need_R);
        if (next) p2g_one(tid, rx, rv, rF, rC, rJp, R, rmat);
      }
      continue;
    }
    for (int p = tid; p < P.n; p += stride) {
      float x[D], v[D];
#pragma unroll
      for (int d = 0; d < D; ++d) x[d] = s.x[(size_t)d * st + p];
      Mat<D> F = load_mat<D>(s.F, st, p), C;
      float Jp = s.Jp[p];
      const int material = s.mat ? (int)s.mat[p] : P.model;
      const Mat<D> R = g2p_one(x, v, F, C, Jp, material, need_R);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        s.x[(size_t)d * st + p] = x[d];
        s.v[(size_t)d * st + p] = v[d];
      }
      store_mat<D>(s.F, st, p, F);
      store_mat<D>(s.C, st, p, C);
      s.Jp[p] = Jp;
      if (next) p2g_one(p, x, v, F, C, Jp, R, material);
    }
  }
  if (mine) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      s.x[(size_t)d * st + tid] = rx[d];
      s.v[(size_t)d * st + tid] = rv[d];
    }
    store_mat<D>(s.F, st, tid, rF);
    store_mat<D>(s.C, st, tid, rC);
    s.Jp[tid] = rJp;
  }
}

template <int D, bool kRef>
__global__ void __launch_bounds__(kSmallThreads) small_batch_kernel(
    PState s, const Scene *__restrict__ scenes, const uint16_t *__restrict__ cta_scene,
    const int *__restrict__ group_first, float4 *__restrict__ Gall, float4 *__restrict__ Vall,
    uint8_t *__restrict__ flags_all, int steps, int *err_all, unsigned *bars, BarrierTest bt) {
  constexpr int S = (D == 3) ? 27 : 9;
  constexpr int BS = Tiling<D>::BS;
  constexpr int BN = (D == 3) ? BS * BS * BS : BS * BS;
  __shared__ Params sP;
  __shared__ int64_t s_node_off;
  __shared__ int s_block_off, s_slot_off, s_first, s_ctas;
  const int sid = (int)cta_scene[blockIdx.x];
  if (threadIdx.x == 0) {
    sP = scenes[sid].P;
    s_node_off = scenes[sid].node_off;
    s_block_off = scenes[sid].block_off;
    s_slot_off = scenes[sid].slot_off;
    s_first = group_first[sid];
    s_ctas = group_first[sid + 1] - group_first[sid];
  }
  __syncthreads();
  const Params &P = sP;
  float4 *__restrict__ G = Gall + s_node_off;
  float4 *__restrict__ V = Vall + s_node_off;
  uint8_t *__restrict__ flags = flags_all + s_block_off;
  int *err = err_all + 2 * sid;
  unsigned *bar = bars + 2 * sid;
  const unsigned ctas = (unsigned)s_ctas;
  const int stride = s_ctas * blockDim.x;
  const int tid = (blockIdx.x - s_first) * blockDim.x + threadIdx.x;
  const int warps = s_ctas * (blockDim.x >> 5), warp = tid >> 5, lane = threadIdx.x & 31;
  const int st = s.stride, N = P.N, p0 = s_slot_off;
  for (int step = 0; step < steps; ++step) {
    // ---- p2g (src/nclr.h:104-165), marking the touched blocks ----
    for (int q = tid; q < P.n; q += stride) {
      const int p = p0 + q;
      float x[D], mv[D], fx[D], w[3][D];
      int base[D];
#pragma unroll
      for (int d = 0; d < D; ++d) x[d] = s.x[(size_t)d * st + p];
      const Mat<D> F = load_mat<D>(s.F, st, p), C = load_mat<D>(s.C, st, p);
      const float m = s.mass[p];
      const int material = s.mat ? (int)s.mat[p] : P.model;
      Mat<D> A = fused_affine<D>(F, stress_R<D>(F, P, material), C, s.Jp[p], m, s.vol[p],
                                 material, lame0(s, p, P), P);
#pragma unroll
      for (int d = 0; d < D; ++d) mv[d] = s.v[(size_t)d * st + p] * m;
      stencil<D>(x, P.inv_dx, base, fx, w);
      p2g_terms<D>(fx, P.dx, mv, A);
      const int64_t f0 = flat_index<D>(base, N);
#pragma unroll
      for (int o = 0; o < S; ++o) {
        const int64_t f = stencil_flat<D>(f0, o, N);
        if (f < 0 || f >= P.nodes) {
          atomicOr(err, kErrOutOfRange);
          continue;
        }
        float c[4];
        p2g_contrib<D>(o, w, mv, m, A, c);
        red_add_v4(G + f, c[0], c[1], c[2], c[3]);
      }
      mark_stencil<D>(flags, base, P);
    }
    if (!grid_barrier(bar, err, ctas + bt.extra, bt.spins)) return;
    // ---- grid_op (src/nclr.h:263-310) on the flagged blocks: V = op(G), G = 0 ----
    for (int b = warp; b < P.nblocks; b += warps) {
      const uint8_t fl = __ldcg(flags + b);
      if (!fl) continue;
      int bc[D];
      {
        int r = b;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          bc[d] = (r % P.nb) * BS;
          r /= P.nb;
        }
      }
      for (int t = lane; t < BN; t += 32) {
        int idx[D];
        bool in = true;
        int r = t;
#pragma unroll
        for (int d = D - 1; d >= 0; --d) {
          idx[d] = bc[d] + r % BS;
          r /= BS;
          in &= idx[d] < N;
        }
        if (!in) continue;
        const int64_t f = flat_index<D>(idx, N);
        float v[D], m;
        grid_update<D>(__ldcg(G + f), idx, P, v, m);
        V[f] = make_float4(v[0], v[1], D == 3 ? v[D - 1] : 0.0f, m);
        G[f] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
      if (lane == 0) flags[b] = (fl & kPending) ? kVNonzero : 0;
    }
    if (!grid_barrier(bar, err, ctas + bt.extra, bt.spins)) return;
    // ---- g2p (src/nclr.h:167-261) ----
    for (int q = tid; q < P.n; q += stride) {
      const int p = p0 + q;
      float x[D], v[D], fx[D], w[3][D];
      int base[D];
#pragma unroll
      for (int d = 0; d < D; ++d) {
        x[d] = s.x[(size_t)d * st + p];
        v[d] = 0.0f;
      }
      Mat<D> C;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) C.a[i][j] = 0.0f;
      stencil<D>(x, P.inv_dx, base, fx, w);
      const int64_t f0 = flat_index<D>(base, N);
      g2p_gather<D>(
          [&](int o) {
            const int64_t f = stencil_flat<D>(f0, o, N);
            if (f >= 0 && f < P.nodes) return __ldcg(V + f);
            atomicOr(err, kErrOutOfRange);
            return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
          },
          fx, w, v, C);
      scale_mat<D>(C, P.cscale);
#pragma unroll
      for (int d = 0; d < D; ++d) x[d] += P.dt * v[d];
      Mat<D> F = load_mat<D>(s.F, st, p);
      float Jp = s.Jp[p];
      update_F<D, kRef>(C, F, Jp, s.mat ? (int)s.mat[p] : P.model, P.dt, false);
#pragma unroll
      for (int d = 0; d < D; ++d) {
        s.x[(size_t)d * st + p] = x[d];
        s.v[(size_t)d * st + p] = v[d];
      }
      store_mat<D>(s.F, st, p, F);
      store_mat<D>(s.C, st, p, C);
      s.Jp[p] = Jp;
    }
  }
}

// ---------------------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------------------
inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

template <int D>
void launch_grid_sweep(float4 *G, float4 *V, uint8_t *flags, const Scene *scenes,
                       const uint16_t *block_scene, const Params &P0, int total_blocks,
                       int *work, int sms, cudaStream_t st, int *fix_count) {
  // one wave: as many CTAs as are resident at once (a second, partial wave left the SMs idle
  // for 45% of the kernel)
  static int resident[2] = {0, 0};
  const bool batch = block_scene != nullptr;
  int &res = resident[batch];
  if (!res) {
    if (batch)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&res, grid_sweep_kernel<D, true>, 256, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&res, grid_sweep_kernel<D, false>, 256, 0);
    if (res < 1) res = 1;
  }
  int64_t blocks = blocks_for((int64_t)total_blocks * 32, 256);
  if (blocks > (int64_t)sms * res) blocks = (int64_t)sms * res;
  if (blocks < 1) blocks = 1;
  if (batch)
    launch_overlapped(grid_sweep_kernel<D, true>, (unsigned)blocks, 256, 0, st, G, V, flags,
                      scenes, block_scene, P0, total_blocks, work, fix_count);
  else
    launch_overlapped(grid_sweep_kernel<D, false>, (unsigned)blocks, 256, 0, st, G, V, flags,
                      scenes, block_scene, P0, total_blocks, work, fix_count);
}

// ---------------------------------------------------------------------------------------
// snow_fix: the snow clamps the last fused launch left for FP64 (SnowFix), one per thread.
// Each recomputes its FP32 result as the fused kernel did (the same functions on the same
// F_hat and Jp), and the clamp in FP64; writes the FP64 F and Jp to the particle (and to the
// recorded caller-order rows of a rollout segment); and, when that launch did the next step's
// P2G, adds to G the difference the FP64 stress makes there: weight_o (A_64 - A_32) (o - fx)
// dx for the stencil of the particle's updated position, with A the stress part of the fused
// APIC momentum (src/nclr.h:313-337; the m C part is the same in both).
// ---------------------------------------------------------------------------------------
template <int D, bool kRef>
__global__ void __launch_bounds__(128) snow_fix_kernel(PState s, Params P0,
                                                       const Scene *__restrict__ scenes,
                                                       SnowFix fix, float4 *__restrict__ Gall,
                                                       int scatter, Record rec) {
  const int count = min(*fix.count, fix.cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const int p = fix.slot[i];
    const int sid = s.scene ? (int)s.scene[p] : 0;
    const Params P = scenes ? scenes[sid].P : P0;
    Mat<D> Fh;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = 0; b < D; ++b) Fh.a[a][b] = fix.Fh[((size_t)i * D + a) * D + b];
    const float Jp_in = fix.Jp[i];
    const bool need_R = P.stress == kCorotated;
    // the FP32 result the fused launch carried on with
    Mat<D> U, Vm, F32 = Fh, R32 = Fh;
    float sig[D], Jp32 = Jp_in;
    if constexpr (D == 3) {
      svd3(Fh, U, sig, Vm);
    } else {
      svd2<kRef>(Fh, U, sig, Vm);
    }
    snow_clamp_fp32<D>(U, sig, Vm, F32, Jp32, R32, need_R);
    // the FP64 one
    Mat<D> F64, R64;
    float Jp64 = Jp_in;
    snow_clamp_fp64<D, kRef>(&Fh, &Vm, &Jp64, &F64, &R64);
    const int st = s.stride;
    store_mat<D>(s.F, st, p, F64);
    s.Jp[p] = Jp64;
    if (rec.F) {  // a rollout segment's recorded rows (caller order)
      const size_t q = (size_t)s.id[p];
#pragma unroll
      for (int a = 0; a < D; ++a)
#pragma unroll
        for (int b = 0; b < D; ++b) rec.F[(q * D + a) * D + b] = F64.a[a][b];
      if (rec.Jp) rec.Jp[q] = Jp64;
    }
    if (!scatter) continue;
    Mat<D> Z;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = 0; b < D; ++b) Z.a[a][b] = 0.0f;
    const float m = s.mass[p], vol = s.vol[p];
    const float2 l0 = lame0(s, p, P);
    const Mat<D> A64 = fused_affine<D>(F64, need_R ? R64 : F64, Z, Jp64, m, vol, kSnow, l0, P);
    const Mat<D> A32 = fused_affine<D>(F32, need_R ? R32 : F32, Z, Jp32, m, vol, kSnow, l0, P);
    Mat<D> dA;
#pragma unroll
    for (int a = 0; a < D; ++a)
#pragma unroll
      for (int b = 0; b < D; ++b) dA.a[a][b] = A64.a[a][b] - A32.a[a][b];
    float x[D], fx[D], w[3][D], q0[D];
    int base[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      x[d] = s.x[(size_t)d * st + p];
      q0[d] = 0.0f;
    }
    stencil<D>(x, P.inv_dx, base, fx, w);
    p2g_terms<D>(fx, P.dx, q0, dA);  // q0 = -dA fx dx, dA becomes dA dx
    float4 *G = Gall + (scenes ? scenes[sid].node_off : 0);
    const int64_t f0 = flat_index<D>(base, P.N);
    constexpr int S = (D == 3) ? 27 : 9;
#pragma unroll
    for (int o = 0; o < S; ++o) {
      const int64_t f = stencil_flat<D>(f0, o, P.N);
      if (f < 0 || f >= P.nodes) continue;  // the fused launch reported it already
      float c[4];
      p2g_contrib<D>(o, w, q0, 0.0f, dA, c);
      red_add_v4(G + f, c[0], c[1], c[2], 0.0f);
    }
  }
}

template <int D>
void launch_snow_fix(const PState &s, const Params &P0, const Scene *scenes, const SnowFix &fix,
                     float4 *G, bool scatter, bool ref, const Record &rec, int sms,
                     cudaStream_t st) {
  if (!fix.count) return;
  // two CTAs per SM: the list is usually empty or a small fraction of the particles, and the
  // FP64 work of a full one is bound by the SMs' FP64 rate, not by latency
  const unsigned blocks = (unsigned)std::max(1, 2 * sms);
  if (ref)
    snow_fix_kernel<D, true><<<blocks, 128, 0, st>>>(s, P0, scenes, fix, G, scatter ? 1 : 0, rec);
  else
    snow_fix_kernel<D, false><<<blocks, 128, 0, st>>>(s, P0, scenes, fix, G, scatter ? 1 : 0, rec);
}

template <int D>
void launch_discard_pending(float4 *G, uint8_t *flags, const Scene *scenes,
                            const uint16_t *block_scene, int total_blocks, int sms,
                            cudaStream_t st) {
  int64_t blocks = blocks_for((int64_t)total_blocks * 32, 256);
  if (blocks > (int64_t)sms * 8) blocks = (int64_t)sms * 8;
  if (blocks < 1) blocks = 1;
  discard_pending_kernel<D><<<(unsigned)blocks, 256, 0, st>>>(G, flags, scenes, block_scene,
                                                               total_blocks);
}

// The fused step (kStep or kFinalStep) of a single simulation whose particles all have
// `material`, fixed at compile time.  Defined and instantiated for 3D in step3d_mat.cu, a
// translation unit of its own that compiles beside step3d.cu.
template <int D>
void launch_g2p2g_fixed(const PState &s, const Params &P0, const float4 *V, float4 *G,
                        uint8_t *flags, const int *blocks, const int *nactive,
                        const int *bstart, const int *sparse, int *work, int *err, int next_slot,
                        bool ref, int mode, int material, int ctas, cudaStream_t st,
                        const Record &rec, const SnowFix &fix);
// Raises the dynamic shared-memory limit of every launch_g2p2g_fixed<D> kernel to `bytes`.
template <int D>
void g2p2g_fixed_set_smem(int bytes);

template <int D>
void launch_g2p2g(const PState &s, const Params &P0, const Scene *scenes,
                  const uint16_t *block_scene, const float4 *V, float4 *G, uint8_t *flags,
                  const int *blocks, const int *nactive, const int *bstart, const int *sparse,
                  int *work, int *err, int next_slot, bool ref, int mode, int ctas,
                  cudaStream_t st, const Record &rec, const SnowFix &fix, int item_threads) {
  if constexpr (D == 3) {  // one material for every particle: the specialised kernel
    if (!block_scene && !s.mat && (mode == kStep || mode == kFinalStep) &&
        (P0.model == kSnow || P0.model == kJelly || P0.model == kLiquid)) {
      launch_g2p2g_fixed<D>(s, P0, V, G, flags, blocks, nactive, bstart, sparse, work, err,
                            next_slot, ref, mode, P0.model, ctas, st, rec, fix);
      return;
    }
  }
#define MPM_G2P2G(R, MODE, B)                                                                \
  launch_overlapped(g2p2g_kernel<D, R, MODE, B>, (unsigned)ctas, kG2P2GThreads,               \
                    (MODE) == kG2PFinal ? g2p_final_smem_bytes<D>() : g2p2g_smem_bytes<D, B>(), \
                    st, s, P0, scenes, block_scene, V, G, flags, blocks, nactive, bstart,      \
                    sparse, work, err, next_slot, rec, fix)
// 2D batches with whole-CTA items (item_threads 256) instead of the default half-CTA ones
#define MPM_G2P2G_ITEM(R, MODE)                                                               \
  launch_overlapped(g2p2g_kernel<D, R, MODE, true, -1, kG2P2GThreads>, (unsigned)ctas,        \
                    kG2P2GThreads, g2p2g_smem_bytes<D, true, kG2P2GThreads>(), st, s, P0,      \
                    scenes, block_scene, V, G, flags, blocks, nactive, bstart, sparse, work,   \
                    err, next_slot, rec, fix)
#define MPM_G2P2G_B(R, MODE)                                      \
  if (block_scene && D == 2 && item_threads == kG2P2GThreads) {   \
    MPM_G2P2G_ITEM(R, MODE);                                      \
  } else if (block_scene) {                                       \
    MPM_G2P2G(R, MODE, true);                                     \
  } else {                                                        \
    MPM_G2P2G(R, MODE, false);                                    \
  }
  if (mode == kG2PFinal && !block_scene) {  // single simulations only
    if (ref) {
      MPM_G2P2G(true, kG2PFinal, false);
    } else {
      MPM_G2P2G(false, kG2PFinal, false);
    }
  } else if (ref) {
    if (mode == kFinalStep || mode == kG2PFinal) { MPM_G2P2G_B(true, kFinalStep) }
    else if (mode == kP2GOnly) { MPM_G2P2G_B(true, kP2GOnly) }
    else { MPM_G2P2G_B(true, kStep) }
  } else {
    if (mode == kFinalStep || mode == kG2PFinal) { MPM_G2P2G_B(false, kFinalStep) }
    else if (mode == kP2GOnly) { MPM_G2P2G_B(false, kP2GOnly) }
    else { MPM_G2P2G_B(false, kStep) }
  }
#undef MPM_G2P2G_B
#undef MPM_G2P2G_ITEM
#undef MPM_G2P2G
}

// The small-scene launch: `ctas` CTAs, all resident (cooperative launch), `steps` steps.
// bar (2 unsigned) must be zero.  Returns the launch error (e.g. too many CTAs).
template <int D>
cudaError_t launch_small_steps(const PState &s, const Params &P, float4 *G, float4 *V, int steps,
                               int *err, unsigned *bar, bool ref, int ctas, cudaStream_t st,
                               BarrierTest bt) {
  PState sv = s;
  Params Pv = P;
  void *args[] = {&sv, &Pv, &G, &V, &steps, &err, &bar, &bt};
  const void *fn = ref ? (const void *)small_steps_kernel<D, true> : (const void *)small_steps_kernel<D, false>;
  return cudaLaunchCooperativeKernel(fn, dim3((unsigned)ctas), dim3(kSmallThreads), args, 0, st);
}

// The small-scene kernel as one thread-block cluster of `ctas` CTAs of `threads` threads
// (threads <= small_cluster_threads<D>(); ctas <= small_cluster_max<D>(threads)).
template <int D>
cudaError_t launch_small_cluster(const PState &s, const Params &P, float4 *G, float4 *V,
                                 int steps, int *err, unsigned *bar, bool ref, int ctas,
                                 int threads, cudaStream_t st) {
  PState sv = s;
  Params Pv = P;
  BarrierTest bt{};
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)ctas);
  cfg.blockDim = dim3((unsigned)threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)ctas;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return ref ? cudaLaunchKernelEx(&cfg, small_steps_kernel<D, true, true>, sv, Pv, G, V, steps,
                                  err, bar, bt)
             : cudaLaunchKernelEx(&cfg, small_steps_kernel<D, false, true>, sv, Pv, G, V, steps,
                                  err, bar, bt);
}

// The largest cluster (CTAs) the small-scene kernel can be launched as with `threads` threads
// per CTA: 16 where the device allows non-portable clusters, else 8 (0: no cluster launch).
template <int D>
int small_cluster_max(bool ref, int threads) {
  const void *fn = ref ? (const void *)small_steps_kernel<D, true, true>
                       : (const void *)small_steps_kernel<D, false, true>;
  cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(16);
  cfg.blockDim = dim3((unsigned)threads);
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = 16;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  int size = 0;
  if (cudaOccupancyMaxPotentialClusterSize(&size, fn, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return size >= 16 ? 16 : (size >= 8 ? 8 : size);
}

template <int D>
cudaError_t launch_small_batch(const PState &s, const Scene *scenes, const uint16_t *cta_scene,
                               const int *group_first, float4 *G, float4 *V, uint8_t *flags,
                               int steps, int *err, unsigned *bars, bool ref, int ctas,
                               cudaStream_t st, BarrierTest bt) {
  PState sv = s;
  void *args[] = {&sv, &scenes, &cta_scene, &group_first, &G, &V, &flags, &steps, &err, &bars,
                  &bt};
  const void *fn = ref ? (const void *)small_batch_kernel<D, true> : (const void *)small_batch_kernel<D, false>;
  return cudaLaunchCooperativeKernel(fn, dim3((unsigned)ctas), dim3(kSmallThreads), args, 0, st);
}

template <int D>
int small_batch_ctas_per_sm(bool ref) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &n, ref ? small_batch_kernel<D, true> : small_batch_kernel<D, false>, kSmallThreads, 0);
  return n;
}

template <int D>
int small_ctas_per_sm(bool ref) {
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      &n, ref ? small_steps_kernel<D, true> : small_steps_kernel<D, false>, kSmallThreads, 0);
  return n;
}

template <int D>
int g2p2g_ctas_per_sm() {
  // the tiles exceed the default 48 KB of dynamic shared memory in 3D
  const int bytes = (int)std::max(g2p2g_smem_bytes<D, false>(), g2p2g_smem_bytes<D, true>());
  {
    const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kStep, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kFinalStep, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kP2GOnly, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kStep, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kFinalStep, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kP2GOnly, false>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kStep, true>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kFinalStep, true>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, true, kP2GOnly, true>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kStep, true>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kFinalStep, true>, a, bytes);
    cudaFuncSetAttribute(g2p2g_kernel<D, false, kP2GOnly, true>, a, bytes);
    if constexpr (D == 3) g2p2g_fixed_set_smem<D>(bytes);
  }
  int n = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, g2p2g_kernel<D, true, kStep, true>, kG2P2GThreads,
                                                g2p2g_smem_bytes<D, true>());
  return n > 0 ? n : 1;
}

// Resident CTAs per SM of the G2P-only final step (registers and its one tile).
template <int D>
int g2p_final_ctas_per_sm() {
  int a = 0, b = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, g2p2g_kernel<D, true, kG2PFinal, false>,
                                                kG2P2GThreads, g2p_final_smem_bytes<D>());
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, g2p2g_kernel<D, false, kG2PFinal, false>,
                                                kG2P2GThreads, g2p_final_smem_bytes<D>());
  const int n = a < b ? a : b;
  return n > 0 ? n : 1;
}

template <int D>
void launch_copy_vgrid(const float4 *V, int64_t nodes, float *vel, float *mass, cudaStream_t st) {
  copy_vgrid_kernel<D><<<blocks_for(nodes, 256), 256, 0, st>>>(V, nodes, vel, mass);
}

template <int D>
void launch_export_grid(const float4 *grid, const Params &P, float *vel, float *mass, cudaStream_t st) {
  export_grid_kernel<D><<<blocks_for(P.nodes, 256), 256, 0, st>>>(grid, P, vel, mass);
}

template <int D>
void launch_export_rows(const PState &s, const int *inv, int id_off, int n, float *x, float *v,
                        float *F, float *C, float *Jp, cudaStream_t st) {
  if (n == 0) return;
  export_rows_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(s, inv, id_off, n, x, v, F, C, Jp);
}

template <int D>
void launch_import_rows(const PState &s, int id_off, int n, const float *x,
                        const float *v, const float *F, const float *C, const float *Jp,
                        const Scene *scenes, const int *slot_block, int *moved, cudaStream_t st) {
  if (n == 0) return;
  import_rows_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(s, id_off, n, x, v, F, C, Jp, scenes,
                                                            slot_block, moved);
}

template <int D>
void launch_block_keys(const PState &s, int n, const Scene *scenes, int *key, int *rank, int *count,
                       cudaStream_t st) {
  if (n == 0) return;
  block_keys_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(s.x, s.scene, s.stride, n, scenes, key,
                                                           rank, count);
}

template <int D>
void launch_sort_move(const PState &src, const PState &dst, int n, const int *key, const int *rank,
                      const int *bstart, const int4 *rounds, const int *count, bool move_vc,
                      int *inv, int *slot_block, cudaStream_t st) {
  if (n == 0) return;
  sort_move_kernel<D><<<blocks_for(n, 256), 256, 0, st>>>(src, dst, n, key, rank, bstart, rounds,
                                                          count, move_vc ? 1 : 0, inv, slot_block);
}

#define MPM_INSTANTIATE(D)                                                                       \
  template void launch_grid_sweep<D>(float4 *, float4 *, uint8_t *, const Scene *,              \
                                     const uint16_t *, const Params &, int, int *, int,          \
                                     cudaStream_t, int *);                                       \
  template void launch_snow_fix<D>(const PState &, const Params &, const Scene *,                \
                                   const SnowFix &, float4 *, bool, bool, const Record &, int,   \
                                   cudaStream_t);                                                \
  template void launch_discard_pending<D>(float4 *, uint8_t *, const Scene *, const uint16_t *,  \
                                          int, int, cudaStream_t);                               \
  template void launch_g2p2g<D>(const PState &, const Params &, const Scene *, const uint16_t *, \
                                const float4 *, float4 *, uint8_t *, const int *, const int *,   \
                                const int *, const int *, int *, int *, int, bool, int, int,     \
                                cudaStream_t, const Record &, const SnowFix &, int);             \
  template int g2p2g_ctas_per_sm<D>();                                                           \
  template int g2p_final_ctas_per_sm<D>();                                                       \
  template cudaError_t launch_small_cluster<D>(const PState &, const Params &, float4 *,          \
                                               float4 *, int, int *, unsigned *, bool, int, int, \
                                               cudaStream_t);                                    \
  template int small_cluster_max<D>(bool, int);                                                  \
  template cudaError_t launch_small_steps<D>(const PState &, const Params &, float4 *, float4 *,   \
                                             int, int *, unsigned *, bool, int, cudaStream_t,   \
                                             BarrierTest);                                       \
  template int small_ctas_per_sm<D>(bool);                                                       \
  template cudaError_t launch_small_batch<D>(const PState &, const Scene *, const uint16_t *,      \
                                             const int *, float4 *, float4 *, uint8_t *, int,     \
                                             int *, unsigned *, bool, int, cudaStream_t,          \
                                             BarrierTest);                                        \
  template int small_batch_ctas_per_sm<D>(bool);                                                 \
  template void launch_copy_vgrid<D>(const float4 *, int64_t, float *, float *, cudaStream_t);   \
  template void launch_export_grid<D>(const float4 *, const Params &, float *, float *,          \
                                      cudaStream_t);                                             \
  template void launch_export_rows<D>(const PState &, const int *, int, int, float *, float *,    \
                                      float *, float *, float *, cudaStream_t);                  \
  template void launch_import_rows<D>(const PState &, int, int, const float *,                   \
                                      const float *, const float *, const float *,               \
                                      const float *, const Scene *, const int *, int *,          \
                                      cudaStream_t);                                             \
  template void launch_block_keys<D>(const PState &, int, const Scene *, int *, int *, int *,    \
                                     cudaStream_t);                                              \
  template void launch_sort_move<D>(const PState &, const PState &, int, const int *, const int *, \
                                    const int *, const int4 *, const int *, bool, int *, int *,    \
                                    cudaStream_t);

}  // namespace mpm
