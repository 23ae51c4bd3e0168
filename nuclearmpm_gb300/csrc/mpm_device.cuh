// Device side of the MLS-MPM step (the reference's MPMSimulation<dim>::advance(),
// src/nclr.h:80-310), written for sm_103a.
//
// HBM layout
//   particles  SoA, component-major: field component c of particle slot p at
//              field[c * stride + p] (x: dim comps; F, C: dim*dim comps, row-major; v: dim;
//              Jp, mass, volume: 1).  `id[p]` is the caller's index of slot p: slots are
//              re-sorted by grid block every few steps and the caller's order is restored on
//              download.  `mat[p]` (optional) is a per-particle material and `lame[p]`
//              (optional) per-particle base Lame parameters (mu_0, lambda_0).  v and C are written
//              only by the last step of an advance() call (nothing else reads them: each
//              G2P rebuilds them from the grid).
//   G          dense (res+1)^dim float4 nodes {sum w (m v + A dpos), sum w m} (the reference's
//              x-major node order): the P2G accumulator of the coming step.
//   V          dense (res+1)^dim float4 nodes {v (post grid update), m}: the grid() of the
//              last step, read by G2P.  The grid sweep turns G into V and zeroes G.
//   blocks     the grid is tiled into blocks of BS^dim cells (BS = 4 in 3D, 8 in 2D); slots
//              are sorted by the block of their base node, and the G2P+P2G kernel stages a
//              (BS+4)^dim node tile of V and of the next G around each block in shared memory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_math.cuh"

namespace mpm {

enum : int { kSnow = 0, kJelly = 1, kLiquid = 2 };
enum : int { kErrOutOfRange = 1, kErrBarrier = 2 };  // error flag bits
// Stress models: the reference's fixed-corotated stress (src/nclr.h:313-337) and the
// neo-Hookean one it lists as a TODO (src/nclr.h:339).
enum : int { kCorotated = 0, kNeoHookean = 1 };

// Block tiling of the grid (see the layout note above).  Particles are sorted by block and,
// inside a block, stored cell by cell in rounds (the first particle of every cell in x-major
// cell order, then the second, ...), so the consecutive slots a warp takes sit in different,
// neighbouring cells.
// Both shared-memory tiles hold float4 nodes with a y stride of 12 (= 4 mod 8): the 8 lanes
// of one 128-byte wavefront, which cover 2 (y) x 4 (z) neighbouring cells, then fall in
// 8 different 16-byte bank groups.
template <int D>
struct Tiling {
  static constexpr int BS = (D == 3) ? 4 : 8;  // cells per block side
  static constexpr int CPB = (D == 3) ? BS * BS * BS : BS * BS;  // cells per block
  static constexpr int T = BS + 4;             // tile side in nodes: block - 1 .. block + BS + 2
  static constexpr int NODES = (D == 3) ? T * T * T : T * T;
  // shared-memory strides of a tile (3D: x, y; z stride 1.  2D: x; y stride 1)
  static constexpr int SX = (D == 3) ? (T - 1) * 12 + T : T, SY = 12;
  static constexpr int SIZE = (D == 3) ? (T - 1) * SX + (T - 1) * SY + T : T * T;
};

struct Params {
  int res, N;           // N = res + 1 nodes per axis
  int n;                // particles
  int model;            // material of every particle (when mat == nullptr)
  float dt, dx, inv_dx, gravity;
  float allowed;        // dx*0.9/dt evaluated in double, stored as float (src/nclr.h:285)
  float mu0, lambda0;   // src/nclr.h:77-78
  float Dinv;           // 4 inv_dx^2 (src/nclr.h:325)
  float cscale;         // 4 inv_dx  (src/nclr.h:206,223)
  float dt_gravity;     // dt * gravity (src/nclr.h:292)
  int stress;           // kCorotated or kNeoHookean
  int thin_max;         // batches: blocks with fewer particles skip the shared-memory tiles
  int tail_max;         // single simulations: a block's last pass of fewer particles than
                        // this goes to the thin-block chunks (compact_blocks_kernel)
  int64_t nodes;        // N^dim
  int nb;               // grid blocks per axis: ceil(N / Tiling<dim>::BS)
  int nblocks;          // nb^dim
};

struct PState {
  float *x, *v, *F, *C, *Jp, *mass, *vol;  // v and C: see the layout note
  int *id;
  uint8_t *mat;     // may be null
  float2 *lame;     // per-particle (mu_0, lambda_0); null: the scene's P.mu0, P.lambda0
  uint16_t *scene;  // scene of each slot (batched simulations), null for a single scene
  int stride;       // component stride (capacity)
};

// One simulation of a batch (a single simulation is a batch of one).  Scenes share the
// particle store (scene s owns slots [slot_off, slot_off + n)), the grids G and V (scene s owns
// nodes [node_off, node_off + P.nodes)) and the block key space (blocks [block_off,
// block_off + P.nblocks)).
struct Scene {
  Params P;
  int64_t node_off;
  int block_off;
  int slot_off;
};

// ---------------------------------------------------------------------------------------
// Quadratic B-spline stencil (src/nclr.h:115-127 and 172-183): base = trunc(x inv_dx - 0.5)
// (the cast truncates toward zero), fx = x inv_dx - base, weights per axis.
// ---------------------------------------------------------------------------------------
template <int D>
__device__ __forceinline__ void stencil(const float x[D], float inv_dx, int base[D], float fx[D],
                                        float w[3][D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const float s = x[d] * inv_dx;
    base[d] = __float2int_rz(s - 0.5f);
    fx[d] = s - (float)base[d];
    const float a = 1.5f - fx[d], b = fx[d] - 1.0f, c = fx[d] - 0.5f;
    w[0][d] = 0.5f * (a * a);
    w[1][d] = 0.75f - b * b;
    w[2][d] = 0.5f * (c * c);
  }
}

template <int D>
__device__ __forceinline__ int64_t flat_index(const int b[D], int N) {
  if (D == 3) return ((int64_t)b[0] * N + b[1]) * N + b[D - 1];
  return (int64_t)b[0] * N + b[D - 1];
}

// Grid update of one node (src/nclr.h:284-310): if m > 0, v = (mv)/m, v_y += dt g, clamp to
// +-allowed; then the sticky boundary zeroes v when a node in the 3-node border moves
// outward.  `idx` is the node's per-axis index.
template <int D>
__device__ __forceinline__ void grid_update(const float4 g, const int idx[D], const Params &P,
                                            float v[D], float &m) {
  v[0] = g.x;
  v[1] = g.y;
  if (D == 3) v[D - 1] = g.z;
  m = g.w;
  if (m > 0.0f) {
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = v[d] / m;
    v[1] += P.dt_gravity;
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = clampf_(v[d], -P.allowed, P.allowed);
  }
  bool stick = false;
#pragma unroll
  for (int d = 0; d < D; ++d)
    stick |= (idx[d] < 3 && v[d] < 0.0f) || (idx[d] >= P.N - 3 && v[d] > 0.0f);
  if (stick) {
#pragma unroll
    for (int d = 0; d < D; ++d) v[d] = 0.0f;
    m = 0.0f;
  }
}

// Per-axis index of a node from its flat index (only needed when a stencil wraps).
template <int D>
__device__ __forceinline__ void unflatten(int64_t f, int N, int idx[D]) {
#pragma unroll
  for (int d = D - 1; d >= 0; --d) {
    idx[d] = (int)(f % N);
    f /= N;
  }
}

// The snow clamp's bounds on the singular values (src/nclr.h:237-241): 1 - 2.5e-2, 1 + 4.5e-3.
constexpr float kSnowLo = 1.0f - 2.5e-2f, kSnowHi = 1.0f + 4.5e-3f;

// hardening (src/nclr.h:351-372): snow e = exp(10 (1 - Jp)); jelly 0.3; liquid 1.0.
__device__ __forceinline__ float hardening(int material, float Jp) {
  if (material == kSnow) return expf(10.0f * (1.0f - Jp));
  return material == kJelly ? 0.3f : 1.0f;
}

// Base Lame parameters of slot p: its own (per-particle moduli) or the scene's.
__device__ __forceinline__ float2 lame0(const PState &s, int p, const Params &P) {
  return s.lame ? s.lame[p] : make_float2(P.mu0, P.lambda0);
}

// Affine momentum of the fused P2G (src/nclr.h:313-337):
//   A = -(dt vol) Dinv PF + m C, with the Kirchhoff stress PF of the scene's stress model:
//   fixed corotated  2 mu (F - R) F^T + constmat(lambda (J - 1) J)   (the reference; constmat
//                    adds the term to every entry, src/nclr_math.h:40-43)
//   neo-Hookean      mu (F F^T - I) + lambda ln(J) I                 (src/nclr.h:339's TODO;
//                    R is not used)
// mu, lambda = (mu_0, lambda_0) of `l0` times the material's hardening (src/nclr.h:351-372).
template <int D>
__device__ __forceinline__ Mat<D> fused_affine(const Mat<D> &F, const Mat<D> &R, const Mat<D> &C,
                                               float Jp, float m, float vol, int material,
                                               float2 l0, const Params &P) {
  const float e = hardening(material, Jp);
  const float mu = l0.x * e, lambda = l0.y * e;
  const float J = det(F);
  Mat<D> PF;
  float lam;
  bool every_entry;
  if (P.stress == kNeoHookean) {
    PF = mat_mul_t<D>(F, F);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) PF.a[i][j] = mu * (PF.a[i][j] - (i == j ? 1.0f : 0.0f));
    lam = lambda * logf(J);
    every_entry = false;
  } else {
    Mat<D> FmR;
    const float two_mu = 2.0f * mu;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) FmR.a[i][j] = two_mu * (F.a[i][j] - R.a[i][j]);
    PF = mat_mul_t<D>(FmR, F);
    lam = lambda * (J - 1.0f) * J;
    every_entry = true;
  }
  const float s = -(P.dt * vol);
  Mat<D> A;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j)
      A.a[i][j] = s * (P.Dinv * (PF.a[i][j] + ((every_entry || i == j) ? lam : 0.0f))) +
                  m * C.a[i][j];
  return A;
}

// The rotation the stress needs: the polar factor of F for the corotated model, nothing for
// the neo-Hookean one.  Snow takes it with correctly rounded rotations, as the fused step
// takes it from the clamp's SVD (the hardened snow stress amplifies a rotation's rounding).
template <int D>
__device__ __forceinline__ Mat<D> stress_R(const Mat<D> &F, const Params &P, int material) {
  if (P.stress == kNeoHookean) return F;
  return material == kSnow ? polar_R_exact(F) : polar_R(F);
}

template <int D>
__device__ __forceinline__ Mat<D> load_mat(const float *__restrict__ f, int stride, int p) {
  Mat<D> M;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M.a[i][j] = f[(size_t)(i * D + j) * stride + p];
  return M;
}

template <int D>
__device__ __forceinline__ void store_mat(float *__restrict__ f, int stride, int p, const Mat<D> &M) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) f[(size_t)(i * D + j) * stride + p] = M.a[i][j];
}

// diag<dim>(1) (src/nclr_math.h:13-19): reference physics sets only (0,0) and (1,1).
template <int D, bool kRef>
__device__ __forceinline__ float diag_one(int i, int j) {
  return (i == j && (!kRef || i < 2)) ? 1.0f : 0.0f;
}

__device__ __forceinline__ void red_add_v4(float4 *addr, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(a), "f"(b),
               "f"(c), "f"(d)
               : "memory");
}

}  // namespace mpm
