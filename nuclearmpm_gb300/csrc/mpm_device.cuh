// Device side of the MLS-MPM step (the reference's MPMSimulation<dim>::advance(),
// src/nclr.h:80-310), written for sm_103a.
//
// HBM layout
//   particles  SoA, component-major: field component c of particle slot p at
//              field[c * stride + p] (x, v: dim comps; F, C: dim*dim comps, row-major;
//              Jp, mass, volume: 1).  `id[p]` is the caller's index of slot p: slots are
//              re-sorted by grid cell every few steps, the caller's order is restored on
//              download.  `mat[p]` (optional) is a per-particle material.
//   payload    the P2G input of each slot, computed by the previous G2P (or by
//              prepare_payload after an upload): 3D {x0,x1,x2,m} {mv0,mv1,mv2,A00}
//              {A01,A02,A10,A11} {A12,A20,A21,A22}; 2D {x0,x1,m,mv0} {mv1,A00,A01,A10}
//              {A11,0,0,0}, where A is the fused APIC + stress matrix (src/nclr.h:313-337)
//              and mv = m v.  One 64 B (3D) / 48 B (2D) record per slot, read whole.
//   grid       dense (res+1)^dim float4 nodes {sum w m v (x,y,z), sum w m}, the reference's
//              x-major node order; zeroed before each P2G.  The grid update (normalise,
//              gravity, clamp, sticky boundary; src/nclr.h:263-310) is applied on the fly
//              where nodes are read (G2P, grid export), never stored.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mpm_math.cuh"

namespace mpm {

enum : int { kSnow = 0, kJelly = 1, kLiquid = 2 };
enum : int { kErrOutOfRange = 1 };

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
  int64_t nodes;        // N^dim
};

struct PState {
  float *x, *v, *F, *C, *Jp, *mass, *vol;
  int *id;
  uint8_t *mat;  // may be null
  int stride;    // component stride (capacity)
};

template <int D>
struct PayloadRecs {
  static constexpr int value = (D == 3) ? 4 : 3;
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

// hardening (src/nclr.h:351-372): snow e = exp(10 (1 - Jp)); jelly 0.3; liquid 1.0.
__device__ __forceinline__ float hardening(int material, float Jp) {
  if (material == kSnow) return expf(10.0f * (1.0f - Jp));
  return material == kJelly ? 0.3f : 1.0f;
}

// first_piola_kirchoff_stress (src/nclr.h:313-337):
//   A = -(dt vol) Dinv (2 mu (F - R) F^T + constmat(lambda (J - 1) J)) + m C
template <int D>
__device__ __forceinline__ Mat<D> fused_affine(const Mat<D> &F, const Mat<D> &R, const Mat<D> &C,
                                               float Jp, float m, float vol, int material,
                                               const Params &P) {
  const float e = hardening(material, Jp);
  const float mu = P.mu0 * e, lambda = P.lambda0 * e;
  const float J = det(F);
  Mat<D> FmR;
  const float two_mu = 2.0f * mu;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) FmR.a[i][j] = two_mu * (F.a[i][j] - R.a[i][j]);
  const Mat<D> PF = mat_mul_t<D>(FmR, F);
  const float lam = lambda * (J - 1.0f) * J;
  const float s = -(P.dt * vol);
  Mat<D> A;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) A.a[i][j] = s * (P.Dinv * (PF.a[i][j] + lam)) + m * C.a[i][j];
  return A;
}

template <int D>
__device__ __forceinline__ void store_payload(float4 *__restrict__ pay, int p, const float x[D],
                                              float m, const float v[D], const Mat<D> &A) {
  if (D == 3) {
    float4 *r = pay + (size_t)p * 4;
    r[0] = make_float4(x[0], x[1], x[D - 1], m);
    r[1] = make_float4(v[0] * m, v[1] * m, v[D - 1] * m, A.a[0][0]);
    r[2] = make_float4(A.a[0][1], A.a[0][D - 1], A.a[1][0], A.a[1][1]);
    r[3] = make_float4(A.a[1][D - 1], A.a[D - 1][0], A.a[D - 1][1], A.a[D - 1][D - 1]);
  } else {
    float4 *r = pay + (size_t)p * 3;
    r[0] = make_float4(x[0], x[1], m, v[0] * m);
    r[1] = make_float4(v[1] * m, A.a[0][0], A.a[0][1], A.a[1][0]);
    r[2] = make_float4(A.a[1][1], 0.0f, 0.0f, 0.0f);
  }
}

template <int D>
__device__ __forceinline__ void load_payload(const float4 *__restrict__ pay, int p, float x[D],
                                             float &m, float mv[D], Mat<D> &A) {
  if (D == 3) {
    const float4 *r = pay + (size_t)p * 4;
    const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), e = __ldg(r + 3);
    x[0] = a.x; x[1] = a.y; x[D - 1] = a.z; m = a.w;
    mv[0] = b.x; mv[1] = b.y; mv[D - 1] = b.z;
    A.a[0][0] = b.w; A.a[0][1] = c.x; A.a[0][D - 1] = c.y;
    A.a[1][0] = c.z; A.a[1][1] = c.w; A.a[1][D - 1] = e.x;
    A.a[D - 1][0] = e.y; A.a[D - 1][1] = e.z; A.a[D - 1][D - 1] = e.w;
  } else {
    const float4 *r = pay + (size_t)p * 3;
    const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2);
    x[0] = a.x; x[1] = a.y; m = a.z; mv[0] = a.w;
    mv[1] = b.x; A.a[0][0] = b.y; A.a[0][1] = b.z; A.a[1][0] = b.w;
    A.a[1][1] = c.x;
  }
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
