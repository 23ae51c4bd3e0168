// Reverse-mode kernels of one step (the adjoint of MPMSimulation<dim>::advance(),
// src/nclr.h:80-372, for jelly and for the plasticity of snow and liquid).  A step maps
// s_t = (x, v, F, C, Jp) to s_{t+1}; given the adjoint of s_{t+1} these kernels produce the
// adjoint of s_t and accumulate the adjoints of mu_0 and lambda_0:
//   adj_g2p   per particle: reverse of the G2P gather, F update (with the snow clamp or the
//             liquid reset) and advection; scatters the adjoint of the updated grid velocity
//             to the nodes;
//   adj_grid  per node: reverse of the grid update (v = clamp(mv / m + dt g)); clamped
//             components and stuck or empty nodes pass nothing;
//   adj_p2g   per particle: gathers the node adjoints, reverses the P2G scatter, the APIC +
//             stress term, the polar rotation and (snow) the Jp-dependent hardening.
// All arrays are particle-major rows in the caller's order (the layout of the C ABI) and the
// updated grid V_t of the step is the float4 {v, m} grid the forward step produced.
#include <cuda_runtime.h>

#include <type_traits>

#include "mpm_device.cuh"
#include "mpm_launch.h"

namespace mpm {

namespace {

template <int D>
struct Stencil {
  int base[D];
  float fx[D], w[3][D], dw[3][D];
};

template <int D>
__device__ __forceinline__ Stencil<D> make_stencil(const float x[D], float inv_dx) {
  Stencil<D> s;
  stencil<D>(x, inv_dx, s.base, s.fx, s.w);
#pragma unroll
  for (int d = 0; d < D; ++d) {
    const float f = s.fx[d];
    s.dw[0][d] = f - 1.5f;
    s.dw[1][d] = -2.0f * (f - 1.0f);
    s.dw[2][d] = f - 0.5f;
  }
  return s;
}

template <int D>
__device__ __forceinline__ void offs(int o, int oo[3]) {
  oo[0] = (D == 3) ? o / 9 : o / 3;
  oo[1] = (D == 3) ? (o / 3) % 3 : o % 3;
  oo[2] = (D == 3) ? o % 3 : 0;
}

template <int D>
__device__ __forceinline__ float wprod(const Stencil<D> &s, const int oo[3]) {
  float w = s.w[oo[0]][0] * s.w[oo[1]][1];
  if (D == 3) w *= s.w[oo[2]][D - 1];
  return w;
}

// d fx from the adjoint Wbar of one stencil weight W_o = prod_d w_d(o_d), accumulated node by
// node (so no array of the 27 weight adjoints stays live across the stencil loop).
template <int D>
__device__ __forceinline__ void weight_backward(const Stencil<D> &s, const int oo[3], float Wbar,
                                                float gfx[D]) {
#pragma unroll
  for (int d = 0; d < D; ++d) {
    float other = 1.0f;
#pragma unroll
    for (int e = 0; e < D; ++e)
      if (e != d) other *= s.w[oo[e]][e];
    gfx[d] += Wbar * other * s.dw[oo[d]][d];
  }
}

template <int D>
__device__ __forceinline__ Mat<D> load_row_mat(const float *a, int p) {
  Mat<D> m;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) m.a[i][j] = a[((size_t)p * D + i) * D + j];
  return m;
}

template <int D>
__device__ __forceinline__ void store_row_mat(float *a, int p, const Mat<D> &m) {
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) a[((size_t)p * D + i) * D + j] = m.a[i][j];
}

template <int D>
__device__ __forceinline__ Mat<D> row_mat_or_zero(const float *a, int p) {
  Mat<D> m;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) m.a[i][j] = a ? a[((size_t)p * D + i) * D + j] : 0.0f;
  return m;
}

__device__ __forceinline__ Mat<2> cofactor(const Mat<2> &a) {
  Mat<2> c;
  c.a[0][0] = a.a[1][1];
  c.a[0][1] = -a.a[1][0];
  c.a[1][0] = -a.a[0][1];
  c.a[1][1] = a.a[0][0];
  return c;
}
__device__ __forceinline__ Mat<3> cofactor(const Mat<3> &a) {
  Mat<3> c;
  c.a[0][0] = a.a[1][1] * a.a[2][2] - a.a[1][2] * a.a[2][1];
  c.a[0][1] = a.a[1][2] * a.a[2][0] - a.a[1][0] * a.a[2][2];
  c.a[0][2] = a.a[1][0] * a.a[2][1] - a.a[1][1] * a.a[2][0];
  c.a[1][0] = a.a[0][2] * a.a[2][1] - a.a[0][1] * a.a[2][2];
  c.a[1][1] = a.a[0][0] * a.a[2][2] - a.a[0][2] * a.a[2][0];
  c.a[1][2] = a.a[0][1] * a.a[2][0] - a.a[0][0] * a.a[2][1];
  c.a[2][0] = a.a[0][1] * a.a[1][2] - a.a[0][2] * a.a[1][1];
  c.a[2][1] = a.a[0][2] * a.a[1][0] - a.a[0][0] * a.a[1][2];
  c.a[2][2] = a.a[0][0] * a.a[1][1] - a.a[0][1] * a.a[1][0];
  return c;
}

// Adjoint of the polar rotation: 2D closed form (src/nclr_math.h:80-89); 3D with F = U S V^T,
// R = U V^T: F_bar = U Z V^T, Z_ij = (P_ij - P_ji) / (s_i + s_j), P = U^T R_bar V.
__device__ __forceinline__ Mat<2> polar_backward(const Mat<2> &F, const Mat<2> &Rb) {
  const float a = F.a[0][0] + F.a[1][1], b = F.a[1][0] - F.a[0][1];
  const float r2 = a * a + b * b;
  const float inv_r3 = 1.0f / (r2 * sqrtf(r2));
  const float cb = Rb.a[0][0] + Rb.a[1][1], sb = Rb.a[1][0] - Rb.a[0][1];
  const float ab = (cb * b * b - sb * a * b) * inv_r3;
  const float bb = (-cb * a * b + sb * a * a) * inv_r3;
  Mat<2> out;
  out.a[0][0] = ab;
  out.a[1][1] = ab;
  out.a[1][0] = bb;
  out.a[0][1] = -bb;
  return out;
}
// With the SVD of F already at hand (R = U V^T).
__device__ __forceinline__ Mat<3> polar_backward_svd(const Mat<3> &U, const float sg[3],
                                                     const Mat<3> &V, const Mat<3> &Rb) {
  // P = U^T Rb V
  Mat<3> UtR;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j)
      UtR.a[i][j] = U.a[0][i] * Rb.a[0][j] + U.a[1][i] * Rb.a[1][j] + U.a[2][i] * Rb.a[2][j];
  const Mat<3> Pm = mat_mul<3>(UtR, V);
  Mat<3> Z;
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float sden = sg[i] + sg[j];
      Z.a[i][j] = (i != j && fabsf(sden) > 1e-30f) ? (Pm.a[i][j] - Pm.a[j][i]) / sden : 0.0f;
    }
  return mat_mul_t<3>(mat_mul<3>(U, Z), V);
}

// The polar rotation of F and what its adjoint needs: 3D keeps the SVD, 2D nothing.
template <int D>
struct Polar;
template <>
struct Polar<2> {
  Mat<2> R;
  __device__ __forceinline__ explicit Polar(const Mat<2> &F) : R(polar_rotation(F)) {}
  __device__ __forceinline__ Mat<2> backward(const Mat<2> &F, const Mat<2> &Rb) const {
    return polar_backward(F, Rb);
  }
};
template <>
struct Polar<3> {
  Mat<3> U, V, R;
  float sg[3];
  __device__ __forceinline__ explicit Polar(const Mat<3> &F) {
    svd3<false>(F, U, sg, V);  // the same factorisation as the forward stress (polar_R)
    R = uvt<3>(U, V);
  }
  __device__ __forceinline__ Mat<3> backward(const Mat<3> &, const Mat<3> &Rb) const {
    return polar_backward_svd(U, sg, V, Rb);
  }
};
// What the neo-Hookean stress has in place of the polar rotation: nothing (R is unused).
template <int D>
struct NoPolar {
  Mat<D> R;
  __device__ __forceinline__ explicit NoPolar(const Mat<D> &F) : R(F) {}
};

}  // namespace

// Reverse of the snow plasticity of src/nclr.h:237-250 (F_hat -> F' = U f(S) V^T, f the clamp
// to [1 - 2.5e-2, 1 + 4.5e-3], and Jp' = clamp(Jp det F_hat / det F', 0.6, 20)) given the
// adjoints Fb of F' and Jpb of Jp': the adjoint of F_hat, and that of Jp into *Jp_bar.  With
// P_bar = U^T Fb V, the adjoint in the singular frame is K_ii = f'(s_i) P_bar_ii and
// K_ij = (a_ij + b_ij)/2 P_bar_ij + (a_ij - b_ij)/2 P_bar_ji, a_ij = (f_i - f_j) / (s_i - s_j),
// b_ij = (f_i + f_j) / (s_i + s_j) (the derivative of a function of the singular values;
// f' = 0 on a clamped value), plus the Jp terms on the diagonal; the result is U K V^T.  The
// SVD is the one the forward step takes (signed in 3D and in the corrected 2D physics).
template <int D, bool kRef>
__device__ __forceinline__ Mat<D> snow_backward(const Mat<D> &Fh, float Jp, const Mat<D> &Fb,
                                                float Jpb, float *Jp_bar) {
  Mat<D> U, V;
  float s[D], f[D], fp[D];
  if constexpr (D == 3) {
    svd3<true>(Fh, U, s, V);
  } else {
    svd2<kRef>(Fh, U, s, V);
  }
#pragma unroll
  for (int i = 0; i < D; ++i) {
    f[i] = clampf_(s[i], kSnowLo, kSnowHi);
    fp[i] = (s[i] > kSnowLo && s[i] < kSnowHi) ? 1.0f : 0.0f;
  }
  Mat<D> UtF;  // U^T Fb
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float acc = 0.0f;
#pragma unroll
      for (int k = 0; k < D; ++k) acc += U.a[k][i] * Fb.a[k][j];
      UtF.a[i][j] = acc;
    }
  const Mat<D> Pb = mat_mul<D>(UtF, V);
  Mat<D> K;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      if (i == j) {
        K.a[i][i] = fp[i] * Pb.a[i][i];
        continue;
      }
      const float dm = s[i] - s[j], dp = s[i] + s[j];
      const float a = fabsf(dm) > 1e-6f * (fabsf(s[i]) + fabsf(s[j])) ? (f[i] - f[j]) / dm
                                                                        : 0.5f * (fp[i] + fp[j]);
      const float b = fabsf(dp) > 1e-30f ? (f[i] + f[j]) / dp : 0.0f;
      K.a[i][j] = 0.5f * (a + b) * Pb.a[i][j] + 0.5f * (a - b) * Pb.a[j][i];
    }
  // Jp' = clamp(r, 0.6, 20), r = Jp prod s / prod f (the det U det V factors cancel)
  float ps = 1.0f, pf = 1.0f;
#pragma unroll
  for (int i = 0; i < D; ++i) {
    ps *= s[i];
    pf *= f[i];
  }
  const float r = Jp * ps / pf;
  if (r > 0.6f && r < 20.0f && Jpb != 0.0f) {
    *Jp_bar += Jpb * ps / pf;
#pragma unroll
    for (int i = 0; i < D; ++i) {
      float others = 1.0f;
#pragma unroll
      for (int k = 0; k < D; ++k)
        if (k != i) others *= s[k];
      K.a[i][i] += Jpb * (Jp * others / pf - r * fp[i] / f[i]);
    }
  }
  return mat_mul_t<D>(mat_mul<D>(U, K), V);
}

// ---------------------------------------------------------------------------------------
// adj_g2p: reverse of x' = x + dt v', v' = sum W vg, C' = 4 inv_dx sum W vg (o - fx)^T,
// F_hat = (I + dt C') F and the material's F' (jelly F_hat; snow the clamp, which also moves
// Jp; liquid the reset to diag with F'_00 = J, the product of the signed singular values).
// Writes the adjoint of x, F and Jp (partial; adj_p2g adds the P2G part) and scatters the
// adjoint of the updated grid velocity into VB.
// ---------------------------------------------------------------------------------------
// kMat >= 0 fixes the material at compile time (jelly: the plastic branches and their registers
// drop out); -1 reads it from `model_rt`.
template <int D, bool kRef, int kMat>
__global__ void __launch_bounds__(128) adj_g2p_kernel(
    int n, const float *__restrict__ x, const float *__restrict__ F,
    const float *__restrict__ Jp, const float *__restrict__ Cn, const float4 *__restrict__ V,
    Params P, int model_rt, const float *__restrict__ gx, const float *__restrict__ gv,
    const float *__restrict__ gF, const float *__restrict__ gC, const float *__restrict__ gJp,
    float *__restrict__ ox, float *__restrict__ oF, float *__restrict__ oJp,
    float *__restrict__ VB, int *err) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int model = kMat >= 0 ? kMat : model_rt;
  constexpr int S = (D == 3) ? 27 : 9;
  float xp[D];
#pragma unroll
  for (int d = 0; d < D; ++d) xp[d] = x[(size_t)p * D + d];
  const Stencil<D> st = make_stencil<D>(xp, P.inv_dx);
  const Mat<D> Fm = load_row_mat<D>(F, p);
  const Mat<D> Cm = load_row_mat<D>(Cn, p);
  Mat<D> gFn = row_mat_or_zero<D>(gF, p);
  Mat<D> gCt = row_mat_or_zero<D>(gC, p);
  Mat<D> M;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) M.a[i][j] = diag_one<D, kRef>(i, j) + P.dt * Cm.a[i][j];
  // the adjoint of F_hat = M F from that of F' (and Jp'), per material; gFn becomes it
  const float gJpn = gJp ? gJp[p] : 0.0f;
  float gJp0 = gJpn;  // jelly and liquid keep Jp
  if (model != kJelly) {
    const Mat<D> Fh = mat_mul<D>(M, Fm);
    if (model == kSnow) {
      gJp0 = 0.0f;
      gFn = snow_backward<D, kRef>(Fh, Jp[p], gFn, gJpn, &gJp0);
    } else {  // liquid: F'_00 = J = prod s = det F_hat (|det F_hat| where sigma >= 0, 2D reference)
      const float g00 = gFn.a[0][0];
      const float sgn = (D == 2 && kRef && det(Fh) < 0.0f) ? -1.0f : 1.0f;
      const Mat<D> cof = cofactor(Fh);
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) gFn.a[i][j] = g00 * sgn * cof.a[i][j];
    }
  }
  if (oJp) oJp[p] = gJp0;
  // F_bar = M^T gF'
  Mat<D> gFp;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = 0.0f;
#pragma unroll
      for (int k = 0; k < D; ++k) s += M.a[k][i] * gFn.a[k][j];
      gFp.a[i][j] = s;
    }
  store_row_mat<D>(oF, p, gFp);
  const Mat<D> gFFt = mat_mul_t<D>(gFn, Fm);
  float gvt[D], gxp[D];
#pragma unroll
  for (int i = 0; i < D; ++i) {
#pragma unroll
    for (int j = 0; j < D; ++j) gCt.a[i][j] += P.dt * gFFt.a[i][j];
    gxp[i] = gx ? gx[(size_t)p * D + i] : 0.0f;
    gvt[i] = (gv ? gv[(size_t)p * D + i] : 0.0f) + P.dt * gxp[i];
  }
  const float cs = P.cscale;
  float gfx[D];
#pragma unroll
  for (int d = 0; d < D; ++d) gfx[d] = 0.0f;
  const int64_t f0 = flat_index<D>(st.base, P.N);
#pragma unroll
  for (int o = 0; o < S; ++o) {
    int oo[3];
    offs<D>(o, oo);
    const int64_t f = (D == 3) ? f0 + ((int64_t)oo[0] * P.N + oo[1]) * P.N + oo[2]
                               : f0 + (int64_t)oo[0] * P.N + oo[1];
    if (f < 0 || f >= P.nodes) {
      atomicOr(err, kErrOutOfRange);
      continue;
    }
    const float4 g4 = __ldg(V + f);
    const float vg[3] = {g4.x, g4.y, g4.z};
    const float W = wprod<D>(st, oo);
    float du[D];
#pragma unroll
    for (int d = 0; d < D; ++d) du[d] = (float)oo[d] - st.fx[d];
    float wb = 0.0f, add[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int a = 0; a < D; ++a) {
      float gcdu = 0.0f;
#pragma unroll
      for (int b = 0; b < D; ++b) gcdu += gCt.a[a][b] * du[b];
      add[a] = W * gvt[a] + cs * W * gcdu;
      wb += gvt[a] * vg[a] + cs * vg[a] * gcdu;
    }
    red_add_v4(reinterpret_cast<float4 *>(VB) + f, add[0], add[1], add[2], 0.0f);
    weight_backward<D>(st, oo, wb, gfx);
#pragma unroll
    for (int b = 0; b < D; ++b) {
      float gctv = 0.0f;
#pragma unroll
      for (int a = 0; a < D; ++a) gctv += gCt.a[a][b] * vg[a];
      gfx[b] -= cs * W * gctv;
    }
  }
#pragma unroll
  for (int d = 0; d < D; ++d) ox[(size_t)p * D + d] = gxp[d] + P.inv_dx * gfx[d];
}

// ---------------------------------------------------------------------------------------
// adj_grid: reverse of vg = clamp(mv / m + dt g e_y) (src/nclr.h:284-298) from the updated
// grid V (its m is 0 where the node was empty or stuck).  VB is cleared for the next step.
// ---------------------------------------------------------------------------------------
template <int D>
__global__ void __launch_bounds__(256) adj_grid_kernel(const float4 *__restrict__ V,
                                                       float *__restrict__ VB,
                                                       float4 *__restrict__ GB, Params P) {
  const int64_t f = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= P.nodes) return;
  const float4 g4 = V[f];
  const float vg[3] = {g4.x, g4.y, g4.z};
  const float m = g4.w;
  float gmv[3] = {0.0f, 0.0f, 0.0f}, gm = 0.0f;
  if (m > 0.0f) {
#pragma unroll
    for (int d = 0; d < D; ++d) {
      const float u = VB[f * 4 + d];
      if (fabsf(vg[d]) >= P.allowed) continue;  // clamped
      const float raw = vg[d] - (d == 1 ? P.dt_gravity : 0.0f);
      gmv[d] = u / m;
      gm -= u * raw / m;
    }
  }
  GB[f] = make_float4(gmv[0], gmv[1], gmv[2], gm);
  reinterpret_cast<float4 *>(VB)[f] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// (hi, lo) += (h2, l2) for sums kept as unevaluated pairs of floats: Knuth's TwoSum gives the
// rounding error of hi + h2 exactly, and the low parts collect it.
__device__ __forceinline__ void pair_add(float &hi, float &lo, float h2, float l2) {
  const float s = __fadd_rn(hi, h2);
  const float bp = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(h2, bp));
  hi = s;
  lo = lo + l2 + err;
}

// ---------------------------------------------------------------------------------------
// adj_p2g: reverse of mv_i += W (m v + A dpos), m_i += W m, with the fused APIC + stress
// A = -(dt vol Dinv) PF + m C (jelly: mu = 0.3 mu_0, lambda = 0.3 lambda_0) and PF the
// fixed-corotated 2 mu (F - R) F^T + lambda (J - 1) J 1 or (kStress == kNeoHookean)
// mu (F F^T - I) + lambda ln(J) I.  Adds to the adjoints of x and F, writes those of v and C,
// and accumulates the adjoints of mu_0 and lambda_0 into gml[0..1].  With per-particle moduli
// (rm.lame: each row's mu_0, lambda_0) it also accumulates each row's own adjoints into
// rm.grad[2 row], rm.grad[2 row + 1]: one thread per row, so no atomics.
// ---------------------------------------------------------------------------------------
template <int D, int kStress, int kMat>
__global__ void __launch_bounds__(128) adj_p2g_kernel(
    int n, const float *__restrict__ x, const float *__restrict__ v, const float *__restrict__ F,
    const float *__restrict__ C, const float *__restrict__ Jp, const float *__restrict__ mass,
    const float *__restrict__ vol, const float4 *__restrict__ GB, Params P, int model_rt,
    float *__restrict__ ox, float *__restrict__ ov, float *__restrict__ oF,
    float *__restrict__ oC, float *__restrict__ oJp, double *gml, RowModuli rm, int *err) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int model = kMat >= 0 ? kMat : model_rt;  // as in adj_g2p_kernel
  constexpr int S = (D == 3) ? 27 : 9;
  float gmu = 0.0f, glam = 0.0f;
  if (p < n) {
    float xp[D], vp[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      xp[d] = x[(size_t)p * D + d];
      vp[d] = v[(size_t)p * D + d];
    }
    const Stencil<D> st = make_stencil<D>(xp, P.inv_dx);
    const Mat<D> Fm = load_row_mat<D>(F, p);
    const Mat<D> Cm = load_row_mat<D>(C, p);
    const float m = mass[p], vo = vol[p];
    const float2 l0 = rm.lame ? rm.lame[p] : make_float2(P.mu0, P.lambda0);
    // the corotated stress's polar rotation, whose factorisation its adjoint reuses
    const std::conditional_t<kStress == kNeoHookean, NoPolar<D>, Polar<D>> pol(Fm);
    const float Jpp = Jp ? Jp[p] : 1.0f;
    const Mat<D> A = fused_affine<D>(Fm, pol.R, Cm, Jpp, m, vo, model, l0, P);
    Mat<D> gA;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gA.a[i][j] = 0.0f;
    float gvp[D], gfx[D];
#pragma unroll
    for (int d = 0; d < D; ++d) {
      gvp[d] = 0.0f;
      gfx[d] = 0.0f;
    }
    const int64_t f0 = flat_index<D>(st.base, P.N);
#pragma unroll
    for (int o = 0; o < S; ++o) {
      int oo[3];
      offs<D>(o, oo);
      const int64_t f = (D == 3) ? f0 + ((int64_t)oo[0] * P.N + oo[1]) * P.N + oo[2]
                                 : f0 + (int64_t)oo[0] * P.N + oo[1];
      if (f < 0 || f >= P.nodes) {
        atomicOr(err, kErrOutOfRange);
        continue;
      }
      const float4 g4 = __ldg(GB + f);
      const float g[3] = {g4.x, g4.y, g4.z};
      const float W = wprod<D>(st, oo);
      float dpos[D];
#pragma unroll
      for (int d = 0; d < D; ++d) dpos[d] = ((float)oo[d] - st.fx[d]) * P.dx;
      float wb = g4.w * m;
#pragma unroll
      for (int a = 0; a < D; ++a) {
        float ad = 0.0f;
#pragma unroll
        for (int b = 0; b < D; ++b) {
          ad += A.a[a][b] * dpos[b];
          gA.a[a][b] += W * g[a] * dpos[b];
        }
        gvp[a] += W * m * g[a];
        wb += g[a] * (m * vp[a] + ad);
      }
      weight_backward<D>(st, oo, wb, gfx);
#pragma unroll
      for (int b = 0; b < D; ++b) {
        float atg = 0.0f;
#pragma unroll
        for (int a = 0; a < D; ++a) atg += A.a[a][b] * g[a];
        gfx[b] -= P.dx * W * atg;
      }
    }
#pragma unroll
    for (int d = 0; d < D; ++d) {
      ox[(size_t)p * D + d] += P.inv_dx * gfx[d];
      ov[(size_t)p * D + d] = gvp[d];
    }
    Mat<D> gC;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gC.a[i][j] = m * gA.a[i][j];
    store_row_mat<D>(oC, p, gC);
    // stress
    const float kappa = P.dt * vo * P.Dinv;
    const float e = hardening(model, Jpp);  // src/nclr.h:351-372
    const float mu = l0.x * e, lam = l0.y * e;
    const float J = det(Fm);
    Mat<D> gF = load_row_mat<D>(oF, p);
    const Mat<D> cof = cofactor(Fm);  // d det(F) / dF = J F^-T
    if constexpr (kStress == kNeoHookean) {
      // PF = mu (F F^T - I) + lambda ln(J) I; G = dL/dPF:
      //   F_bar = mu (G + G^T) F + lambda tr(G) F^-T, mu_bar = <G, F F^T - I>,
      //   lambda_bar = tr(G) ln(J)
      Mat<D> G;
      float trG = 0.0f;
#pragma unroll
      for (int i = 0; i < D; ++i) {
#pragma unroll
        for (int j = 0; j < D; ++j) G.a[i][j] = -kappa * gA.a[i][j];
        trG += G.a[i][i];
      }
      const Mat<D> FFt = mat_mul_t<D>(Fm, Fm);
      Mat<D> Sg;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) {
          gmu += G.a[i][j] * (FFt.a[i][j] - (i == j ? 1.0f : 0.0f));
          Sg.a[i][j] = mu * (G.a[i][j] + G.a[j][i]);
        }
      glam = trG * logf(J);
      const Mat<D> SF = mat_mul<D>(Sg, Fm);
      const float c = lam * trG / J;
#pragma unroll
      for (int i = 0; i < D; ++i)
#pragma unroll
        for (int j = 0; j < D; ++j) gF.a[i][j] += SF.a[i][j] + c * cof.a[i][j];
    } else {
    const Mat<D> &R = pol.R;
    Mat<D> X, G;
    float sbar = 0.0f;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        X.a[i][j] = Fm.a[i][j] - R.a[i][j];
        G.a[i][j] = -kappa * gA.a[i][j];
        sbar += G.a[i][j];
      }
    const Mat<D> Q = mat_mul_t<D>(X, Fm);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gmu += 2.0f * G.a[i][j] * Q.a[i][j];
    glam = sbar * (J - 1.0f) * J;
    Mat<D> Qb;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) Qb.a[i][j] = 2.0f * mu * G.a[i][j];
    const Mat<D> Xb = mat_mul<D>(Qb, Fm);
    Mat<D> Rb, FQ;
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) {
        Rb.a[i][j] = -Xb.a[i][j];
        float s = 0.0f;
#pragma unroll
        for (int k = 0; k < D; ++k) s += Qb.a[k][i] * X.a[k][j];
        FQ.a[i][j] = s;
      }
    const Mat<D> Fp = pol.backward(Fm, Rb);
    const float dJ = sbar * lam * (2.0f * J - 1.0f);
#pragma unroll
    for (int i = 0; i < D; ++i)
#pragma unroll
      for (int j = 0; j < D; ++j) gF.a[i][j] += FQ.a[i][j] + Xb.a[i][j] + Fp.a[i][j] + dJ * cof.a[i][j];
    }
    store_row_mat<D>(oF, p, gF);
    // snow: e = exp(10 (1 - Jp)), so the adjoint of Jp gains (mu_0 mu_bar + lambda_0
    // lambda_bar) de/dJp with de/dJp = -10 e (gmu, glam: the adjoints of the hardened pair)
    if (model == kSnow && oJp) oJp[p] += (gmu * l0.x + glam * l0.y) * (-10.0f * e);
    gmu *= e;  // the adjoints of mu_0 and lambda_0
    glam *= e;
    if (rm.grad) {
      rm.grad[2 * (size_t)p] += gmu;
      rm.grad[2 * (size_t)p + 1] += glam;
    }
  }
  // warp reduction of the parameter adjoints, one double atomic per warp; the sums are carried
  // as unevaluated FP32 pairs (hi + lo), so they keep double-class accuracy without the FP64 pipe
  float ah = gmu, al = 0.0f, bh = glam, bl = 0.0f;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pair_add(ah, al, __shfl_xor_sync(0xffffffffu, ah, o), __shfl_xor_sync(0xffffffffu, al, o));
    pair_add(bh, bl, __shfl_xor_sync(0xffffffffu, bh, o), __shfl_xor_sync(0xffffffffu, bl, o));
  }
  if ((threadIdx.x & 31) == 0 && (ah != 0.0f || bh != 0.0f)) {
    atomicAdd(gml, (double)ah + (double)al);
    atomicAdd(gml + 1, (double)bh + (double)bl);
  }
}

// ---------------------------------------------------------------------------------------
template <int D>
void launch_adjoint_step(int n, const float *x, const float *v, const float *F, const float *C,
                         const float *Jp, const float *Cn, const float *mass, const float *vol,
                         const float4 *V, const Params &P, bool ref, const float *gx,
                         const float *gv, const float *gF, const float *gC, const float *gJp,
                         float *ox, float *ov, float *oF, float *oC, float *oJp, float *VB,
                         float4 *GB, double *gml, RowModuli rm, int *err, cudaStream_t st,
                         cudaEvent_t *ev) {
  const unsigned pb = (unsigned)((n + 127) / 128);
  const int model = P.model;
  if (ev) cudaEventRecord(ev[0], st);
  // jelly rollouts run the kernels with the material fixed (fewer registers, more warps
  // resident to cover the grid gathers); snow and liquid the runtime-material ones
  const bool jelly = model == kJelly;
  auto g2p = [&](auto r, auto mat) {
    adj_g2p_kernel<D, decltype(r)::value, decltype(mat)::value><<<pb, 128, 0, st>>>(
        n, x, F, Jp, Cn, V, P, model, gx, gv, gF, gC, gJp, ox, oF, oJp, VB, err);
  };
  using Jel = std::integral_constant<int, kJelly>;
  using Any = std::integral_constant<int, -1>;
  if (n > 0) {
    if (ref) {
      if (jelly) g2p(std::true_type{}, Jel{});
      else g2p(std::true_type{}, Any{});
    } else {
      if (jelly) g2p(std::false_type{}, Jel{});
      else g2p(std::false_type{}, Any{});
    }
  }
  if (ev) cudaEventRecord(ev[1], st);
  adj_grid_kernel<D><<<(unsigned)((P.nodes + 255) / 256), 256, 0, st>>>(V, VB, GB, P);
  if (ev) cudaEventRecord(ev[2], st);
  auto p2g = [&](auto stress, auto mat) {
    adj_p2g_kernel<D, decltype(stress)::value, decltype(mat)::value><<<pb, 128, 0, st>>>(
        n, x, v, F, C, Jp, mass, vol, GB, P, model, ox, ov, oF, oC, oJp, gml, rm, err);
  };
  using Neo = std::integral_constant<int, kNeoHookean>;
  using Cor = std::integral_constant<int, kCorotated>;
  if (n > 0) {
    if (P.stress == kNeoHookean) {
      if (jelly) p2g(Neo{}, Jel{});
      else p2g(Neo{}, Any{});
    } else {
      if (jelly) p2g(Cor{}, Jel{});
      else p2g(Cor{}, Any{});
    }
  }
  if (ev) cudaEventRecord(ev[3], st);
}

namespace {

// Row q's E and nu adjoints from its mu_0 / lambda_0 adjoints (src/nclr.h:77-78):
//   dmu/dE = 1 / (2 (1 + nu)),  dmu/dnu = -E / (2 (1 + nu)^2),
//   dlambda/dE = nu / q,  dlambda/dnu = E (1 + 2 nu^2) / q^2,  q = (1 + nu)(1 - 2 nu).
__global__ void moduli_grads_kernel(int n, const float *__restrict__ E, const float *__restrict__ nu,
                                    const double *__restrict__ grad, float *__restrict__ gE,
                                    float *__restrict__ gnu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double e = E[i], v = nu[i], gm = grad[2 * (size_t)i], gl = grad[2 * (size_t)i + 1];
  const double q = (1.0 + v) * (1.0 - 2.0 * v);
  if (gE) gE[i] = (float)(gm / (2.0 * (1.0 + v)) + gl * v / q);
  if (gnu) gnu[i] = (float)(-gm * e / (2.0 * (1.0 + v) * (1.0 + v)) + gl * e * (1.0 + 2.0 * v * v) / (q * q));
}

}  // namespace

cudaError_t launch_moduli_grads(int n, const float *E, const float *nu, const double *grad,
                                float *gE, float *gnu, cudaStream_t st) {
  if (n > 0) moduli_grads_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, E, nu, grad, gE, gnu);
  return cudaGetLastError();
}

template void launch_adjoint_step<2>(int, const float *, const float *, const float *, const float *,
                                     const float *, const float *, const float *, const float *,
                                     const float4 *, const Params &, bool, const float *,
                                     const float *, const float *, const float *, const float *,
                                     float *, float *, float *, float *, float *, float *,
                                     float4 *, double *, RowModuli, int *, cudaStream_t,
                                     cudaEvent_t *);
template void launch_adjoint_step<3>(int, const float *, const float *, const float *, const float *,
                                     const float *, const float *, const float *, const float *,
                                     const float4 *, const Params &, bool, const float *,
                                     const float *, const float *, const float *, const float *,
                                     float *, float *, float *, float *, float *, float *,
                                     float4 *, double *, RowModuli, int *, cudaStream_t,
                                     cudaEvent_t *);

}  // namespace mpm
