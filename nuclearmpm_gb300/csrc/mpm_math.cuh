// Register-resident small-matrix math for the MPM step: 2x2/3x3 determinant, products, the
// reference's polar decomposition (src/nclr_math.h:76-98) and signed SVD (src/nclr_math.h:
// 50-74).  Everything is plain FP32 on values held in registers; the functions are
// __host__ __device__ so the same code can be exercised on a CPU.
//
// SVD conventions (what the reference's nclr_svd returns after its sign fix):
//   3D: U, V rotations, sigma_1 >= sigma_2 >= |sigma_3|, sigma_3 carrying sign(det A).
//   2D: U, V rotations and sigma_2 carrying sign(det A)  (corrected physics), or
//       U, V possibly reflections and sigma >= 0          (reference physics: its 2D sign
//       fix writes out of bounds and is a no-op).
#pragma once

#include <math.h>
#include <stdint.h>

#ifdef __CUDACC__
#define MPM_HD __host__ __device__ __forceinline__
#else
#define MPM_HD inline
#endif

namespace mpm {

// a / b with the fast reciprocal on the device (no special-value path; |b| < 2^126)
MPM_HD float fast_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}
MPM_HD double fast_div(double a, double b) { return a / b; }

MPM_HD float rsqrt_(float x) {
#ifdef __CUDA_ARCH__
  return rsqrtf(x);
#else
  return 1.0f / sqrtf(x);
#endif
}
MPM_HD double rsqrt_(double x) {
#ifdef __CUDA_ARCH__
  return rsqrt(x);
#else
  return 1.0 / sqrt(x);
#endif
}

// Scalar helpers in both precisions (the SVD below runs in FP32, and in FP64 where the snow
// clamp needs it).
MPM_HD float sqrt_(float x) { return sqrtf(x); }
MPM_HD double sqrt_(double x) { return sqrt(x); }
MPM_HD float fabs_(float x) { return fabsf(x); }
MPM_HD double fabs_(double x) { return fabs(x); }
MPM_HD float copysign_(float a, float b) { return copysignf(a, b); }
MPM_HD double copysign_(double a, double b) { return copysign(a, b); }

template <int D>
struct Mat {
  float a[D][D];
};

template <int D>
MPM_HD Mat<D> mat_mul(const Mat<D> &x, const Mat<D> &y) {
  Mat<D> r;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = x.a[i][0] * y.a[0][j];
#pragma unroll
      for (int k = 1; k < D; ++k) s = s + x.a[i][k] * y.a[k][j];
      r.a[i][j] = s;
    }
  return r;
}

// x * y^T
template <int D>
MPM_HD Mat<D> mat_mul_t(const Mat<D> &x, const Mat<D> &y) {
  Mat<D> r;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) {
      float s = x.a[i][0] * y.a[j][0];
#pragma unroll
      for (int k = 1; k < D; ++k) s = s + x.a[i][k] * y.a[j][k];
      r.a[i][j] = s;
    }
  return r;
}

// Determinant by cofactor expansion along the first row.
MPM_HD float det(const Mat<2> &m) { return m.a[0][0] * m.a[1][1] - m.a[0][1] * m.a[1][0]; }
MPM_HD float det(const Mat<3> &m) {
  return m.a[0][0] * (m.a[1][1] * m.a[2][2] - m.a[1][2] * m.a[2][1]) -
         m.a[0][1] * (m.a[1][0] * m.a[2][2] - m.a[1][2] * m.a[2][0]) +
         m.a[0][2] * (m.a[1][0] * m.a[2][1] - m.a[1][1] * m.a[2][0]);
}

// Reference 2D polar rotation (src/nclr_math.h:80-89): closed form.
MPM_HD Mat<2> polar_rotation(const Mat<2> &m) {
  const float x = m.a[0][0] + m.a[1][1];
  const float y = m.a[1][0] - m.a[0][1];
  const float scale = 1.0f / sqrtf(x * x + y * y);
  const float c = x * scale, s = y * scale;
  Mat<2> R;
  R.a[0][0] = c;
  R.a[0][1] = -s;
  R.a[1][0] = s;
  R.a[1][1] = c;
  return R;
}

MPM_HD float atan2_(float y, float x) { return atan2f(y, x); }
MPM_HD double atan2_(double y, double x) { return atan2(y, x); }
MPM_HD void sincos_(float a, float *s, float *c) { sincosf(a, s, c); }
MPM_HD void sincos_(double a, double *s, double *c) {
#ifdef __CUDA_ARCH__
  sincos(a, s, c);
#else
  *s = sin(a);
  *c = cos(a);
#endif
}

// 2x2 SVD in closed form.  With E=(a00+a11)/2, F=(a00-a11)/2, G=(a10+a01)/2,
// H=(a10-a01)/2:  A = rot(phi) diag(Q+R, Q-R) rot(theta), Q = |(E,H)|, R = |(F,G)|,
// phi = (atan2(H,E) + atan2(G,F))/2, theta = (atan2(H,E) - atan2(G,F))/2.
// So U = rot(phi), V = rot(theta)^T; sigma_2 = Q - R carries sign(det A).
template <bool kNonNegative, typename T>
MPM_HD void svd2_t(const T A[2][2], T U[2][2], T sig[2], T V[2][2]) {
  const T E = T(0.5) * (A[0][0] + A[1][1]);
  const T F = T(0.5) * (A[0][0] - A[1][1]);
  const T G = T(0.5) * (A[1][0] + A[0][1]);
  const T H = T(0.5) * (A[1][0] - A[0][1]);
  const T Q = sqrt_(E * E + H * H);
  const T R = sqrt_(F * F + G * G);
  const T a1 = atan2_(G, F), a2 = atan2_(H, E);
  const T phi = T(0.5) * (a2 + a1), theta = T(0.5) * (a2 - a1);
  T sp, cp, st, ct;
  sincos_(phi, &sp, &cp);
  sincos_(theta, &st, &ct);
  sig[0] = Q + R;
  sig[1] = Q - R;
  U[0][0] = cp;
  U[0][1] = -sp;
  U[1][0] = sp;
  U[1][1] = cp;
  // V = rot(theta)^T
  V[0][0] = ct;
  V[0][1] = st;
  V[1][0] = -st;
  V[1][1] = ct;
  if (kNonNegative && sig[1] < T(0)) {
    sig[1] = -sig[1];
    U[0][1] = -U[0][1];
    U[1][1] = -U[1][1];
  }
}

template <bool kNonNegative>
MPM_HD void svd2(const Mat<2> &A, Mat<2> &U, float sig[2], Mat<2> &V) {
  svd2_t<kNonNegative, float>(A.a, U.a, sig, V.a);
}

// ---------------------------------------------------------------------------------------
// 3x3 SVD following the structure of McAdams, Selle, Tamstorf, Teran, Sifakis, "Computing
// the Singular Value Decomposition of 3x3 matrices with minimal branching and elementary
// floating point operations" (UW-Madison TR1690, 2011), with exact Jacobi rotations:
//   1. cyclic Jacobi eigen-analysis of S = A^T A, V = product of the rotations;
//   2. B = A V, columns sorted by decreasing norm (one column negated per swap so that V
//      stays a rotation);
//   3. Givens QR of B: B = U R, with U a rotation; sigma = diag(R), so sigma_3 carries
//      sign(det A).
// ---------------------------------------------------------------------------------------
namespace detail {

// Jacobi sweeps and stopping threshold per precision: done once every S_pq^2 is below
// (2 eps)^2 S_pp S_qq, eps the precision's unit roundoff (2.4e-7 in FP32; 1.1e-16 in FP64).
template <typename T>
struct JacobiLimits;
template <>
struct JacobiLimits<float> {
  static constexpr int kSweeps = 4;
  static constexpr float kDone = 2.3e-13f;  // (4.8e-7)^2
};
template <>
struct JacobiLimits<double> {
  static constexpr int kSweeps = 6;
  static constexpr double kDone = 4.9e-32;  // (2.2e-16)^2
};

// Conjugate symmetric S (stored full) by the Jacobi rotation in the (p,q) plane that zeroes
// S_pq (the symmetric Schur rotation of Golub & Van Loan, Alg. 8.4.2, in the numerically
// stable small-angle form); accumulate it into V (V <- V Q).
// kExact: the rotation's cosine (here and in qr_givens) is correctly rounded rather than from
// the approximate reciprocal square root, so a rotation by a rounding-level angle is exactly
// the identity and the singular values of a matrix that is the identity to within rounding
// come out exactly 1.  Plasticity needs that (the liquid's J = prod sigma enters the
// pressure lambda (J - 1) J on every entry; snow recomposes F from the clamped sigma); the
// polar rotation of the stress does not, and takes the cheaper form below.  kExact only
// concerns FP32: the FP64 results are rounded to FP32, and FP64 takes the cheaper form
// whatever kExact says.
template <int P, int Q, bool kExact, typename T>
MPM_HD void jacobi_rotate(T S[3][3], T V[3][3]) {
  constexpr int R = 3 - P - Q;
  const T app = S[P][P], aqq = S[Q][Q], apq = S[P][Q];
  if (apq == T(0)) return;
  T c, s, t;
  if constexpr (sizeof(T) == 8 || !kExact) {
    // FP64 (the snow clamp's fix-up, where the FP64 pipe is the limit) and the FP32 polar
    // rotation of the stress: a pair already below the stopping threshold is left alone, the
    // rotation comes from two reciprocal square roots and no division, and S is updated in
    // five products (below).  With d = S_qq - S_pp, e = 2 S_pq and h = |(d, e)|:
    // t = sgn(d) e / (h + |d|); with g = 1 / sqrt(2 h (h + |d|)), c = (h + |d|) g,
    // s = sgn(d) e g (so c^2 + s^2 = 1) and t = s / c = 2 h g^2 sgn(d) e.  For the polar
    // rotation, measured on the 1M jelly scene, fused launch: 157 -> 152 us under the
    // corrected physics (where F has full rank), 142 -> 141 us under the reference's.
    if (apq * apq <= JacobiLimits<T>::kDone * fabs_(app * aqq)) return;
    T d = aqq - app, e = T(2) * apq;
    if constexpr (sizeof(T) == 4) {
      // c, s and t depend on d / e only: scaled so the larger is 1, d^2 + e^2 cannot
      // underflow (a pair below the normal range is numerically zero: left alone)
      const T mx = fmaxf(fabsf(d), fabsf(e));
      if (!(mx > 1e-36f)) return;
      const T r = fast_div(1.0f, mx);
      d *= r;
      e *= r;
    }
    const T ad = fabs_(d);
    const T q = d * d + e * e;
    const T h = q * rsqrt_(q);
    const T g = rsqrt_(T(2) * h * (h + ad));
    const T se = copysign_(T(1), d) * e;
    c = (h + ad) * g;
    s = se * g;
    t = T(2) * h * g * g * se;
  } else {
    // tau and t only choose the angle; c and s below are formed from t consistently, so the
    // fast reciprocal does here (|tau| -> inf gives t = 0, the identity)
    const T tau = fast_div(aqq - app, T(2) * apq);
    t = fast_div(copysign_(T(1), tau), fabs_(tau) + sqrt_(T(1) + tau * tau));
    c = kExact ? T(1) / sqrt_(T(1) + t * t) : rsqrt_(T(1) + t * t);
    s = t * c;
  }
  // S <- Q^T S Q with Q = I except Q_pp = c, Q_pq = s, Q_qp = -s, Q_qq = c
  if constexpr (sizeof(T) == 8 || !kExact) {
    // the rotated diagonal is S_pp - t S_pq and S_qq + t S_pq, and only the two entries in the
    // third row and column mix besides (the updates of Rutishauser's cyclic Jacobi, as in
    // Numerical Recipes' `jacobi`): five products instead of the two-sided product
    const T apr = S[P][R], aqr = S[Q][R];
    S[P][P] = app - t * apq;
    S[Q][Q] = aqq + t * apq;
    const T npr = c * apr - s * aqr, nqr = s * apr + c * aqr;
    S[P][R] = npr;
    S[R][P] = npr;
    S[Q][R] = nqr;
    S[R][Q] = nqr;
  } else {
    // FP32 with kExact: the two-sided product (the snow clamp's results are pinned to its
    // rounding)
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // columns: S Q
      const T skp = S[k][P], skq = S[k][Q];
      S[k][P] = c * skp - s * skq;
      S[k][Q] = s * skp + c * skq;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {  // rows: Q^T (S Q)
      const T spk = S[P][k], sqk = S[Q][k];
      S[P][k] = c * spk - s * sqk;
      S[Q][k] = s * spk + c * sqk;
    }
  }
  S[P][Q] = T(0);
  S[Q][P] = T(0);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const T vkp = V[k][P], vkq = V[k][Q];
    V[k][P] = c * vkp - s * vkq;
    V[k][Q] = s * vkp + c * vkq;
  }
}

// Swap columns i and j of B and V when |b_i| < |b_j|, negating the new column j so V stays
// a rotation.
template <int I, int J, typename T>
MPM_HD void cond_swap(T B[3][3], T V[3][3], T rho[3]) {
  if (rho[I] < rho[J]) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const T b = B[k][I];
      B[k][I] = B[k][J];
      B[k][J] = -b;
      const T v = V[k][I];
      V[k][I] = V[k][J];
      V[k][J] = -v;
    }
    const T r = rho[I];
    rho[I] = rho[J];
    rho[J] = r;
  }
}

// Givens rotation on rows (P,Q) of B zeroing B[Q][COL]; accumulates U <- U G.
template <int P, int Q, int COL, bool kExact, typename T>
MPM_HD void qr_givens(T B[3][3], T U[3][3]) {
  const T a1 = B[P][COL], a2 = B[Q][COL];
  const T n2 = a1 * a1 + a2 * a2;
  T c = T(1), s = T(0);
  if (n2 > T(1e-38)) {
    if constexpr (kExact && sizeof(T) == 4) {  // c = +-1, s = 0 exactly when a2 is negligible
      const T r = sqrt_(n2);
      c = a1 / r;
      s = a2 / r;
    } else {
      const T inv = rsqrt_(n2);
      c = a1 * inv;
      s = a2 * inv;
    }
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {  // rows: G^T B with G = [[c,-s],[s,c]] in (P,Q)
    const T bp = B[P][k], bq = B[Q][k];
    B[P][k] = c * bp + s * bq;
    B[Q][k] = -s * bp + c * bq;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {  // U <- U G
    const T up = U[k][P], uq = U[k][Q];
    U[k][P] = c * up + s * uq;
    U[k][Q] = -s * up + c * uq;
  }
}

// Columns of V made orthonormal (modified Gram-Schmidt): a rotation given to lower precision
// becomes one to the precision of T.
template <typename T>
MPM_HD void orthonormalize_columns(T V[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
#pragma unroll
    for (int p = 0; p < c; ++p) {
      const T d = V[0][p] * V[0][c] + V[1][p] * V[1][c] + V[2][p] * V[2][c];
#pragma unroll
      for (int k = 0; k < 3; ++k) V[k][c] -= d * V[k][p];
    }
    const T inv = rsqrt_(V[0][c] * V[0][c] + V[1][c] * V[1][c] + V[2][c] * V[2][c]);
#pragma unroll
    for (int k = 0; k < 3; ++k) V[k][c] *= inv;
  }
}

// The SVD of a 3x3 array in precision T (see svd3 below for the conventions).  V0 (may be
// null): a rotation close to the right singular vectors, from which the Jacobi sweeps start
// (S = V0^T A^T A V0 is then nearly diagonal and they stop after one or two).
template <bool kExact, typename T>
MPM_HD void svd3_t(const T A[3][3], T U[3][3], T sig[3], T V[3][3], const T (*V0)[3] = nullptr) {
  T S[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      S[i][j] = A[0][i] * A[0][j] + A[1][i] * A[1][j] + A[2][i] * A[2][j];
      V[i][j] = V0 ? V0[i][j] : ((i == j) ? T(1) : T(0));
    }
  if (V0) {  // S <- V^T S V with V the start made orthonormal in T
    orthonormalize_columns<T>(V);
    T SV[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) SV[i][j] = S[i][0] * V[0][j] + S[i][1] * V[1][j] + S[i][2] * V[2][j];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int j = 0; j < 3; ++j) S[i][j] = V[0][i] * SV[0][j] + V[1][i] * SV[1][j] + V[2][i] * SV[2][j];
  }
#pragma unroll 1
  for (int sweep = 0; sweep < JacobiLimits<T>::kSweeps; ++sweep) {
    // Done once every off-diagonal S_pq is below 2 eps sqrt(S_pp S_qq) (the relative
    // threshold of a two-sided Jacobi SVD such as Eigen's JacobiSVD, on A^T A); tested before
    // the first sweep as well, so an input that is diagonal to within rounding is not rotated
    // at all and keeps its diagonal exactly.
    const T done = JacobiLimits<T>::kDone;
    if (S[0][1] * S[0][1] <= done * fabs_(S[0][0] * S[1][1]) &&
        S[0][2] * S[0][2] <= done * fabs_(S[0][0] * S[2][2]) &&
        S[1][2] * S[1][2] <= done * fabs_(S[1][1] * S[2][2]))
      break;
    jacobi_rotate<0, 1, kExact>(S, V);
    jacobi_rotate<1, 2, kExact>(S, V);
    jacobi_rotate<0, 2, kExact>(S, V);
  }
  T B[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) B[i][j] = A[i][0] * V[0][j] + A[i][1] * V[1][j] + A[i][2] * V[2][j];
  T rho[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) rho[j] = B[0][j] * B[0][j] + B[1][j] * B[1][j] + B[2][j] * B[2][j];
  cond_swap<0, 1>(B, V, rho);
  cond_swap<0, 2>(B, V, rho);
  cond_swap<1, 2>(B, V, rho);
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) U[i][j] = (i == j) ? T(1) : T(0);
  qr_givens<0, 1, 0, kExact>(B, U);
  qr_givens<0, 2, 0, kExact>(B, U);
  qr_givens<1, 2, 1, kExact>(B, U);
  sig[0] = B[0][0];
  sig[1] = B[1][1];
  sig[2] = B[2][2];
}

}  // namespace detail

template <bool kExact = true>
MPM_HD void svd3(const Mat<3> &A, Mat<3> &Uo, float sig[3], Mat<3> &Vo) {
  detail::svd3_t<kExact, float>(A.a, Uo.a, sig, Vo.a);
}

// U diag(s) V^T
template <int D>
MPM_HD Mat<D> usv(const Mat<D> &U, const float s[D], const Mat<D> &V) {
  Mat<D> US;
#pragma unroll
  for (int i = 0; i < D; ++i)
#pragma unroll
    for (int j = 0; j < D; ++j) US.a[i][j] = U.a[i][j] * s[j];
  return mat_mul_t<D>(US, V);
}

// U V^T
template <int D>
MPM_HD Mat<D> uvt(const Mat<D> &U, const Mat<D> &V) {
  return mat_mul_t<D>(U, V);
}

// Rotation part of the reference's nclr_polar: 2D closed form, 3D U V^T of the signed SVD.
MPM_HD Mat<2> polar_R(const Mat<2> &F) { return polar_rotation(F); }
MPM_HD Mat<3> polar_R(const Mat<3> &F) {
  Mat<3> U, V;
  float s[3];
  svd3<false>(F, U, s, V);
  return uvt<3>(U, V);
}

// The same rotation from svd3<true> (correctly rounded rotations): what the fused step takes
// from the snow clamp's own SVD, so a snow particle's stress sees the same R on every path.
MPM_HD Mat<2> polar_R_exact(const Mat<2> &F) { return polar_rotation(F); }
MPM_HD Mat<3> polar_R_exact(const Mat<3> &F) {
  Mat<3> U, V;
  float s[3];
  svd3<true>(F, U, s, V);
  return uvt<3>(U, V);
}

MPM_HD float clampf_(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

}  // namespace mpm
