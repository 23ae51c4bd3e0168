// CPU ORACLE -- test infrastructure only.
//
// A plain C++17 restatement of NuclearMPM's time step MPMSimulation<dim>::advance()
// (src/nclr.h:80-84) and of the math it calls (src/nclr_math.h:13-98).  Only the tests,
// the smoke check and the bench's CPU-baseline leg may use it, and only as the checker:
// the GPU library never links or calls it.
//
// Templated on the dimension (2 or 3) and on the scalar (float = the reference's `real`,
// src/nclr_math.h:11; double = the FP64 oracle).  Every function cites the reference
// line it follows.  The reference depends on Eigen3 (unpinned, not vendored); the parts
// of Eigen it uses are restated here from their published definitions:
//   * JacobiSVD (src/nclr_math.h:57)  -> one-sided (Hestenes) Jacobi SVD, then Eigen's
//     output convention: singular values >= 0 sorted in decreasing order, full U and V;
//   * determinant() (src/nclr.h:246,248,318) -> cofactor expansion along the first row;
//   * LinSpaced (src/nclr_math.h:103-104,114-116) -> Eigen 3.4's linspaced rule;
//   * small matrix products -> plain dot products in index order.
//
// Physics modes:
//   kReference  reproduces the reference exactly, including two defects:
//                 - diag<dim>(v) sets only (0,0) and (1,1) (src/nclr_math.h:13-19), so in
//                   3D the identity used by the F update and the liquid reset is diag(1,1,0);
//                 - nclr_svd flips U.col(2)/values(2) (src/nclr_math.h:63-71); in 2D those
//                   writes are out of bounds (undefined behaviour under NDEBUG) and are
//                   treated as no-ops.
//   kCorrected  diag is the true identity and the 2D sign fix acts on column dim-1.
//
// Two extensions of the reference's model, both off by default:
//   * per-particle Young's modulus and Poisson ratio (Particle::mu0 / lambda0, from
//     lame_of(E, nu), the constructor's formula src/nclr.h:77-78) in place of the
//     simulation's one pair (src/nclr.h:74-78);
//   * the neo-Hookean stress (Stress::kNeoHookean), the model src/nclr.h:339 leaves as a TODO:
//     Kirchhoff stress mu (F F^T - I) + lambda ln(J) I in place of the fixed-corotated
//     2 mu (F - R) F^T + constmat(lambda (J - 1) J).
#pragma once

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <utility>
#include <vector>

namespace oracle {

enum class Model : int { kSnow = 0, kJelly = 1, kLiquid = 2 };  // src/nclr.h:57-61
enum class Physics : int { kReference = 0, kCorrected = 1 };
enum class Stress : int { kCorotated = 0, kNeoHookean = 1 };

// mu_0, lambda_0 of (E, nu) in the scalar type (src/nclr.h:77-78).
template <typename T>
std::pair<T, T> lame_of(T E, T nu) {
  return {E / (T(2) * (T(1) + nu)), E * nu / ((T(1) + nu) * (T(1) - T(2) * nu))};
}

template <typename T, int D>
struct Vec {
  T v[D];
  T &operator[](int i) { return v[i]; }
  const T &operator[](int i) const { return v[i]; }
  static Vec constant(T c) {
    Vec r;
    for (int i = 0; i < D; ++i) r.v[i] = c;
    return r;
  }
};

template <typename T, int D>
struct Mat {
  T m[D][D];
  T &operator()(int i, int j) { return m[i][j]; }
  const T &operator()(int i, int j) const { return m[i][j]; }
  static Mat constant(T c) {  // constmat<dim>, src/nclr_math.h:40-43
    Mat r;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) r.m[i][j] = c;
    return r;
  }
  static Mat identity() {
    Mat r = constant(T(0));
    for (int i = 0; i < D; ++i) r.m[i][i] = T(1);
    return r;
  }
};

template <typename T, int D>
Mat<T, D> mul(const Mat<T, D> &a, const Mat<T, D> &b) {
  Mat<T, D> r;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) {
      T s = a(i, 0) * b(0, j);
      for (int k = 1; k < D; ++k) s = s + a(i, k) * b(k, j);
      r(i, j) = s;
    }
  return r;
}

template <typename T, int D>
Vec<T, D> mul(const Mat<T, D> &a, const Vec<T, D> &x) {
  Vec<T, D> r;
  for (int i = 0; i < D; ++i) {
    T s = a(i, 0) * x[0];
    for (int k = 1; k < D; ++k) s = s + a(i, k) * x[k];
    r[i] = s;
  }
  return r;
}

template <typename T, int D>
Mat<T, D> transpose(const Mat<T, D> &a) {
  Mat<T, D> r;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) r(i, j) = a(j, i);
  return r;
}

// Cofactor expansion along the first row.
template <typename T>
T det(const Mat<T, 2> &a) {
  return a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0);
}
template <typename T>
T det(const Mat<T, 3> &a) {
  return a(0, 0) * (a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1)) -
         a(0, 1) * (a(1, 0) * a(2, 2) - a(1, 2) * a(2, 0)) +
         a(0, 2) * (a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0));
}

// diag<dim>(v), src/nclr_math.h:13-19: only (0,0) and (1,1) are set, so in 3D the result
// is diag(v, v, 0).  kCorrected gives the true v*I.
template <typename T, int D>
Mat<T, D> diag_of(T value, Physics mode) {
  Mat<T, D> r = Mat<T, D>::constant(T(0));
  r(0, 0) = value;
  r(1, 1) = value;
  if (mode == Physics::kCorrected)
    for (int i = 2; i < D; ++i) r(i, i) = value;
  return r;
}

// ---------------------------------------------------------------------------------------
// SVD.  Eigen::JacobiSVD (src/nclr_math.h:57) returns U, V orthogonal and singular values
// >= 0 in decreasing order.  Restated as a one-sided Jacobi iteration on the columns of A
// (Hestenes 1958), run to convergence in the scalar type T.  Columns belonging to a zero
// singular value are completed to an orthonormal basis with det(U) = +1.
// ---------------------------------------------------------------------------------------
template <typename T, int D>
void jacobi_svd(const Mat<T, D> &a, Mat<T, D> &U, Vec<T, D> &sigma, Mat<T, D> &V) {
  Mat<T, D> W = a;  // columns are rotated until mutually orthogonal: W = U * diag(sigma)
  V = Mat<T, D>::identity();
  const T eps = std::numeric_limits<T>::epsilon();
  for (int sweep = 0; sweep < 64; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < D - 1; ++p)
      for (int q = p + 1; q < D; ++q) {
        T alpha = 0, beta = 0, gamma = 0;
        for (int i = 0; i < D; ++i) {
          alpha += W(i, p) * W(i, p);
          beta += W(i, q) * W(i, q);
          gamma += W(i, p) * W(i, q);
        }
        if (gamma == T(0) || std::fabs(gamma) <= eps * std::sqrt(alpha * beta)) continue;
        rotated = true;
        const T zeta = (beta - alpha) / (T(2) * gamma);
        const T t = (zeta >= T(0) ? T(1) : T(-1)) / (std::fabs(zeta) + std::sqrt(T(1) + zeta * zeta));
        const T c = T(1) / std::sqrt(T(1) + t * t);
        const T s = c * t;
        for (int i = 0; i < D; ++i) {
          const T wp = W(i, p), wq = W(i, q);
          W(i, p) = c * wp - s * wq;
          W(i, q) = s * wp + c * wq;
          const T vp = V(i, p), vq = V(i, q);
          V(i, p) = c * vp - s * vq;
          V(i, q) = s * vp + c * vq;
        }
      }
    if (!rotated) break;
  }
  // singular values = column norms; sort decreasing (selection sort keeps it explicit)
  int order[D];
  T norms[D];
  for (int j = 0; j < D; ++j) {
    T s = 0;
    for (int i = 0; i < D; ++i) s += W(i, j) * W(i, j);
    norms[j] = std::sqrt(s);
    order[j] = j;
  }
  for (int i = 0; i < D; ++i)
    for (int j = i + 1; j < D; ++j)
      if (norms[order[j]] > norms[order[i]]) std::swap(order[i], order[j]);
  Mat<T, D> Vs, Us = Mat<T, D>::constant(T(0));
  bool have[D];
  const T tiny = norms[order[0]] * eps * T(D) + std::numeric_limits<T>::min();
  for (int j = 0; j < D; ++j) {
    const int src = order[j];
    sigma[j] = norms[src];
    for (int i = 0; i < D; ++i) Vs(i, j) = V(i, src);
    have[j] = false;
    if (j == D - 1 && j >= 1 && have[0] && (D == 2 || have[1])) {
      // The last left vector is fixed up to sign by the others (exactly orthogonal):
      // the cross product in 3D, the perpendicular in 2D; the sign follows W's column so
      // that sigma stays >= 0.
      T c[D];
      if constexpr (D == 3) {
        c[0] = Us(1, 0) * Us(2, 1) - Us(2, 0) * Us(1, 1);
        c[1] = Us(2, 0) * Us(0, 1) - Us(0, 0) * Us(2, 1);
        c[2] = Us(0, 0) * Us(1, 1) - Us(1, 0) * Us(0, 1);
      } else {
        c[0] = -Us(1, 0);
        c[1] = Us(0, 0);
      }
      T d = 0;
      for (int i = 0; i < D; ++i) d += c[i] * W(i, src);
      const T sgn = d < T(0) ? T(-1) : T(1);
      for (int i = 0; i < D; ++i) Us(i, j) = sgn * c[i];
      have[j] = true;
      continue;
    }
    if (norms[src] > tiny) {
      T u[D];
      for (int i = 0; i < D; ++i) u[i] = W(i, src) / norms[src];
      for (int k = 0; k < j; ++k) {  // re-orthogonalise against the earlier columns
        if (!have[k]) continue;
        T dd = 0;
        for (int i = 0; i < D; ++i) dd += Us(i, k) * u[i];
        for (int i = 0; i < D; ++i) u[i] -= dd * Us(i, k);
      }
      T n = 0;
      for (int i = 0; i < D; ++i) n += u[i] * u[i];
      n = std::sqrt(n);
      for (int i = 0; i < D; ++i) Us(i, j) = u[i] / n;
      have[j] = true;
    }
  }
  // Complete U where a singular value vanished: Gram-Schmidt on the canonical basis.
  for (int j = 0; j < D; ++j) {
    if (have[j]) continue;
    for (int e = 0; e < D && !have[j]; ++e) {
      T cand[D];
      for (int i = 0; i < D; ++i) cand[i] = (i == e) ? T(1) : T(0);
      for (int k = 0; k < D; ++k) {
        if (!have[k]) continue;
        T d = 0;
        for (int i = 0; i < D; ++i) d += Us(i, k) * cand[i];
        for (int i = 0; i < D; ++i) cand[i] -= d * Us(i, k);
      }
      T n = 0;
      for (int i = 0; i < D; ++i) n += cand[i] * cand[i];
      n = std::sqrt(n);
      if (n > T(0.5)) {
        for (int i = 0; i < D; ++i) Us(i, j) = cand[i] / n;
        have[j] = true;
      }
    }
  }
  U = Us;
  V = Vs;
}

// nclr_svd, src/nclr_math.h:50-74: JacobiSVD then the sign fix on column 2.
// In 2D the reference's writes to column/entry 2 are out of bounds; kReference treats them
// as no-ops (U, V may be reflections, sigma >= 0), kCorrected applies them to column 1.
// Returns how many sign flips were requested (for counting inverted elements).
template <typename T, int D>
int nclr_svd(const Mat<T, D> &a, Mat<T, D> &U, Mat<T, D> &sig, Mat<T, D> &V, Physics mode) {
  Vec<T, D> values;
  jacobi_svd<T, D>(a, U, values, V);
  int flips = 0;
  const int c = (D == 3) ? 2 : ((mode == Physics::kCorrected) ? D - 1 : -1);
  if (det(U) < T(0)) {  // src/nclr_math.h:63-66
    ++flips;
    if (c >= 0) {
      for (int i = 0; i < D; ++i) U(i, c) = -U(i, c);
      values[c] = -values[c];
    }
  }
  if (det(V) < T(0)) {  // src/nclr_math.h:68-71
    ++flips;
    if (c >= 0) {
      for (int i = 0; i < D; ++i) V(i, c) = -V(i, c);
      values[c] = -values[c];
    }
  }
  sig = Mat<T, D>::identity();  // src/nclr_math.h:54,72-73
  for (int i = 0; i < D; ++i) sig(i, i) = values[i];
  return flips;
}

// nclr_polar, src/nclr_math.h:76-98.  2D: closed-form rotation; 3D: R = U V^T.
template <typename T, int D>
Mat<T, D> nclr_polar_R(const Mat<T, D> &m, Physics mode) {
  Mat<T, D> R = Mat<T, D>::identity();
  if constexpr (D == 2) {
    const T x = m(0, 0) + m(1, 1);
    const T y = m(1, 0) - m(0, 1);
    const T scale = T(1) / std::sqrt(x * x + y * y);
    const T c = x * scale, s = y * scale;
    R(0, 0) = c;
    R(0, 1) = -s;
    R(1, 0) = s;
    R(1, 1) = c;
  } else {
    Mat<T, D> U, sig, V;
    nclr_svd<T, D>(m, U, sig, V, mode);
    R = mul(U, transpose(V));
  }
  return R;
}

// Particle<dim>, src/nclr.h:20-48.
template <typename T, int D>
struct Particle {
  Vec<T, D> x, v;
  Mat<T, D> F, C;
  T Jp, mass, volume;
  int material = -1;  // per-particle material (an extension); -1: the simulation's model
  T mu0 = T(-1), lambda0 = T(0);  // per-particle base moduli (an extension); mu0 < 0: the
                                  // simulation's mu_0, lambda_0
};

// Cell<dim>, src/nclr.h:50-55.
template <typename T, int D>
struct Cell {
  Vec<T, D> velocity;
  T mass;
};

struct Counters {  // atomic: the multi-threaded baseline (nclr_oracle_mt.h) shares them
  std::atomic<int64_t> inverted_svd{0};  // G2P SVDs of an inverted element (det F_hat < 0)
  std::atomic<int64_t> out_of_range{0};  // node indices outside the grid (vector::at throws)
};

// MPMSimulation<dim>, src/nclr.h:63-384.
template <typename T, int D>
class Simulation {
 public:
  // src/nclr.h:74-78: dx = 1.0/res (double, narrowed), inv_dx = 1/dx, mu_0 and lambda_0
  // evaluated in the scalar type.
  Simulation(std::vector<Particle<T, D>> particles, Model model, int res, T dt, T E, T nu,
             T gravity, Physics mode)
      : mu_0(E / (T(2) * (T(1) + nu))),
        lambda_0(E * nu / ((T(1) + nu) * (T(1) - T(2) * nu))),
        model_(model), mode_(mode), res_(res), dt_(dt), dx_(T(1.0 / res)), inv_dx_(T(1) / dx_),
        gravity_(gravity), particles_(std::move(particles)) {}

  const T mu_0, lambda_0;

  // src/nclr.h:80-84
  void advance() {
    p2g();
    grid_op();
    g2p();
  }
  std::vector<Particle<T, D>> &particles() { return particles_; }
  const std::vector<Cell<T, D>> &grid() const { return cells_; }
  Counters counters;

  // Internals are public: the adjoint restatement (nclr_adjoint.h) steps the phases itself.
  const Model model_;
  const Physics mode_;
  Stress stress_ = Stress::kCorotated;  // the reference's model unless set
  const int res_;
  const T dt_, dx_, inv_dx_, gravity_;
  std::vector<Cell<T, D>> cells_;
  std::vector<Particle<T, D>> particles_;

  int64_t num_nodes() const {
    int64_t n = 1;
    for (int d = 0; d < D; ++d) n *= (res_ + 1);
    return n;
  }

  // vector::at (src/nclr.h:163-164,199): an index outside [0, N^dim) throws.
  Cell<T, D> &at(int64_t index) {
    if (index < 0 || index >= (int64_t)cells_.size()) {
      ++counters.out_of_range;
      throw std::out_of_range("grid node index out of range");
    }
    return cells_[index];
  }

  // base = cast<int>(x*inv_dx - 0.5) truncates toward zero; fx = x*inv_dx - base;
  // quadratic B-spline weights (src/nclr.h:115-127, 172-183).
  void kernel(const Vec<T, D> &x, int base[D], Vec<T, D> &fx, Vec<T, D> w[3]) const {
    for (int d = 0; d < D; ++d) {
      base[d] = (int)(x[d] * inv_dx_ - T(0.5));
      fx[d] = x[d] * inv_dx_ - (T)base[d];
      const T a = T(1.5) - fx[d], b = fx[d] - T(1.0), c = fx[d] - T(0.5);
      w[0][d] = T(0.5) * (a * a);
      w[1][d] = T(0.75) - b * b;
      w[2][d] = T(0.5) * (c * c);
    }
  }

  int64_t flat(const int base[D], const int o[D]) const {
    const int64_t N = res_ + 1;
    if constexpr (D == 3)
      return (int64_t)(base[0] + o[0]) * N * N + (int64_t)(base[1] + o[1]) * N + (base[2] + o[2]);
    else
      return (int64_t)(base[0] + o[0]) * N + (base[1] + o[1]);
  }

  // The material of particle p: the simulation's model (src/nclr.h:90) unless the particle
  // carries its own (the mixed-material extension).
  Model model_of(const Particle<T, D> &p) const {
    return p.material < 0 ? model_ : (Model)p.material;
  }

  // hardening, src/nclr.h:351-372.  Snow: e = exp(10*(1.0 - Jp)) in double, narrowed to
  // the scalar (constant_hardening takes `real`); jelly 0.3; liquid 1.0.  The base moduli
  // are the particle's own when it carries them.
  std::pair<T, T> hardening(const Particle<T, D> &p) const {
    T e;
    switch (model_of(p)) {
      case Model::kSnow: e = (T)std::exp((double)T(10.0) * (1.0 - (double)p.Jp)); break;
      case Model::kJelly: e = T(0.3); break;
      case Model::kLiquid: e = T(1.0); break;
      default: e = T(0); break;
    }
    return p.mu0 < T(0) ? std::pair<T, T>{mu_0 * e, lambda_0 * e}
                        : std::pair<T, T>{p.mu0 * e, p.lambda0 * e};
  }

  // first_piola_kirchoff_stress, src/nclr.h:313-337 (and the neo-Hookean extension).
  Mat<T, D> affine(const Particle<T, D> &p) const {
    const auto [mu, lambda] = hardening(p);
    const T J = det(p.F);
    const T Dinv = T(4) * inv_dx_ * inv_dx_;
    const Mat<T, D> FT = transpose(p.F);
    Mat<T, D> PF;
    if (stress_ == Stress::kNeoHookean) {  // mu (F F^T - I) + lambda ln(J) I
      PF = mul(p.F, FT);
      const T lam_term = lambda * std::log(J);
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) PF(i, j) = mu * (PF(i, j) - (i == j ? T(1) : T(0)));
      for (int i = 0; i < D; ++i) PF(i, i) = PF(i, i) + lam_term;
    } else {
      const Mat<T, D> r = nclr_polar_R<T, D>(p.F, mode_);
      Mat<T, D> FmR;
      const T two_mu = T(2) * mu;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) FmR(i, j) = two_mu * (p.F(i, j) - r(i, j));
      PF = mul(FmR, FT);
      const T lam_term = lambda * (J - T(1)) * J;  // constmat: every entry, src/nclr.h:328
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) PF(i, j) = PF(i, j) + lam_term;
    }
    const T s = -(dt_ * p.volume);
    Mat<T, D> out;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) out(i, j) = s * (Dinv * PF(i, j)) + p.mass * p.C(i, j);
    return out;
  }

  // p2g + compute_fused_momentum, src/nclr.h:104-165.
  void p2g() {
    cells_.assign((size_t)num_nodes(), Cell<T, D>{Vec<T, D>::constant(T(0)), T(0)});
    for (auto &p : particles_) p2g_particle(p);
  }

  // One particle's scatter of p2g (the loop body of src/nclr.h:111-165).
  void p2g_particle(const Particle<T, D> &p) {
    int base[D];
    Vec<T, D> fx, w[3];
    kernel(p.x, base, fx, w);
    const Mat<T, D> A = affine(p);
    Vec<T, D> mv;
    for (int d = 0; d < D; ++d) mv[d] = p.v[d] * p.mass;
    int o[3] = {0, 0, 0};
    for (o[0] = 0; o[0] < 3; ++o[0])
      for (o[1] = 0; o[1] < 3; ++o[1])
        for (o[2] = 0; o[2] < (D == 3 ? 3 : 1); ++o[2]) {
          Vec<T, D> dpos;
          for (int d = 0; d < D; ++d) dpos[d] = ((T)o[d] - fx[d]) * dx_;
          T weight = w[o[0]][0] * w[o[1]][1];
          if constexpr (D == 3) weight = weight * w[o[2]][2];
          Cell<T, D> &cell = at(flat(base, o));
          const Vec<T, D> Ad = mul(A, dpos);
          for (int d = 0; d < D; ++d) cell.velocity[d] += weight * (mv[d] + Ad[d]);
          cell.mass += weight * p.mass;
        }
  }

  // grid_op + grid_normalization + sticky_boundary, src/nclr.h:263-310.
  void grid_op() {
    const int64_t total = num_nodes();
    for (int64_t index = 0; index < total; ++index) grid_node(index);
  }

  // One node of grid_op (the loop body of src/nclr.h:264-309).
  void grid_node(int64_t index) {
    // allowed_velocity = dx*0.9/dt evaluated in double, stored in the scalar (src/nclr.h:285)
    const T allowed = (T)((double)dx_ * 0.9 / (double)dt_);
    const int N = res_ + 1;
    int idx[D];
    int64_t rem = index;
    for (int d = D - 1; d >= 0; --d) {
      idx[d] = (int)(rem % N);
      rem /= N;
    }
    Cell<T, D> &g = cells_[index];
    if (g.mass > T(0)) {
      for (int d = 0; d < D; ++d) g.velocity[d] = g.velocity[d] / g.mass;
      g.velocity[1] += dt_ * gravity_;
      for (int d = 0; d < D; ++d) g.velocity[d] = std::clamp(g.velocity[d], -allowed, allowed);
    }
    for (int d = 0; d < D; ++d) {
      if ((idx[d] < 3 && g.velocity[d] < T(0)) || (idx[d] >= N - 3 && g.velocity[d] > T(0))) {
        g.velocity = Vec<T, D>::constant(T(0));
        g.mass = T(0);
      }
    }
  }

  // g2p, src/nclr.h:167-261.
  void g2p() {
    for (auto &p : particles_) g2p_particle(p);
  }

  // One particle of g2p (the loop body of src/nclr.h:168-260).
  void g2p_particle(Particle<T, D> &p) {
    const Mat<T, D> I = diag_of<T, D>(T(1), mode_);
    const T cscale = T(4) * inv_dx_;
    int base[D];
    Vec<T, D> fx, w[3];
    kernel(p.x, base, fx, w);
    p.C = Mat<T, D>::constant(T(0));
    p.v = Vec<T, D>::constant(T(0));
    int o[3] = {0, 0, 0};
    for (o[0] = 0; o[0] < 3; ++o[0])
      for (o[1] = 0; o[1] < 3; ++o[1])
        for (o[2] = 0; o[2] < (D == 3 ? 3 : 1); ++o[2]) {
          Vec<T, D> dpos;
          for (int d = 0; d < D; ++d) dpos[d] = (T)o[d] - fx[d];
          const Vec<T, D> gv = at(flat(base, o)).velocity;
          T weight = w[o[0]][0] * w[o[1]][1];
          if constexpr (D == 3) weight = weight * w[o[2]][2];
          Vec<T, D> wgv;
          for (int d = 0; d < D; ++d) {
            wgv[d] = weight * gv[d];
            p.v[d] += wgv[d];
          }
          for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) p.C(i, j) += (cscale * wgv[i]) * dpos[j];
        }
    for (int d = 0; d < D; ++d) p.x[d] += dt_ * p.v[d];
    Mat<T, D> M;
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) M(i, j) = I(i, j) + dt_ * p.C(i, j);
    Mat<T, D> Fh = mul(M, p.F);
    const Model model = model_of(p);
    if (model == Model::kJelly) {
      p.F = Fh;
      return;
    }
    Mat<T, D> U, sig, V;
    nclr_svd<T, D>(Fh, U, sig, V, mode_);
    if (det(Fh) < T(0)) ++counters.inverted_svd;  // the 2D sign-fix ambiguity only bites here
    if (model == Model::kSnow) {
      for (int d = 0; d < D; ++d)
        sig(d, d) = std::clamp(sig(d, d), T(1.0 - 2.5e-2), T(1.0 + 4.5e-3));
      const T old_J = det(Fh);
      Fh = mul(mul(U, sig), transpose(V));
      p.Jp = std::clamp(p.Jp * old_J / det(Fh), T(0.6), T(20.0));
      p.F = Fh;
    } else {  // kLiquid: J accumulated in double, src/nclr.h:253-257
      double J = 1.0;
      for (int d = 0; d < D; ++d) J *= (double)sig(d, d);
      p.F = diag_of<T, D>(T(1.0), mode_);
      p.F(0, 0) = (T)J;
    }
  }
};

// cube<dim>(res, min, max), src/nclr_math.h:100-129, with Eigen 3.4's LinSpaced rule:
// step = (high-low)/(n-1); entries low + i*step, the last one pinned to high (or, when
// |high| < |low|, high - (n-1-i)*step with the first pinned to low).
template <typename T>
std::vector<T> linspaced(int n, T low, T high) {
  std::vector<T> r((size_t)std::max(n, 0));
  if (n == 1) {
    r[0] = high;
    return r;
  }
  const T step = (high - low) / T(n - 1);
  const bool flip = std::fabs(high) < std::fabs(low);
  for (int i = 0; i < n; ++i) {
    if (flip)
      r[i] = (i == 0) ? low : T(high - T(n - 1 - i) * step);
    else
      r[i] = (i == n - 1) ? high : T(low + T(i) * step);
  }
  return r;
}

}  // namespace oracle
