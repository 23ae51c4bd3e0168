/*
 * nclr.h -- drop-in replacement for NuclearMPM's header-only solver API (src/nclr.h and the
 * parts of src/nclr_math.h it uses) running the time step on a GB300 through libnclr_gpu.so
 * (include/nclr_gpu.h).
 *
 * Same names, signatures, defaults and error behaviour as the reference:
 *   nclr::real, Vector<T, dim>, Matrix<T, dim>                   src/nclr_math.h:5-11
 *   diag<dim>, constmat<dim>, constvec<dim>                      src/nclr_math.h:13-48
 *   nc_rand_int, nc_rand, randvec<dim>                           src/nclr_math.h:22-39
 *   cube<dim>(res, min, max)                                     src/nclr_math.h:100-129
 *   Particle<dim>(x, c, v = 0, mass = 1, volume = 1)             src/nclr.h:20-48
 *   Cell<dim>                                                    src/nclr.h:50-55
 *   MaterialModel::{kSnow, kJelly, kLiquid}                      src/nclr.h:57-61
 *   MPMSimulation<dim>(particles, model, res = 64, dt = 1e-4, E = 1e4, nu = 0.2,
 *                      gravity = -100)                           src/nclr.h:74-78
 *     advance(), particles(), grid(), mu_0, lambda_0, kBoundary, k*Hardening
 *                                                                src/nclr.h:66-87
 * advance() throws std::out_of_range when a particle's stencil leaves the grid (the
 * reference's vector::at, src/nclr.h:163-164,199) and std::runtime_error on a CUDA failure.
 *
 * particles() and grid() return references to host copies that are refreshed lazily after each
 * advance() (they stay valid until the next advance(), as the reference's do).
 *
 * Vector/Matrix are Eigen's fixed-size types when <Eigen/Dense> is available (as in the
 * reference; define NCLR_NO_EIGEN to opt out), otherwise the small built-in types below,
 * which offer the subset of Eigen's interface the reference API and its examples use.
 *
 * Link with libnclr_gpu.so (nuclearmpm_gb300/_build).
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "nclr_gpu.h"

#if !defined(NCLR_NO_EIGEN) && defined(__has_include)
#if __has_include(<Eigen/Dense>)
#define NCLR_HAVE_EIGEN 1
#endif
#endif

#ifdef NCLR_HAVE_EIGEN
#include <Eigen/Dense>
#endif

namespace nclr {

using real = float;  // src/nclr_math.h:11

#ifdef NCLR_HAVE_EIGEN
template <typename T, int dim>
using Vector = Eigen::Matrix<T, dim, 1>;
template <typename T, int dim>
using Matrix = Eigen::Matrix<T, dim, dim>;
#else
// --- built-in fixed-size vector and matrix (an Eigen-like subset) -------------------------
template <typename T, int dim>
class Vector {
 public:
  Vector() {
    for (auto &e : a_) e = T(0);
  }
  template <typename A, typename B, int D = dim, typename = std::enable_if_t<D == 2>>
  Vector(A x, B y) : a_{T(x), T(y)} {}
  template <typename A, typename B, typename C, int D = dim, typename = std::enable_if_t<D == 3>>
  Vector(A x, B y, C z) : a_{T(x), T(y), T(z)} {}
  static Vector Constant(T c) {
    Vector v;
    for (auto &e : v.a_) e = c;
    return v;
  }
  static Vector Zero() { return Constant(T(0)); }
  static Vector Ones() { return Constant(T(1)); }
  T &operator()(int i) { return a_[i]; }
  const T &operator()(int i) const { return a_[i]; }
  T &operator[](int i) { return a_[i]; }
  const T &operator[](int i) const { return a_[i]; }
  T &x() { return a_[0]; }
  T &y() { return a_[1]; }
  T &z() { return a_[dim - 1]; }
  T x() const { return a_[0]; }
  T y() const { return a_[1]; }
  T z() const { return a_[dim - 1]; }
  static constexpr int rows() { return dim; }
  static constexpr int size() { return dim; }
  T *data() { return a_; }
  const T *data() const { return a_; }
  T dot(const Vector &o) const {
    T s = T(0);
    for (int i = 0; i < dim; ++i) s += a_[i] * o.a_[i];
    return s;
  }
  T squaredNorm() const { return dot(*this); }
  T norm() const { return std::sqrt(squaredNorm()); }
  Vector cwiseProduct(const Vector &o) const {
    Vector r;
    for (int i = 0; i < dim; ++i) r.a_[i] = a_[i] * o.a_[i];
    return r;
  }
  Vector &operator+=(const Vector &o) {
    for (int i = 0; i < dim; ++i) a_[i] += o.a_[i];
    return *this;
  }
  Vector &operator-=(const Vector &o) {
    for (int i = 0; i < dim; ++i) a_[i] -= o.a_[i];
    return *this;
  }
  Vector &operator*=(T s) {
    for (auto &e : a_) e *= s;
    return *this;
  }
  Vector &operator/=(T s) {
    for (auto &e : a_) e /= s;
    return *this;
  }
  friend Vector operator+(Vector a, const Vector &b) { return a += b; }
  friend Vector operator-(Vector a, const Vector &b) { return a -= b; }
  friend Vector operator-(Vector a) { return a *= T(-1); }
  friend Vector operator*(Vector a, T s) { return a *= s; }
  friend Vector operator*(T s, Vector a) { return a *= s; }
  friend Vector operator/(Vector a, T s) { return a /= s; }
  friend bool operator==(const Vector &a, const Vector &b) {
    for (int i = 0; i < dim; ++i)
      if (a.a_[i] != b.a_[i]) return false;
    return true;
  }

 private:
  T a_[dim];
};

template <typename T, int dim>
class Matrix {
 public:
  Matrix() {
    for (auto &e : a_) e = T(0);
  }
  static Matrix Constant(T c) {
    Matrix m;
    for (auto &e : m.a_) e = c;
    return m;
  }
  static Matrix Zero() { return Constant(T(0)); }
  static Matrix Identity() {
    Matrix m;
    for (int i = 0; i < dim; ++i) m(i, i) = T(1);
    return m;
  }
  T &operator()(int i, int j) { return a_[i * dim + j]; }
  const T &operator()(int i, int j) const { return a_[i * dim + j]; }
  static constexpr int rows() { return dim; }
  static constexpr int cols() { return dim; }
  Matrix transpose() const {
    Matrix r;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) r(i, j) = (*this)(j, i);
    return r;
  }
  T determinant() const {
    const Matrix &m = *this;
    if constexpr (dim == 2) {
      return m(0, 0) * m(1, 1) - m(0, 1) * m(1, 0);
    } else {
      return m(0, 0) * (m(1, 1) * m(2, 2) - m(1, 2) * m(2, 1)) -
             m(0, 1) * (m(1, 0) * m(2, 2) - m(1, 2) * m(2, 0)) +
             m(0, 2) * (m(1, 0) * m(2, 1) - m(1, 1) * m(2, 0));
    }
  }
  Matrix &operator+=(const Matrix &o) {
    for (int i = 0; i < dim * dim; ++i) a_[i] += o.a_[i];
    return *this;
  }
  Matrix &operator-=(const Matrix &o) {
    for (int i = 0; i < dim * dim; ++i) a_[i] -= o.a_[i];
    return *this;
  }
  Matrix &operator*=(T s) {
    for (auto &e : a_) e *= s;
    return *this;
  }
  friend Matrix operator+(Matrix a, const Matrix &b) { return a += b; }
  friend Matrix operator-(Matrix a, const Matrix &b) { return a -= b; }
  friend Matrix operator*(Matrix a, T s) { return a *= s; }
  friend Matrix operator*(T s, Matrix a) { return a *= s; }
  friend Matrix operator*(const Matrix &a, const Matrix &b) {
    Matrix r;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) {
        T s = T(0);
        for (int k = 0; k < dim; ++k) s += a(i, k) * b(k, j);
        r(i, j) = s;
      }
    return r;
  }
  friend Vector<T, dim> operator*(const Matrix &a, const Vector<T, dim> &x) {
    Vector<T, dim> r;
    for (int i = 0; i < dim; ++i) {
      T s = T(0);
      for (int k = 0; k < dim; ++k) s += a(i, k) * x(k);
      r(i) = s;
    }
    return r;
  }

 private:
  T a_[dim * dim];
};
#endif

// --- helpers of src/nclr_math.h ------------------------------------------------------------

// diag<dim>(v): the reference sets only (0,0) and (1,1) (src/nclr_math.h:13-19), so diag<3>
// is diag(v, v, 0); kept as is, since the default physics reproduces the reference.
template <int dim>
inline Matrix<real, dim> diag(const float value) {
  Matrix<real, dim> m = Matrix<real, dim>::Zero();
  m(0, 0) = value;
  m(1, 1) = value;
  return m;
}

template <int dim>
inline Matrix<real, dim> constmat(const float value) {
  return Matrix<real, dim>::Constant(value);
}

template <int dim>
inline Vector<real, dim> constvec(const float value) {
  return Vector<real, dim>::Constant(value);
}

// The reference's global xorshift128 stream (src/nclr_math.h:22-33).
inline uint32_t nc_rand_int() {
  static uint32_t x = 123456789u, y = 362436069u, z = 521288629u, w = 88675123u;
  const uint32_t t = x ^ (x << 11);
  x = y;
  y = z;
  z = w;
  return (w = (w ^ (w >> 19)) ^ (t ^ (t >> 8)));
}

inline float nc_rand() { return nc_rand_int() * (1.0f / 4294967296.0f); }

template <int dim>
inline Vector<real, dim> randvec() {
  Vector<real, dim> r;
  for (int i = 0; i < dim; ++i) r(i) = nc_rand();
  return r;
}

namespace detail {
// LinSpaced(n, low, high) in float (Eigen 3.4's rule): step (high-low)/(n-1); the end that
// has the larger magnitude is computed from the other end, the last entry pinned.
inline std::vector<real> linspaced(int n, real low, real high) {
  std::vector<real> r((size_t)(n > 0 ? n : 0));
  if (n == 1) {
    r[0] = high;
    return r;
  }
  if (n <= 0) return r;
  const real step = (high - low) / real(n - 1);
  const bool flip = std::fabs(high) < std::fabs(low);
  for (int i = 0; i < n; ++i) {
    if (flip)
      r[(size_t)i] = (i == 0) ? low : real(high - real(n - 1 - i) * step);
    else
      r[(size_t)i] = (i == n - 1) ? high : real(low + real(i) * step);
  }
  return r;
}
}  // namespace detail

// cube<dim>(res, min, max): a res^dim lattice over [min, max]^dim, x outermost
// (src/nclr_math.h:100-129).
template <int dim>
inline std::vector<Vector<real, dim>> cube(int res, real min, real max) {
  const auto ax = detail::linspaced(res, min, max);
  std::vector<Vector<real, dim>> pts;
  if constexpr (dim == 2) {
    for (real a : ax)
      for (real b : ax) pts.emplace_back(a, b);
  } else {
    for (real a : ax)
      for (real b : ax)
        for (real c : ax) pts.emplace_back(a, b, c);
  }
  return pts;
}

// --- the solver types of src/nclr.h --------------------------------------------------------

template <int dim>
struct Particle {
  Vector<real, dim> x;  // position
  Vector<real, dim> v;  // velocity
  Matrix<real, dim> F;  // deformation gradient
  Matrix<real, dim> C;  // APIC affine momentum
  real Jp;              // plastic volume ratio
  real mass;
  real volume;
  int c;  // colour

  Particle(Vector<real, dim> x, int c, Vector<real, dim> v = constvec<dim>(0), real mass = 1.0,
           real volume = 1.0)
      : x(x), v(v), F(diag<dim>(1)), C(constmat<dim>(0)), Jp(1.0), mass(mass), volume(volume),
        c(c) {}
};

template <int dim>
struct Cell {
  Vector<real, dim> velocity;
  real mass;
  Cell() : velocity(constvec<dim>(0)), mass(0.0) {}
};

enum class MaterialModel {
  kSnow = 0,
  kJelly,
  kLiquid,
};

template <int dim>
class MPMSimulation {
  static_assert(dim == 2 || dim == 3, "MPMSimulation is 2D or 3D");

 public:
  constexpr static int kBoundary = 3;
  constexpr static real kSnowHardening = 10.0;
  constexpr static real kJellyHardening = 0.3;
  constexpr static real kLiquidHardening = 1.0;

  const real mu_0;
  const real lambda_0;

  MPMSimulation(std::vector<Particle<dim>> particles, const MaterialModel model, int res = 64,
                real dt = 1e-4, real E = 1e4, real nu = 0.2, real gravity = -100)
      : MPMSimulation(std::move(particles), model, res, dt, E, nu, gravity, nullptr) {}

  // An extension: the same with the options of include/nclr_gpu.h (physics mode, stress
  // model, sort interval, ...); opt == nullptr gives the defaults.
  MPMSimulation(std::vector<Particle<dim>> particles, const MaterialModel model, int res,
                real dt, real E, real nu, real gravity, const nclr_options *opt)
      : mu_0(E / (2 * (1 + nu))), lambda_0(E * nu / ((1 + nu) * (1 - 2 * nu))),
        particles_(std::move(particles)), res_(res) {
    const size_t n = particles_.size();
    std::vector<float> x(n * dim), v(n * dim), F(n * dim * dim), C(n * dim * dim), Jp(n), m(n),
        vol(n);
    for (size_t p = 0; p < n; ++p) {
      const Particle<dim> &q = particles_[p];
      for (int d = 0; d < dim; ++d) {
        x[p * dim + d] = q.x(d);
        v[p * dim + d] = q.v(d);
      }
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) {
          F[(p * dim + i) * dim + j] = q.F(i, j);
          C[(p * dim + i) * dim + j] = q.C(i, j);
        }
      Jp[p] = q.Jp;
      m[p] = q.mass;
      vol[p] = q.volume;
    }
    nclr_sim *h = nullptr;
    const nclr_status st =
        nclr_create(&h, dim, (int64_t)n, x.data(), v.data(), F.data(), C.data(), Jp.data(),
                    m.data(), vol.data(), nullptr, (int)model, res, dt, E, nu, gravity, opt);
    if (st != NCLR_OK) throw std::runtime_error(std::string("nclr_create: ") + nclr_last_error(nullptr));
    sim_.reset(h);
  }

  MPMSimulation(const MPMSimulation &) = delete;
  MPMSimulation &operator=(const MPMSimulation &) = delete;

  // One time step (src/nclr.h:80-84).
  auto advance() -> void { advance(1); }

  // `steps` time steps in one call (one synchronisation instead of `steps`).
  auto advance(int64_t steps) -> void {
    const nclr_status st = nclr_advance(sim_.get(), steps);
    particles_fresh_ = false;
    grid_fresh_ = false;
    stepped_ = true;
    if (st == NCLR_ERR_OUT_OF_RANGE) throw std::out_of_range(nclr_last_error(sim_.get()));
    if (st != NCLR_OK) throw std::runtime_error(nclr_last_error(sim_.get()));
  }

  auto particles() const -> const std::vector<Particle<dim>> & {
    if (!particles_fresh_) download_particles();
    return particles_;
  }

  auto grid() const -> const std::vector<Cell<dim>> & {
    if (!grid_fresh_) download_grid();
    return cells_;
  }

  // An extension: every particle's own Young's modulus and Poisson ratio (one value each per
  // particle, in the order of the constructor's particles), from the next advance() on; empty
  // vectors return to the simulation's E and nu.
  auto set_moduli(const std::vector<real> &E, const std::vector<real> &nu) -> void {
    if (E.size() != nu.size() || (!E.empty() && E.size() != particles_.size()))
      throw std::invalid_argument("set_moduli takes one E and one nu per particle");
    const nclr_status st = E.empty() ? nclr_set_moduli(sim_.get(), nullptr, nullptr)
                                     : nclr_set_moduli(sim_.get(), E.data(), nu.data());
    if (st != NCLR_OK) throw std::runtime_error(nclr_last_error(sim_.get()));
  }

  // The underlying C handle, for the extensions of include/nclr_gpu.h.
  nclr_sim *handle() const { return sim_.get(); }

 private:
  struct Deleter {
    void operator()(nclr_sim *s) const { nclr_destroy(s); }
  };
  std::unique_ptr<nclr_sim, Deleter> sim_;
  mutable std::vector<Particle<dim>> particles_;
  mutable std::vector<Cell<dim>> cells_;
  mutable bool particles_fresh_ = true;  // the constructor's particles are the state
  mutable bool grid_fresh_ = true;       // empty before the first advance (src/nclr.h:101)
  bool stepped_ = false;
  const int res_;

  void download_particles() const {
    const size_t n = particles_.size();
    std::vector<float> x(n * dim), v(n * dim), F(n * dim * dim), C(n * dim * dim), Jp(n);
    const nclr_status st = nclr_get_particles(sim_.get(), x.data(), v.data(), F.data(), C.data(), Jp.data());
    if (st != NCLR_OK) throw std::runtime_error(nclr_last_error(sim_.get()));
    for (size_t p = 0; p < n; ++p) {
      Particle<dim> &q = particles_[p];
      for (int d = 0; d < dim; ++d) {
        q.x(d) = x[p * dim + d];
        q.v(d) = v[p * dim + d];
      }
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) {
          q.F(i, j) = F[(p * dim + i) * dim + j];
          q.C(i, j) = C[(p * dim + i) * dim + j];
        }
      q.Jp = Jp[p];
    }
    particles_fresh_ = true;
  }

  void download_grid() const {
    if (!stepped_) {
      cells_.clear();
      grid_fresh_ = true;
      return;
    }
    const size_t nodes = (size_t)nclr_num_nodes(sim_.get());
    std::vector<float> vel(nodes * dim), mass(nodes);
    const nclr_status st = nclr_get_grid(sim_.get(), vel.data(), mass.data());
    if (st != NCLR_OK) throw std::runtime_error(nclr_last_error(sim_.get()));
    cells_.assign(nodes, Cell<dim>());
    for (size_t k = 0; k < nodes; ++k) {
      for (int d = 0; d < dim; ++d) cells_[k].velocity(d) = vel[k * dim + d];
      cells_[k].mass = mass[k];
    }
    grid_fresh_ = true;
  }
};

}  // namespace nclr
