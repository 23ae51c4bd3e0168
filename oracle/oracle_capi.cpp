// CPU ORACLE -- test infrastructure only (see nclr_oracle.h).
//
// extern "C" wrappers so the Python tests and the bench's CPU-baseline leg can drive the
// oracle through ctypes.  All arrays are float64 on the boundary; in FP32 mode each value
// is converted to float on entry (exact for float inputs) and back on exit.
//   x[p*dim+d], v[p*dim+d], F[p*dim*dim + r*dim + c] (row-major), C likewise, Jp[p],
//   mass[p], volume[p]; grid_vel[node*dim+d], grid_mass[node] in the reference's x-major
//   node order (src/nclr.h:141-142,152).
#include <cstring>
#include <vector>

#include "nclr_oracle.h"

using namespace oracle;

namespace {

template <typename T, int D>
int run(int physics, int64_t n, double *x, double *v, double *F, double *C, double *Jp,
        const double *mass, const double *volume, int model, int res, double dt, double E,
        double nu, double gravity, int nsteps, double *grid_vel, double *grid_mass,
        int64_t *counters) {
  std::vector<Particle<T, D>> ps((size_t)n);
  for (int64_t p = 0; p < n; ++p) {
    auto &q = ps[(size_t)p];
    for (int d = 0; d < D; ++d) {
      q.x[d] = (T)x[p * D + d];
      q.v[d] = (T)v[p * D + d];
    }
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        q.F(i, j) = (T)F[p * D * D + i * D + j];
        q.C(i, j) = (T)C[p * D * D + i * D + j];
      }
    q.Jp = (T)Jp[p];
    q.mass = (T)mass[p];
    q.volume = (T)volume[p];
  }
  Simulation<T, D> sim(std::move(ps), (Model)model, res, (T)dt, (T)E, (T)nu, (T)gravity,
                       (Physics)physics);
  int status = 0;
  try {
    for (int s = 0; s < nsteps; ++s) sim.advance();
  } catch (const std::out_of_range &) {
    status = 2;
  }
  auto &out = sim.particles();
  for (int64_t p = 0; p < n; ++p) {
    const auto &q = out[(size_t)p];
    for (int d = 0; d < D; ++d) {
      x[p * D + d] = (double)q.x[d];
      v[p * D + d] = (double)q.v[d];
    }
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        F[p * D * D + i * D + j] = (double)q.F(i, j);
        C[p * D * D + i * D + j] = (double)q.C(i, j);
      }
    Jp[p] = (double)q.Jp;
  }
  const auto &g = sim.grid();
  if (grid_vel && grid_mass) {
    for (size_t k = 0; k < g.size(); ++k) {
      for (int d = 0; d < D; ++d) grid_vel[k * D + d] = (double)g[k].velocity[d];
      grid_mass[k] = (double)g[k].mass;
    }
  }
  if (counters) {
    counters[0] = sim.counters.inverted_svd;
    counters[1] = sim.counters.out_of_range;
  }
  return status;
}

template <typename T, int D>
void svd(int physics, const double *A, double *U, double *S, double *V) {
  Mat<T, D> a, u, s, vv;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) a(i, j) = (T)A[i * D + j];
  nclr_svd<T, D>(a, u, s, vv, (Physics)physics);
  for (int i = 0; i < D; ++i) {
    S[i] = (double)s(i, i);
    for (int j = 0; j < D; ++j) {
      U[i * D + j] = (double)u(i, j);
      V[i * D + j] = (double)vv(i, j);
    }
  }
}

template <typename T, int D>
void polar(int physics, const double *A, double *R) {
  Mat<T, D> a;
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) a(i, j) = (T)A[i * D + j];
  const Mat<T, D> r = nclr_polar_R<T, D>(a, (Physics)physics);
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) R[i * D + j] = (double)r(i, j);
}

}  // namespace

extern "C" {

// Runs `nsteps` calls of advance() on the given state, in place.  Returns 0, or 2 when a
// grid index went out of range (the reference's std::out_of_range), or 1 on bad arguments.
int oracle_advance(int dim, int fp64, int physics, int64_t n, double *x, double *v, double *F,
                   double *C, double *Jp, const double *mass, const double *volume, int model,
                   int res, double dt, double E, double nu, double gravity, int nsteps,
                   double *grid_vel, double *grid_mass, int64_t *counters) {
  if (n < 0 || res < 1 || (dim != 2 && dim != 3) || model < 0 || model > 2) return 1;
#define ORACLE_RUN(T, D)                                                                   \
  return run<T, D>(physics, n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, \
                   nsteps, grid_vel, grid_mass, counters)
  if (dim == 2) {
    if (fp64) ORACLE_RUN(double, 2);
    ORACLE_RUN(float, 2);
  }
  if (fp64) ORACLE_RUN(double, 3);
  ORACLE_RUN(float, 3);
#undef ORACLE_RUN
}

// nclr_svd (src/nclr_math.h:50-74): U, V row-major dim x dim, S the dim diagonal entries.
int oracle_svd(int dim, int fp64, int physics, const double *A, double *U, double *S, double *V) {
  if (dim == 2) {
    if (fp64) svd<double, 2>(physics, A, U, S, V); else svd<float, 2>(physics, A, U, S, V);
  } else if (dim == 3) {
    if (fp64) svd<double, 3>(physics, A, U, S, V); else svd<float, 3>(physics, A, U, S, V);
  } else {
    return 1;
  }
  return 0;
}

// nclr_polar's R (src/nclr_math.h:76-98).
int oracle_polar(int dim, int fp64, int physics, const double *A, double *R) {
  if (dim == 2) {
    if (fp64) polar<double, 2>(physics, A, R); else polar<float, 2>(physics, A, R);
  } else if (dim == 3) {
    if (fp64) polar<double, 3>(physics, A, R); else polar<float, 3>(physics, A, R);
  } else {
    return 1;
  }
  return 0;
}

// cube<dim>'s per-axis coordinates: LinSpaced(n, lo, hi) in float (src/nclr_math.h:103).
void oracle_linspaced(int n, float lo, float hi, float *out) {
  const auto r = linspaced<float>(n, lo, hi);
  for (int i = 0; i < n; ++i) out[i] = r[(size_t)i];
}

}  // extern "C"
