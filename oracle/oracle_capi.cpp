// CPU ORACLE -- test infrastructure only (see nclr_oracle.h).
//
// extern "C" wrappers so the Python tests and the bench's CPU-baseline leg can drive the
// oracle through ctypes.  All arrays are float64 on the boundary; in FP32 mode each value
// is converted to float on entry (exact for float inputs) and back on exit.
//   x[p*dim+d], v[p*dim+d], F[p*dim*dim + r*dim + c] (row-major), C likewise, Jp[p],
//   mass[p], volume[p]; grid_vel[node*dim+d], grid_mass[node] in the reference's x-major
//   node order (src/nclr.h:141-142,152).
#include <cstring>
#include <tuple>
#include <vector>

#include "nclr_adjoint.h"
#include "nclr_oracle_mt.h"
#include "nclr_oracle.h"

using namespace oracle;

namespace {

template <typename T, int D>
int run(int physics, int64_t n, double *x, double *v, double *F, double *C, double *Jp,
        const double *mass, const double *volume, int model, int res, double dt, double E,
        double nu, double gravity, int nsteps, double *grid_vel, double *grid_mass,
        int64_t *counters, const uint8_t *material, int threads = 1,
        const double *E_p = nullptr, const double *nu_p = nullptr, int stress = 0) {
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
    q.material = material ? (int)material[p] : -1;
    if (E_p && nu_p) std::tie(q.mu0, q.lambda0) = lame_of<T>((T)E_p[p], (T)nu_p[p]);
  }
  Simulation<T, D> sim(std::move(ps), (Model)model, res, (T)dt, (T)E, (T)nu, (T)gravity,
                       (Physics)physics);
  sim.stress_ = (Stress)stress;
  int status = 0;
  try {
    for (int s = 0; s < nsteps; ++s) {
      if (threads > 1)
        advance_threads(sim, threads);
      else
        sim.advance();
    }
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

template <int D>
int adjoint(int physics, int64_t n, const double *x0, const double *v0, const double *F0,
            const double *C0, const double *mass, const double *volume, int res, double dt,
            double E, double nu, double gravity, int nsteps, double *xT, double *vT, double *FT,
            double *CT, const double *gx, const double *gv, const double *gF, const double *gC,
            double *gx0, double *gv0, double *gF0, double *gC0, double *gmu_glambda,
            int stress, const double *E_p, const double *nu_p, double *gmu_rows,
            double *glambda_rows, int model = 1, const double *Jp0 = nullptr,
            double *JpT = nullptr, const double *gJp = nullptr, double *gJp0 = nullptr) {
  using T = double;
  std::vector<Particle<T, D>> ps((size_t)n);
  for (int64_t p = 0; p < n; ++p) {
    auto &q = ps[(size_t)p];
    for (int d = 0; d < D; ++d) {
      q.x[d] = x0[p * D + d];
      q.v[d] = v0[p * D + d];
    }
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        q.F(i, j) = F0[p * D * D + i * D + j];
        q.C(i, j) = C0[p * D * D + i * D + j];
      }
    q.Jp = Jp0 ? Jp0[p] : 1.0;
    q.mass = mass[p];
    q.volume = volume[p];
    if (E_p && nu_p) std::tie(q.mu0, q.lambda0) = lame_of<T>(E_p[p], nu_p[p]);
  }
  try {
    Adjoint<T, D> adj(std::move(ps), (Model)model, res, dt, E, nu, gravity, (Physics)physics,
                      nsteps, (Stress)stress);
    const auto &fin = adj.final_state();
    StepAdjoint<T, D> seed;
    seed.x.resize((size_t)n);
    seed.v.resize((size_t)n);
    seed.F.resize((size_t)n);
    seed.C.resize((size_t)n);
    seed.Jp.assign((size_t)n, 0.0);
    for (int64_t p = 0; p < n; ++p) {
      const auto &q = fin[(size_t)p];
      if (JpT) JpT[p] = q.Jp;
      if (gJp) seed.Jp[(size_t)p] = gJp[p];
      for (int d = 0; d < D; ++d) {
        xT[p * D + d] = q.x[d];
        vT[p * D + d] = q.v[d];
        seed.x[(size_t)p][d] = gx ? gx[p * D + d] : 0.0;
        seed.v[(size_t)p][d] = gv ? gv[p * D + d] : 0.0;
      }
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          FT[p * D * D + i * D + j] = q.F(i, j);
          CT[p * D * D + i * D + j] = q.C(i, j);
          seed.F[(size_t)p](i, j) = gF ? gF[p * D * D + i * D + j] : 0.0;
          seed.C[(size_t)p](i, j) = gC ? gC[p * D * D + i * D + j] : 0.0;
        }
    }
    T gmu = 0, glam = 0;
    std::vector<T> rows_mu, rows_lambda;
    const bool rows = gmu_rows || glambda_rows;
    const StepAdjoint<T, D> out = adj.backward(seed, gmu, glam, rows ? &rows_mu : nullptr,
                                               rows ? &rows_lambda : nullptr);
    for (int64_t p = 0; rows && p < n; ++p) {
      if (gmu_rows) gmu_rows[p] = rows_mu[(size_t)p];
      if (glambda_rows) glambda_rows[p] = rows_lambda[(size_t)p];
    }
    for (int64_t p = 0; p < n; ++p) {
      for (int d = 0; d < D; ++d) {
        gx0[p * D + d] = out.x[(size_t)p][d];
        gv0[p * D + d] = out.v[(size_t)p][d];
      }
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          gF0[p * D * D + i * D + j] = out.F[(size_t)p](i, j);
          gC0[p * D * D + i * D + j] = out.C[(size_t)p](i, j);
        }
    }
    for (int64_t p = 0; gJp0 && p < n; ++p) gJp0[p] = out.Jp[(size_t)p];
    gmu_glambda[0] = gmu;
    gmu_glambda[1] = glam;
  } catch (const std::out_of_range &) {
    return 2;
  }
  return 0;
}

}  // namespace

extern "C" {

// FP64 reverse pass of an `nsteps` jelly rollout (nclr_adjoint.h): the forward final state
// into xT/vT/FT/CT, the adjoint of the initial state (given the final state's adjoint
// gx/gv/gF/gC, any may be NULL = 0) into gx0/gv0/gF0/gC0, and the adjoints of mu_0 and
// lambda_0 into gmu_glambda[0..1].  stress: 0 fixed corotated, 1 neo-Hookean.  E_p / nu_p (may
// be NULL) give every particle its own moduli; gmu_rows / glambda_rows (may be NULL) then
// receive each particle's own mu_0 / lambda_0 adjoints.  Returns 0, 2 (a stencil left the
// grid) or 1.
int oracle_adjoint(int dim, int physics, int64_t n, const double *x0, const double *v0,
                   const double *F0, const double *C0, const double *mass, const double *volume,
                   int res, double dt, double E, double nu, double gravity, int nsteps,
                   double *xT, double *vT, double *FT, double *CT, const double *gx,
                   const double *gv, const double *gF, const double *gC, double *gx0,
                   double *gv0, double *gF0, double *gC0, double *gmu_glambda, int stress,
                   const double *E_p, const double *nu_p, double *gmu_rows,
                   double *glambda_rows) {
  if (n < 0 || res < 1 || nsteps < 0 || stress < 0 || stress > 1 || (!E_p) != (!nu_p)) return 1;
  if (dim == 2)
    return adjoint<2>(physics, n, x0, v0, F0, C0, mass, volume, res, dt, E, nu, gravity, nsteps,
                      xT, vT, FT, CT, gx, gv, gF, gC, gx0, gv0, gF0, gC0, gmu_glambda, stress,
                      E_p, nu_p, gmu_rows, glambda_rows);
  if (dim == 3)
    return adjoint<3>(physics, n, x0, v0, F0, C0, mass, volume, res, dt, E, nu, gravity, nsteps,
                      xT, vT, FT, CT, gx, gv, gF, gC, gx0, gv0, gF0, gC0, gmu_glambda, stress,
                      E_p, nu_p, gmu_rows, glambda_rows);
  return 1;
}

// oracle_adjoint for any material (`model`: 0 snow, 1 jelly, 2 liquid), with the plastic
// volume ratio Jp in the state: Jp0 the initial one (NULL: 1), JpT (may be NULL) receives the
// final one, gJp (may be NULL = 0) is its adjoint's seed and gJp0 (may be NULL) receives the
// adjoint of Jp0.
int oracle_adjoint_model(int dim, int physics, int model, int64_t n, const double *x0,
                         const double *v0, const double *F0, const double *C0,
                         const double *Jp0, const double *mass, const double *volume, int res,
                         double dt, double E, double nu, double gravity, int nsteps, double *xT,
                         double *vT, double *FT, double *CT, double *JpT, const double *gx,
                         const double *gv, const double *gF, const double *gC,
                         const double *gJp, double *gx0, double *gv0, double *gF0,
                         double *gC0, double *gJp0, double *gmu_glambda, int stress) {
  if (n < 0 || res < 1 || nsteps < 0 || stress < 0 || stress > 1 || model < 0 || model > 2)
    return 1;
  if (dim == 2)
    return adjoint<2>(physics, n, x0, v0, F0, C0, mass, volume, res, dt, E, nu, gravity, nsteps,
                      xT, vT, FT, CT, gx, gv, gF, gC, gx0, gv0, gF0, gC0, gmu_glambda, stress,
                      nullptr, nullptr, nullptr, nullptr, model, Jp0, JpT, gJp, gJp0);
  if (dim == 3)
    return adjoint<3>(physics, n, x0, v0, F0, C0, mass, volume, res, dt, E, nu, gravity, nsteps,
                      xT, vT, FT, CT, gx, gv, gF, gC, gx0, gv0, gF0, gC0, gmu_glambda, stress,
                      nullptr, nullptr, nullptr, nullptr, model, Jp0, JpT, gJp, gJp0);
  return 1;
}


// Runs `nsteps` calls of advance() on the given state, in place.  Returns 0, or 2 when a
// grid index went out of range (the reference's std::out_of_range), or 1 on bad arguments.
// `material` (may be NULL): one MaterialModel per particle, the mixed-material extension.
int oracle_advance(int dim, int fp64, int physics, int64_t n, double *x, double *v, double *F,
                   double *C, double *Jp, const double *mass, const double *volume, int model,
                   int res, double dt, double E, double nu, double gravity, int nsteps,
                   double *grid_vel, double *grid_mass, int64_t *counters,
                   const uint8_t *material) {
  if (n < 0 || res < 1 || (dim != 2 && dim != 3) || model < 0 || model > 2) return 1;
#define ORACLE_RUN(T, D)                                                                   \
  return run<T, D>(physics, n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, \
                   nsteps, grid_vel, grid_mass, counters, material)
  if (dim == 2) {
    if (fp64) ORACLE_RUN(double, 2);
    ORACLE_RUN(float, 2);
  }
  if (fp64) ORACLE_RUN(double, 3);
  ORACLE_RUN(float, 3);
#undef ORACLE_RUN
}

// oracle_advance on `threads` host threads (nclr_oracle_mt.h): the multi-threaded CPU
// baseline.  Same arguments and results up to the FP32 summation order of the grid.
int oracle_advance_threads(int dim, int fp64, int physics, int64_t n, double *x, double *v,
                           double *F, double *C, double *Jp, const double *mass,
                           const double *volume, int model, int res, double dt, double E,
                           double nu, double gravity, int nsteps, double *grid_vel,
                           double *grid_mass, int64_t *counters, const uint8_t *material,
                           int threads) {
  if (n < 0 || res < 1 || (dim != 2 && dim != 3) || model < 0 || model > 2 || threads < 1) return 1;
#define ORACLE_RUN(T, D)                                                                   \
  return run<T, D>(physics, n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, \
                   nsteps, grid_vel, grid_mass, counters, material, threads)
  if (dim == 2) {
    if (fp64) ORACLE_RUN(double, 2);
    ORACLE_RUN(float, 2);
  }
  if (fp64) ORACLE_RUN(double, 3);
  ORACLE_RUN(float, 3);
#undef ORACLE_RUN
}

// oracle_advance with the model extensions: E_p / nu_p (both or neither, may be NULL) give
// every particle its own Young's modulus and Poisson ratio; stress 0 is the reference's
// fixed-corotated stress, 1 the neo-Hookean one; threads > 1 runs the multi-threaded step.
int oracle_advance_ex(int dim, int fp64, int physics, int64_t n, double *x, double *v, double *F,
                      double *C, double *Jp, const double *mass, const double *volume, int model,
                      int res, double dt, double E, double nu, double gravity, int nsteps,
                      double *grid_vel, double *grid_mass, int64_t *counters,
                      const uint8_t *material, const double *E_p, const double *nu_p,
                      int stress, int threads) {
  if (n < 0 || res < 1 || (dim != 2 && dim != 3) || model < 0 || model > 2 || threads < 1 ||
      stress < 0 || stress > 1 || (!E_p) != (!nu_p))
    return 1;
#define ORACLE_RUN(T, D)                                                                   \
  return run<T, D>(physics, n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, \
                   nsteps, grid_vel, grid_mass, counters, material, threads, E_p, nu_p, stress)
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
