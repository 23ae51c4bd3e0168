// TEST INFRASTRUCTURE ONLY -- compiles the reference's own step code (src/nclr.h and
// src/nclr_math.h, read in place from the reference tree, unmodified) against the Eigen
// API shim in ref_shim/, and exposes it through the same extern "C" shape as
// oracle_capi.cpp so the tests can pin the oracle restatement to the reference itself.
// Built by oracle/build_oracle.py into oracle/_ref/ (git-ignored) only where the reference
// tree is present.
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "nclr.h"

namespace {

template <int D>
int run(int64_t n, double *x, double *v, double *F, double *C, double *Jp, const double *mass,
        const double *volume, int model, int res, double dt, double E, double nu,
        double gravity, int nsteps, double *grid_vel, double *grid_mass) {
  using nclr::real;
  std::vector<nclr::Particle<D>> ps;
  ps.reserve((size_t)n);
  for (int64_t p = 0; p < n; ++p) {
    nclr::Vector<real, D> px, pv;
    for (int d = 0; d < D; ++d) {
      px(d) = (real)x[p * D + d];
      pv(d) = (real)v[p * D + d];
    }
    nclr::Particle<D> q(px, 0, pv, (real)mass[p], (real)volume[p]);
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        q.F(i, j) = (real)F[p * D * D + i * D + j];
        q.C(i, j) = (real)C[p * D * D + i * D + j];
      }
    q.Jp = (real)Jp[p];
    ps.push_back(q);
  }
  nclr::MPMSimulation<D> sim(ps, (nclr::MaterialModel)model, res, (real)dt, (real)E, (real)nu,
                             (real)gravity);
  int status = 0;
  try {
    for (int s = 0; s < nsteps; ++s) sim.advance();
  } catch (const std::out_of_range &) {
    status = 2;
  }
  const auto &out = sim.particles();
  for (int64_t p = 0; p < n; ++p) {
    const auto &q = out[(size_t)p];
    for (int d = 0; d < D; ++d) {
      x[p * D + d] = (double)q.x(d);
      v[p * D + d] = (double)q.v(d);
    }
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        F[p * D * D + i * D + j] = (double)q.F(i, j);
        C[p * D * D + i * D + j] = (double)q.C(i, j);
      }
    Jp[p] = (double)q.Jp;
  }
  if (grid_vel && grid_mass) {
    const auto &g = sim.grid();
    for (size_t k = 0; k < g.size(); ++k) {
      for (int d = 0; d < D; ++d) grid_vel[k * D + d] = (double)g[k].velocity(d);
      grid_mass[k] = (double)g[k].mass;
    }
  }
  return status;
}

}  // namespace

extern "C" {

// Same contract as oracle_advance (FP32 only: the reference's `real` is float).
int ref_advance(int dim, int64_t n, double *x, double *v, double *F, double *C, double *Jp,
                const double *mass, const double *volume, int model, int res, double dt,
                double E, double nu, double gravity, int nsteps, double *grid_vel,
                double *grid_mass) {
  if (n < 0 || res < 1 || model < 0 || model > 2) return 1;
  if (dim == 2)
    return run<2>(n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, nsteps,
                  grid_vel, grid_mass);
  if (dim == 3)
    return run<3>(n, x, v, F, C, Jp, mass, volume, model, res, dt, E, nu, gravity, nsteps,
                  grid_vel, grid_mass);
  return 1;
}

// The reference's cube<dim>() scene builder (src/nclr_math.h:100-129), flattened
// point-major into `out` (n^dim * dim floats).
void ref_cube(int dim, int n, float lo, float hi, float *out) {
  if (dim == 2) {
    const auto pts = nclr::cube<2>(n, lo, hi);
    for (size_t i = 0; i < pts.size(); ++i)
      for (int d = 0; d < 2; ++d) out[i * 2 + d] = pts[i](d);
  } else {
    const auto pts = nclr::cube<3>(n, lo, hi);
    for (size_t i = 0; i < pts.size(); ++i)
      for (int d = 0; d < 3; ++d) out[i * 3 + d] = pts[i](d);
  }
}

}  // extern "C"
