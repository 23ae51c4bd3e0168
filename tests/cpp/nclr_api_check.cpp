// Drives the drop-in C++ API (include/nclr.h) the way an embedder of the reference's header
// does: builds the two-cube 2D snow scene with cube<2>(), constructs MPMSimulation<2>, steps
// it with advance() and reads particles() and grid(); then checks the out-of-range error and a
// small 3D jelly run; then the extensions: the same scene with the neo-Hookean stress (an
// nclr_options constructor) and per-particle moduli (set_moduli).  Writes the initial and
// final particle states to <out.bin>, and the extension run's initial state, final state and
// moduli to <out.bin>.ext, so the Python test can compare them with the CPU oracle.
//
//   nclr_api_check <out.bin> <steps>
// Exit codes: 0 ok, 10+ a failed check.
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nclr.h"

namespace {

template <int dim>
void write_state(std::ofstream &f, const std::vector<nclr::Particle<dim>> &ps) {
  for (const auto &p : ps) {
    float rec[2 * dim + 2 * dim * dim + 1];
    int k = 0;
    for (int d = 0; d < dim; ++d) rec[k++] = p.x(d);
    for (int d = 0; d < dim; ++d) rec[k++] = p.v(d);
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) rec[k++] = p.F(i, j);
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) rec[k++] = p.C(i, j);
    rec[k++] = p.Jp;
    f.write(reinterpret_cast<const char *>(rec), sizeof(rec));
  }
}

}  // namespace

int main(int argc, char **argv) {
  using namespace nclr;
  const char *out = argc > 1 ? argv[1] : "nclr_api_check.bin";
  const int steps = argc > 2 ? std::atoi(argv[2]) : 1;

  std::vector<Particle<2>> particles;
  for (const auto &pos : cube<2>(50, 0.4, 0.6)) particles.emplace_back(pos, 0);
  auto lower = cube<2>(50, 0.4, 0.6);
  for (auto &pos : lower) {
    pos(1) -= 0.35;
    particles.emplace_back(Particle<2>(pos, 0));
  }
  auto sim = std::make_unique<MPMSimulation<2>>(particles, MaterialModel::kSnow);
  if (!sim->grid().empty()) return 10;  // grid() is empty before the first step
  if (sim->particles().size() != 5000) return 11;
  for (int s = 0; s < steps; ++s) sim->advance();
  const auto &now = sim->particles();
  if (sim->grid().size() != 65u * 65u) return 12;
  double grid_mass = 0.0;
  for (const auto &cell : sim->grid()) grid_mass += cell.mass;
  if (!(grid_mass > 4000.0 && grid_mass <= 5000.0 + 1e-2)) return 13;

  std::ofstream f(out, std::ios::binary);
  write_state<2>(f, particles);
  write_state<2>(f, now);
  f.close();

  // A particle outside the grid: the reference's vector::at throws std::out_of_range.
  std::vector<Particle<2>> bad{Particle<2>(Vector<real, 2>(0.5f, 0.5f), 0),
                               Particle<2>(Vector<real, 2>(-0.2f, 0.5f), 0)};
  MPMSimulation<2> bad_sim(bad, MaterialModel::kJelly);
  bool threw = false;
  try {
    bad_sim.advance();
  } catch (const std::out_of_range &) {
    threw = true;
  }
  if (!threw) return 14;

  // 3D jelly, 8^3 lattice on a 32^3 grid: runs, keeps the caller's particle count and order.
  std::vector<Particle<3>> p3;
  for (const auto &pos : cube<3>(8, 0.4, 0.5)) p3.emplace_back(pos, 1);
  MPMSimulation<3> sim3(p3, MaterialModel::kJelly, 32);
  sim3.advance(5);
  if (sim3.particles().size() != p3.size()) return 15;
  const float dz = sim3.particles()[0].x(2) - p3[0].x(2);
  if (!(dz < 1e-3f && dz > -1e-3f)) return 16;
  if (sim3.mu_0 <= 0.0f || sim3.lambda_0 <= 0.0f) return 17;

  // Extensions: neo-Hookean stress and one E / nu per particle.
  nclr_options opt;
  nclr_default_options(&opt);
  opt.stress_model = NCLR_STRESS_NEOHOOKEAN;
  MPMSimulation<2> ext(particles, MaterialModel::kSnow, 64, 1e-4f, 1e4f, 0.2f, -100.0f, &opt);
  std::vector<real> E(particles.size()), nu(particles.size());
  for (size_t p = 0; p < particles.size(); ++p) {
    E[p] = 2000.0f + 37.0f * (float)(p % 1000);
    nu[p] = 0.1f + 0.0003f * (float)(p % 1000);
  }
  bool rejected = false;
  try {
    ext.set_moduli(std::vector<real>(3, 1.0f), std::vector<real>(3, 0.2f));
  } catch (const std::invalid_argument &) {
    rejected = true;
  }
  if (!rejected) return 18;
  ext.set_moduli(E, nu);
  for (int s = 0; s < steps; ++s) ext.advance();
  std::ofstream g(std::string(out) + ".ext", std::ios::binary);
  write_state<2>(g, particles);
  write_state<2>(g, ext.particles());
  g.write(reinterpret_cast<const char *>(E.data()), sizeof(real) * E.size());
  g.write(reinterpret_cast<const char *>(nu.data()), sizeof(real) * nu.size());
  g.close();
  std::printf("ok\n");
  return 0;
}
