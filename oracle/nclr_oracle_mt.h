// CPU ORACLE -- test infrastructure only (the multi-threaded CPU baseline).
//
// advance_threads(sim, threads) runs the oracle's step (nclr_oracle.h) on `threads` host
// threads, for timing the CPU side at full width.  The reference itself runs on one thread
// (its OpenMP pragmas are inert: it is built without -fopenmp, and nclr.h:264's misspelt
// clause would not compile with it; a naive `omp parallel for` over its P2G would race on
// the grid).  The parallel form here is race-free and does the same arithmetic per particle
// and per node (Simulation::p2g_particle / grid_node / g2p_particle):
//   * P2G: particles are bucketed by x-slab of kSlab = 3 cells (their stencil base, clamped);
//     a particle's stencil spans base .. base + 2, so the nodes written from slab s lie in
//     [3s, 3s + 5).  Even slabs run in parallel (threads take slabs one at a time), then odd
//     slabs: slabs of one colour start 6 cells apart, so no two threads touch the same node.
//     Only the order in which contributions reach a node changes (FP32 summation order);
//   * grid update and G2P: independent per node / per particle, split into contiguous ranges.
// A stencil outside the grid is reported like the serial step (std::out_of_range), after the
// threads join.
#pragma once

#include <atomic>
#include <exception>
#include <thread>
#include <vector>

#include "nclr_oracle.h"

namespace oracle {

template <typename F>
void parallel_ranges(int threads, int64_t n, F &&body) {  // body(begin, end)
  std::vector<std::thread> pool;
  std::atomic<bool> failed{false};
  std::exception_ptr error;
  std::atomic<int> error_taken{0};
  const int64_t chunk = (n + threads - 1) / threads;
  for (int t = 0; t < threads; ++t) {
    const int64_t b = t * chunk, e = std::min<int64_t>(n, b + chunk);
    if (b >= e) break;
    pool.emplace_back([&, b, e] {
      try {
        body(b, e);
      } catch (...) {
        if (error_taken.exchange(1) == 0) error = std::current_exception();
        failed = true;
      }
    });
  }
  for (auto &th : pool) th.join();
  if (failed) std::rethrow_exception(error);
}

// Runs body(k) for k in [0, n) on `threads` threads taking items one at a time (uneven items).
template <typename F>
void parallel_items(int threads, int64_t n, F &&body) {
  std::atomic<int64_t> next{0};
  parallel_ranges(threads, threads, [&](int64_t, int64_t) {
    for (int64_t k; (k = next.fetch_add(1)) < n;) body(k);
  });
}

template <typename T, int D>
void advance_threads(Simulation<T, D> &sim, int threads) {
  constexpr int kSlab = 3;  // the narrowest slab whose colour-mates never share a node
  auto &ps = sim.particles_;
  const int64_t n = (int64_t)ps.size();
  // ---- P2G, two colours of x-slabs ----
  const int64_t nodes = sim.num_nodes();
  sim.cells_.resize((size_t)nodes);
  parallel_ranges(threads, nodes, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) sim.cells_[(size_t)i] = Cell<T, D>{Vec<T, D>::constant(T(0)), T(0)};
  });
  const int nslabs = (sim.res_ + 1) / kSlab + 1;
  std::vector<std::vector<int64_t>> slab((size_t)nslabs);
  for (int64_t p = 0; p < n; ++p) {
    int base[D];
    Vec<T, D> fx, w[3];
    sim.kernel(ps[(size_t)p].x, base, fx, w);
    const int s = std::min(std::max(base[0], 0) / kSlab, nslabs - 1);
    slab[(size_t)s].push_back(p);
  }
  for (int colour = 0; colour < 2; ++colour) {
    std::vector<int> mine;
    for (int s = colour; s < nslabs; s += 2) mine.push_back(s);
    parallel_items(threads, (int64_t)mine.size(), [&](int64_t k) {
      for (int64_t p : slab[(size_t)mine[(size_t)k]]) sim.p2g_particle(ps[(size_t)p]);
    });
  }
  // ---- grid update ----
  parallel_ranges(threads, sim.num_nodes(), [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) sim.grid_node(i);
  });
  // ---- G2P ----
  parallel_ranges(threads, n, [&](int64_t b, int64_t e) {
    for (int64_t p = b; p < e; ++p) sim.g2p_particle(ps[(size_t)p]);
  });
}

}  // namespace oracle
