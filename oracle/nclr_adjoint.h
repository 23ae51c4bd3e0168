// CPU ORACLE -- test infrastructure only.
//
// Reverse-mode derivative (adjoint) of a rollout of MPMSimulation<dim>::advance() steps for
// every material (src/nclr.h:80-372: jelly, and the plasticity of snow and liquid), restated
// in plain C++ on top of the forward restatement in nclr_oracle.h.  It is the checker of the
// GPU adjoint: FP64, every intermediate state and grid of the rollout kept in memory (small
// cases only).
//
// One step maps s_t = (x, v, F, C, Jp) to s_{t+1}; its reverse maps the adjoint of s_{t+1} to
// the adjoint of s_t and accumulates the adjoints of mu_0 and lambda_0:
//   G2P    v' = sum_o W_o vg_i,  C' = 4 inv_dx sum_o W_o vg_i (o - fx)^T,  x' = x + dt v',
//          F_hat = (I + dt C') F, then per material                    (src/nclr.h:167-259)
//            jelly   F' = F_hat
//            snow    F_hat = U S V^T, F' = U f(S) V^T with f the clamp to [1 - 2.5e-2,
//                    1 + 4.5e-3], Jp' = clamp(Jp det F_hat / det F', 0.6, 20)
//            liquid  F' = I with F'_00 = J = prod S (the signed det F_hat; |det F_hat| where
//                    the 2D sign fix is a no-op)
//          The snow F' is a function of the singular values: with P = U^T dF_hat V it moves by
//          U K V^T, K_ii = f'(s_i) P_ii and, off the diagonal,
//          K_ij = (a_ij + b_ij)/2 P_ij + (a_ij - b_ij)/2 P_ji, a_ij = (f_i - f_j) / (s_i - s_j),
//          b_ij = (f_i + f_j) / (s_i + s_j) (f' = 0 where the clamp is active); the adjoint is
//          the same map applied to U^T F'_bar V.  Jp' depends on the s_i through
//          prod s / prod f(s) and is constant where its own clamp is active.
//   grid   vg = clamp(mv / m + dt g e_y) unless m = 0 or the sticky boundary zeroes the node
//                                                                        (src/nclr.h:263-310)
//   P2G    mv_i = sum_p W_o (m v + A dpos_o), m_i = sum_p W_o m, dpos_o = (o - fx) dx,
//          A = -(dt vol 4 inv_dx^2) (2 mu (F - R) F^T + lambda (J - 1) J 1) + m C
//                                                                        (src/nclr.h:104-337)
//          or, with the neo-Hookean stress extension (src/nclr.h:339's TODO),
//          A = -(dt vol 4 inv_dx^2) (mu (F F^T - I) + lambda ln(J) I) + m C, whose F adjoint
//          is mu (G + G^T) F + lambda tr(G) F^-T for the stress adjoint G
// with W_o the product of the quadratic B-spline weights of fx = x inv_dx - base.  Clamped
// velocity components and stuck or empty nodes pass no gradient.  The polar rotation's
// derivative: with F = U S V^T and R = U V^T, a perturbation dF moves R by
// U K V^T with K_ij = (M_ij - M_ji) / (s_i + s_j), M = U^T dF V, so the adjoint is
// F_bar = U Z V^T with Z_ij = (P_ij - P_ji) / (s_i + s_j), P = U^T R_bar V (3D); the 2D polar
// rotation is the closed form of src/nclr_math.h:80-89 and is differentiated directly.
#pragma once

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <vector>

#include "nclr_oracle.h"

namespace oracle {

template <typename T, int D>
struct StepAdjoint {
  std::vector<Vec<T, D>> x, v;
  std::vector<Mat<T, D>> F, C;
  std::vector<T> Jp;  // empty: zero
};

// The snow clamp of src/nclr.h:237-241 and its derivative.
template <typename T>
T snow_clamp(T s) {
  return std::clamp(s, T(1.0 - 2.5e-2), T(1.0 + 4.5e-3));
}
template <typename T>
T snow_clamp_slope(T s) {
  return (s > T(1.0 - 2.5e-2) && s < T(1.0 + 4.5e-3)) ? T(1) : T(0);
}

// Adjoint of the snow plasticity of one particle: F_hat -> (F', Jp') given the adjoints Fb of
// F' and Jpb of Jp'; returns the adjoint of F_hat and adds that of the incoming Jp to *Jp_bar.
template <typename T, int D>
Mat<T, D> snow_backward(const Mat<T, D> &Fh, T Jp, const Mat<T, D> &Fb, T Jpb, Physics mode,
                        T *Jp_bar) {
  Mat<T, D> U, sig, V;
  nclr_svd<T, D>(Fh, U, sig, V, mode);
  T s[D], f[D], fp[D];
  for (int i = 0; i < D; ++i) {
    s[i] = sig(i, i);
    f[i] = snow_clamp(s[i]);
    fp[i] = snow_clamp_slope(s[i]);
  }
  const Mat<T, D> Pb = mul(mul(transpose(U), Fb), V);
  Mat<T, D> K = Mat<T, D>::constant(T(0));
  const T tiny = T(1e-12);
  for (int i = 0; i < D; ++i)
    for (int j = 0; j < D; ++j) {
      if (i == j) {
        K(i, i) = fp[i] * Pb(i, i);
        continue;
      }
      const T a = std::fabs(s[i] - s[j]) > tiny ? (f[i] - f[j]) / (s[i] - s[j])
                                                : T(0.5) * (fp[i] + fp[j]);
      const T b = std::fabs(s[i] + s[j]) > tiny ? (f[i] + f[j]) / (s[i] + s[j]) : T(0);
      K(i, j) = T(0.5) * (a + b) * Pb(i, j) + T(0.5) * (a - b) * Pb(j, i);
    }
  // Jp' = clamp(r, 0.6, 20), r = Jp prod s / prod f (the det U det V factors of det F_hat and
  // det F' cancel)
  T ps = T(1), pf = T(1);
  for (int i = 0; i < D; ++i) {
    ps *= s[i];
    pf *= f[i];
  }
  const T r = Jp * ps / pf;
  if (r > T(0.6) && r < T(20.0) && Jpb != T(0)) {
    *Jp_bar += Jpb * ps / pf;
    for (int i = 0; i < D; ++i) {
      T others = T(1);
      for (int k = 0; k < D; ++k)
        if (k != i) others *= s[k];
      K(i, i) += Jpb * (Jp * others / pf - r * fp[i] / f[i]);
    }
  }
  return mul(mul(U, K), transpose(V));
}

// d det(F) / dF
template <typename T>
Mat<T, 2> cofactor(const Mat<T, 2> &a) {
  Mat<T, 2> c;
  c(0, 0) = a(1, 1);
  c(0, 1) = -a(1, 0);
  c(1, 0) = -a(0, 1);
  c(1, 1) = a(0, 0);
  return c;
}
template <typename T>
Mat<T, 3> cofactor(const Mat<T, 3> &a) {
  Mat<T, 3> c;
  c(0, 0) = a(1, 1) * a(2, 2) - a(1, 2) * a(2, 1);
  c(0, 1) = a(1, 2) * a(2, 0) - a(1, 0) * a(2, 2);
  c(0, 2) = a(1, 0) * a(2, 1) - a(1, 1) * a(2, 0);
  c(1, 0) = a(0, 2) * a(2, 1) - a(0, 1) * a(2, 2);
  c(1, 1) = a(0, 0) * a(2, 2) - a(0, 2) * a(2, 0);
  c(1, 2) = a(0, 1) * a(2, 0) - a(0, 0) * a(2, 1);
  c(2, 0) = a(0, 1) * a(1, 2) - a(0, 2) * a(1, 1);
  c(2, 1) = a(0, 2) * a(1, 0) - a(0, 0) * a(1, 2);
  c(2, 2) = a(0, 0) * a(1, 1) - a(0, 1) * a(1, 0);
  return c;
}

// Adjoint of the polar rotation R(F) (nclr_polar, src/nclr_math.h:76-98).
template <typename T, int D>
Mat<T, D> polar_backward(const Mat<T, D> &F, const Mat<T, D> &Rbar, Physics mode) {
  Mat<T, D> out = Mat<T, D>::constant(T(0));
  if constexpr (D == 2) {
    const T a = F(0, 0) + F(1, 1), b = F(1, 0) - F(0, 1);
    const T r2 = a * a + b * b;
    const T r3 = r2 * std::sqrt(r2);
    const T cbar = Rbar(0, 0) + Rbar(1, 1), sbar = Rbar(1, 0) - Rbar(0, 1);
    const T abar = (cbar * b * b - sbar * a * b) / r3;
    const T bbar = (-cbar * a * b + sbar * a * a) / r3;
    out(0, 0) = abar;
    out(1, 1) = abar;
    out(1, 0) = bbar;
    out(0, 1) = -bbar;
  } else {
    Mat<T, D> U, sig, V;
    nclr_svd<T, D>(F, U, sig, V, mode);
    const Mat<T, D> P = mul(mul(transpose(U), Rbar), V);
    Mat<T, D> Z = Mat<T, D>::constant(T(0));
    for (int i = 0; i < D; ++i)
      for (int j = 0; j < D; ++j) {
        if (i == j) continue;
        const T s = sig(i, i) + sig(j, j);
        if (std::fabs(s) > T(1e-30)) Z(i, j) = (P(i, j) - P(j, i)) / s;
      }
    out = mul(mul(U, Z), transpose(V));
  }
  return out;
}

template <typename T, int D>
class Adjoint {
 public:
  using Sim = Simulation<T, D>;

  // Runs `nsteps` forward steps from `initial`, keeping every state and updated grid.
  Adjoint(std::vector<Particle<T, D>> initial, Model model, int res, T dt, T E, T nu,
          T gravity, Physics mode, int nsteps, Stress stress = Stress::kCorotated)
      : sim_(initial, model, res, dt, E, nu, gravity, mode), mode_(mode) {
    sim_.stress_ = stress;
    states_.push_back(sim_.particles());
    for (int t = 0; t < nsteps; ++t) {
      sim_.p2g();
      sim_.grid_op();
      grids_.push_back(sim_.cells_);
      sim_.g2p();
      states_.push_back(sim_.particles());
    }
  }

  const std::vector<Particle<T, D>> &final_state() const { return states_.back(); }

  // Reverse pass from the adjoint of the final state; returns the adjoint of the initial
  // state, accumulates mu_0 / lambda_0 adjoints.
  // With per-particle moduli (Particle::mu0 / lambda0), gmu_rows / glambda_rows (may be null)
  // receive each particle's own mu_0 / lambda_0 adjoints; gmu0 / glambda0 are their sums.
  StepAdjoint<T, D> backward(StepAdjoint<T, D> adj, T &gmu0, T &glambda0,
                             std::vector<T> *gmu_rows = nullptr,
                             std::vector<T> *glambda_rows = nullptr) {
    gmu0 = T(0);
    glambda0 = T(0);
    rows_mu_ = gmu_rows;
    rows_lambda_ = glambda_rows;
    if (rows_mu_) rows_mu_->assign(states_.front().size(), T(0));
    if (rows_lambda_) rows_lambda_->assign(states_.front().size(), T(0));
    for (int t = (int)grids_.size() - 1; t >= 0; --t) adj = step_backward(t, adj, gmu0, glambda0);
    return adj;
  }

 private:
  Sim sim_;
  Physics mode_;
  std::vector<T> *rows_mu_ = nullptr, *rows_lambda_ = nullptr;  // per-particle adjoints
  std::vector<std::vector<Particle<T, D>>> states_;
  std::vector<std::vector<Cell<T, D>>> grids_;

  struct Stencil {
    int base[D];
    T fx[D], w[3][D], dw[3][D];
  };

  Stencil stencil(const Vec<T, D> &x) const {
    Stencil s;
    for (int d = 0; d < D; ++d) {
      s.base[d] = (int)(x[d] * sim_.inv_dx_ - T(0.5));
      s.fx[d] = x[d] * sim_.inv_dx_ - (T)s.base[d];
      const T f = s.fx[d];
      s.w[0][d] = T(0.5) * (T(1.5) - f) * (T(1.5) - f);
      s.w[1][d] = T(0.75) - (f - T(1)) * (f - T(1));
      s.w[2][d] = T(0.5) * (f - T(0.5)) * (f - T(0.5));
      s.dw[0][d] = f - T(1.5);
      s.dw[1][d] = -T(2) * (f - T(1));
      s.dw[2][d] = f - T(0.5);
    }
    return s;
  }

  static constexpr int kS = (D == 3) ? 27 : 9;
  static void offsets(int o, int oo[3]) {
    oo[0] = (D == 3) ? o / 9 : o / 3;
    oo[1] = (D == 3) ? (o / 3) % 3 : o % 3;
    oo[2] = (D == 3) ? o % 3 : 0;
  }
  T weight(const Stencil &s, const int oo[3]) const {
    T w = s.w[oo[0]][0] * s.w[oo[1]][1];
    if (D == 3) w *= s.w[oo[2]][2];
    return w;
  }
  int64_t node(const Stencil &s, const int oo[3]) const {
    const int64_t N = sim_.res_ + 1;
    int64_t f = 0;
    for (int d = 0; d < D; ++d) f = f * N + (s.base[d] + oo[d]);
    if (f < 0 || f >= (int64_t)sim_.cells_.size()) throw std::out_of_range("stencil left the grid");
    return f;
  }
  // d fx from the adjoints of the stencil weights W_o
  void weight_backward(const Stencil &s, const T Wbar[kS], T gfx[D]) const {
    for (int d = 0; d < D; ++d)
      for (int o = 0; o < kS; ++o) {
        int oo[3];
        offsets(o, oo);
        T other = T(1);
        for (int e = 0; e < D; ++e)
          if (e != d) other *= s.w[oo[e]][e];
        gfx[d] += Wbar[o] * other * s.dw[oo[d]][d];
      }
  }

  StepAdjoint<T, D> step_backward(int t, const StepAdjoint<T, D> &next, T &gmu0, T &glambda0) {
    const auto &P = states_[(size_t)t];
    const auto &Pn = states_[(size_t)t + 1];
    const auto &grid = grids_[(size_t)t];
    const size_t n = P.size();
    const T inv_dx = sim_.inv_dx_, dx = sim_.dx_, dt = sim_.dt_;
    const T cscale = T(4) * inv_dx;
    StepAdjoint<T, D> out;
    out.x.resize(n);
    out.v.resize(n);
    out.F.resize(n);
    out.C.resize(n);
    out.Jp.assign(n, T(0));
    std::vector<Vec<T, D>> VB(grid.size(), Vec<T, D>::constant(T(0)));
    const Mat<T, D> I = diag_of<T, D>(T(1), mode_);
    // ---- G2P reverse ----
    for (size_t p = 0; p < n; ++p) {
      const Stencil s = stencil(P[p].x);
      const Mat<T, D> &F = P[p].F;
      const Mat<T, D> &Cn = Pn[p].C;
      Mat<T, D> M;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) M(i, j) = I(i, j) + dt * Cn(i, j);
      // the adjoint of F_hat = M F from that of F' (and Jp'), per material
      const T Jpb = next.Jp.empty() ? T(0) : next.Jp[p];
      Mat<T, D> Fhb = next.F[p];
      out.Jp[p] = Jpb;  // jelly and liquid keep Jp
      const Model model = sim_.model_of(P[p]);
      if (model != Model::kJelly) {
        const Mat<T, D> Fh = mul(M, F);
        if (model == Model::kSnow) {
          out.Jp[p] = T(0);
          Fhb = snow_backward<T, D>(Fh, P[p].Jp, next.F[p], Jpb, mode_, &out.Jp[p]);
        } else {  // liquid: F'_00 = prod of the signed singular values
          Mat<T, D> U, sig, V;
          nclr_svd<T, D>(Fh, U, sig, V, mode_);
          T ps = T(1);
          for (int i = 0; i < D; ++i) ps *= sig(i, i);
          const T dF = det(Fh);
          const T sgn = (dF == T(0)) ? T(0) : ps / dF;  // +1, or -1 where prod s = |det|
          const Mat<T, D> cof = cofactor(Fh);
          for (int i = 0; i < D; ++i)
            for (int j = 0; j < D; ++j) Fhb(i, j) = next.F[p](0, 0) * sgn * cof(i, j);
        }
      }
      out.F[p] = mul(transpose(M), Fhb);
      Mat<T, D> gC = next.C[p];
      const Mat<T, D> gFFt = mul(Fhb, transpose(F));
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) gC(i, j) += dt * gFFt(i, j);
      Vec<T, D> gv;
      for (int d = 0; d < D; ++d) gv[d] = next.v[p][d] + dt * next.x[p][d];
      out.x[p] = next.x[p];
      T Wbar[kS], gfx[D];
      for (int d = 0; d < D; ++d) gfx[d] = T(0);
      for (int o = 0; o < kS; ++o) {
        int oo[3];
        offsets(o, oo);
        const int64_t f = node(s, oo);
        const T W = weight(s, oo);
        const Vec<T, D> &vg = grid[(size_t)f].velocity;
        Vec<T, D> du;
        for (int d = 0; d < D; ++d) du[d] = (T)oo[d] - s.fx[d];
        const Vec<T, D> gCdu = mul(gC, du);
        Vec<T, D> gCtv;
        for (int b = 0; b < D; ++b) {
          T acc = 0;
          for (int a = 0; a < D; ++a) acc += gC(a, b) * vg[a];
          gCtv[b] = acc;
        }
        T wb = 0;
        for (int a = 0; a < D; ++a) {
          VB[(size_t)f][a] += W * gv[a] + cscale * W * gCdu[a];
          wb += gv[a] * vg[a] + cscale * vg[a] * gCdu[a];
        }
        Wbar[o] = wb;
        for (int b = 0; b < D; ++b) gfx[b] -= cscale * W * gCtv[b];
      }
      weight_backward(s, Wbar, gfx);
      for (int d = 0; d < D; ++d) out.x[p][d] += inv_dx * gfx[d];
    }
    // ---- grid reverse ----
    const T allowed = (T)((double)dx * 0.9 / (double)dt);
    std::vector<Vec<T, D>> Gmv(grid.size(), Vec<T, D>::constant(T(0)));
    std::vector<T> Gm(grid.size(), T(0));
    for (size_t f = 0; f < grid.size(); ++f) {
      const T m = grid[f].mass;
      if (!(m > T(0))) continue;
      for (int d = 0; d < D; ++d) {
        const T vd = grid[f].velocity[d];
        if (std::fabs(vd) >= allowed) continue;  // clamped
        const T raw = vd - (d == 1 ? dt * sim_.gravity_ : T(0));
        Gmv[f][d] = VB[f][d] / m;
        Gm[f] -= VB[f][d] * raw / m;
      }
    }
    // ---- P2G reverse ----
    const T Dinv = T(4) * inv_dx * inv_dx;
    for (size_t p = 0; p < n; ++p) {
      const auto &q = P[p];
      const Stencil s = stencil(q.x);
      const auto [mu, lambda] = sim_.hardening(q);
      const Mat<T, D> A = sim_.affine(q);
      Mat<T, D> gA = Mat<T, D>::constant(T(0));
      Vec<T, D> gv = Vec<T, D>::constant(T(0));
      T Wbar[kS], gfx[D];
      for (int d = 0; d < D; ++d) gfx[d] = T(0);
      for (int o = 0; o < kS; ++o) {
        int oo[3];
        offsets(o, oo);
        const int64_t f = node(s, oo);
        const T W = weight(s, oo);
        Vec<T, D> dpos;
        for (int d = 0; d < D; ++d) dpos[d] = ((T)oo[d] - s.fx[d]) * dx;
        const Vec<T, D> Ad = mul(A, dpos);
        const Vec<T, D> &g = Gmv[(size_t)f];
        T wb = Gm[(size_t)f] * q.mass;
        for (int a = 0; a < D; ++a) {
          gv[a] += W * q.mass * g[a];
          wb += g[a] * (q.mass * q.v[a] + Ad[a]);
          for (int b = 0; b < D; ++b) gA(a, b) += W * g[a] * dpos[b];
        }
        Wbar[o] = wb;
        for (int b = 0; b < D; ++b) {
          T acc = 0;
          for (int a = 0; a < D; ++a) acc += A(a, b) * g[a];
          gfx[b] -= dx * W * acc;
        }
      }
      weight_backward(s, Wbar, gfx);
      for (int d = 0; d < D; ++d) out.x[p][d] += inv_dx * gfx[d];
      out.v[p] = gv;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) out.C[p](i, j) = q.mass * gA(i, j);
      // stress: A = -(dt vol Dinv) PF + m C
      const T kappa = dt * q.volume * Dinv;
      Mat<T, D> G;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) G(i, j) = -kappa * gA(i, j);
      const Mat<T, D> &F = q.F;
      const T J = det(F);
      // the hardening factor e of mu = mu_0 e, lambda = lambda_0 e (src/nclr.h:351-372)
      const Model model = sim_.model_of(q);
      const T e = model == Model::kSnow ? (T)std::exp(10.0 * (1.0 - (double)q.Jp))
                                        : (model == Model::kJelly ? T(0.3) : T(1.0));
      const T mu_b = q.mu0 < T(0) ? sim_.mu_0 : q.mu0;          // base moduli
      const T lambda_b = q.mu0 < T(0) ? sim_.lambda_0 : q.lambda0;
      // snow: e = exp(10 (1 - Jp)), de/dJp = -10 e; the adjoint of e is mu_0 mu_bar + ...
      auto harden = [&](T gmu_h, T glambda_h) {
        if (model == Model::kSnow) out.Jp[p] += (gmu_h * mu_b + glambda_h * lambda_b) * T(-10) * e;
      };
      if (sim_.stress_ == Stress::kNeoHookean) {
        const Mat<T, D> FFt = mul(F, transpose(F));
        T trG = 0, gmu = 0;
        for (int i = 0; i < D; ++i) {
          trG += G(i, i);
          for (int j = 0; j < D; ++j) gmu += G(i, j) * (FFt(i, j) - (i == j ? T(1) : T(0)));
        }
        Mat<T, D> S;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) S(i, j) = mu * (G(i, j) + G(j, i));
        const Mat<T, D> SF = mul(S, F);
        const Mat<T, D> cof = cofactor(F);  // J F^-T
        const T c = lambda * trG / J;
        for (int i = 0; i < D; ++i)
          for (int j = 0; j < D; ++j) out.F[p](i, j) += SF(i, j) + c * cof(i, j);
        gmu0 += e * gmu;
        glambda0 += e * (trG * std::log(J));
        if (rows_mu_) (*rows_mu_)[p] += e * gmu;
        if (rows_lambda_) (*rows_lambda_)[p] += e * (trG * std::log(J));
        harden(gmu, trG * std::log(J));
        continue;
      }
      const Mat<T, D> R = nclr_polar_R<T, D>(F, mode_);
      Mat<T, D> X;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) X(i, j) = F(i, j) - R(i, j);
      const Mat<T, D> Q = mul(X, transpose(F));
      T sbar = 0, gmu = 0;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) {
          sbar += G(i, j);
          gmu += T(2) * G(i, j) * Q(i, j);
        }
      const T glambda = sbar * (J - T(1)) * J;
      Mat<T, D> Qbar;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) Qbar(i, j) = T(2) * mu * G(i, j);
      const Mat<T, D> Xbar = mul(Qbar, F);
      const Mat<T, D> FfromQ = mul(transpose(Qbar), X);
      Mat<T, D> Rbar;
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j) Rbar(i, j) = -Xbar(i, j);
      const Mat<T, D> Fpolar = polar_backward<T, D>(F, Rbar, mode_);
      const Mat<T, D> cof = cofactor(F);
      const T dJ = sbar * lambda * (T(2) * J - T(1));
      for (int i = 0; i < D; ++i)
        for (int j = 0; j < D; ++j)
          out.F[p](i, j) += FfromQ(i, j) + Xbar(i, j) + Fpolar(i, j) + dJ * cof(i, j);
      gmu0 += e * gmu;
      glambda0 += e * glambda;
      if (rows_mu_) (*rows_mu_)[p] += e * gmu;
      if (rows_lambda_) (*rows_lambda_)[p] += e * glambda;
      harden(gmu, glambda);
    }
    return out;
  }
};

}  // namespace oracle
