// ljgb/Adjoint.hpp -- C++ forward/backward Function API over the lj_adjoint_*
// C ABI (include/lj_gb300.h): a differentiable trajectory loss of the EVN
// velocity-Verlet dynamics of a periodic Lennard-Jones box.
//
// The reference has no counterpart.  Usage:
//   ljgb::TrajectoryLoss f(cfg, 20);           // checkpoints every 20 steps
//   f.set_weights(0.0, 1.0, 1.0);             // loss = <V/N + P> over the steps
//   double loss = f.forward(0.005, 200);
//   ljgb::TrajectoryLoss::Gradient g = f.backward();
//   // g.epsilon, g.sigma, g.pos (N x 3), g.vel (N x 3)
#pragma once

#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "lj_gb300.h"

namespace ljgb {

class TrajectoryLoss {
 public:
  struct Gradient {
    double epsilon = 0.0;
    double sigma = 0.0;
    std::vector<double> pos;  // dloss / d x_0, N x 3 interleaved
    std::vector<double> vel;  // dloss / d v_0, N x 3 interleaved
  };

  // cfg as for lj_create (periodic, EVN); the initial state is sampled from it.
  explicit TrajectoryLoss(const lj_config& cfg, int checkpoint_every = 20) : n_(cfg.n) {
    const lj_status st = lj_adjoint_create(&cfg, checkpoint_every, &h_);
    if (st != LJ_OK) throw std::runtime_error("lj_adjoint_create failed with status " + std::to_string((int)st));
  }
  ~TrajectoryLoss() { lj_adjoint_destroy(h_); }
  TrajectoryLoss(const TrajectoryLoss&) = delete;
  TrajectoryLoss& operator=(const TrajectoryLoss&) = delete;
  TrajectoryLoss(TrajectoryLoss&& o) noexcept : h_(std::exchange(o.h_, nullptr)), n_(o.n_) {}

  int n() const { return n_; }

  // Initial positions and velocities (N x 3 each).
  void set_state(const std::vector<double>& pos, const std::vector<double>& vel) {
    if ((int)pos.size() != 3 * n_ || (int)vel.size() != 3 * n_) throw std::invalid_argument("state must be N x 3");
    check(lj_adjoint_set_state(h_, pos.data(), vel.data()), "lj_adjoint_set_state");
  }

  // loss = (1/S) sum_m [ w_kinetic K_m/N + w_potential V_m/N + w_pressure P_m ]
  void set_weights(double w_kinetic, double w_potential, double w_pressure) {
    check(lj_adjoint_set_loss(h_, w_kinetic, w_potential, w_pressure), "lj_adjoint_set_loss");
  }

  double forward(double dt, int nsteps) {
    double loss = 0.0;
    check(lj_adjoint_forward(h_, dt, nsteps, &loss), "lj_adjoint_forward");
    return loss;
  }

  Gradient backward() {
    Gradient g;
    g.pos.resize(3 * (size_t)n_);
    g.vel.resize(3 * (size_t)n_);
    check(lj_adjoint_backward(h_, &g.epsilon, &g.sigma, g.pos.data(), g.vel.data()), "lj_adjoint_backward");
    return g;
  }

 private:
  void check(lj_status st, const char* what) const {
    if (st != LJ_OK) throw std::runtime_error(std::string(what) + ": " + lj_adjoint_last_error(h_));
  }
  lj_adjoint* h_ = nullptr;
  int n_ = 0;
};

}  // namespace ljgb
