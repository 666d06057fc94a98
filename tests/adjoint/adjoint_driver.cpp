// Drives ljgb::TrajectoryLoss (include/ljgb/Adjoint.hpp) as a C++ user would:
// forward, backward, then a central finite difference of the loss along a
// seeded random direction of one particle's initial position, through the
// same API.  Prints key=value lines for the test to parse.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "ljgb/Adjoint.hpp"

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 2048;
  lj_config cfg;
  lj_config_default(&cfg);
  cfg.n = n;
  cfg.density = 0.85;
  cfg.temperature = 1.0;
  cfg.lattice = LJ_LATTICE_FCC;
  cfg.jitter = 0.02;
  cfg.seed = 7;
  try {
    ljgb::TrajectoryLoss f(cfg, 5);
    f.set_weights(0.0, 1.0, 1.0);
    const double dt = 0.005;
    const int steps = 20;
    const double loss = f.forward(dt, steps);
    const ljgb::TrajectoryLoss::Gradient g = f.backward();
    std::vector<double> pos(3 * (size_t)n), vel(3 * (size_t)n), dir(3 * (size_t)n);
    if (lj_sample_initial_state(&cfg, pos.data(), vel.data()) != LJ_OK) return 2;
    std::mt19937_64 rng(11);
    std::normal_distribution<double> nd;
    const size_t p = rng() % (size_t)n;
    double adj = 0.0;
    for (size_t c = 0; c < 3; ++c) {
      dir[3 * p + c] = nd(rng);
      adj += dir[3 * p + c] * g.pos[3 * p + c];
    }
    const double h = 1e-6;
    std::vector<double> p1 = pos, p2 = pos;
    for (size_t k = 0; k < dir.size(); ++k) {
      p1[k] += h * dir[k];
      p2[k] -= h * dir[k];
    }
    f.set_state(p1, vel);
    const double l1 = f.forward(dt, steps);
    f.set_state(p2, vel);
    const double l2 = f.forward(dt, steps);
    std::printf("adjoint loss=%.17g deps=%.17g dsigma=%.17g dpos0=%.17g dvel0=%.17g\n", loss, g.epsilon, g.sigma,
                g.pos[0], g.vel[0]);
    std::printf("direction adj=%.17g fd=%.17g\n", adj, (l1 - l2) / (2 * h));
  } catch (const std::exception& e) {
    std::printf("error %s\n", e.what());
    return 1;
  }
  return 0;
}
