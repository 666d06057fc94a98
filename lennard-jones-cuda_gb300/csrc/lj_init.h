// lj_init.h -- seeded initial conditions (host side).
#pragma once

#include <cstdint>

namespace ljgb {

// Lattice (0 = SC, 1 = FCC) in a box of side L, uniform jitter of half-width
// jitter*sigma, Maxwell velocities at T0 with zero total momentum, rescaled to
// exactly T0.  pos, vel: n x 3 interleaved.  Returns false on bad input.
bool sample_initial_state(int n, double L, double T0, int lattice, double jitter, double sigma, uint64_t seed,
                          double* pos, double* vel);

}  // namespace ljgb
