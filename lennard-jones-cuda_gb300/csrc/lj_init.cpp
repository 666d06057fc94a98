// lj_init.cpp -- seeded initial conditions (host side).
//
// Follows MDSystem::SampleInitialConditions (src/library/MDSystem.cpp:147-181):
// particles on a cell-centred lattice, speeds from the Maxwell distribution by
// the reference's rejection sampler (MaxwellDistributionGenerator,
// MDSystem.cpp:36-53, probmax = 1.2), isotropic directions, zero total
// momentum (CorrectTotalMomentum, :183-216) and an exact rescale to T0
// (RenormalizeVelocities(true), :375-389).  Differences, by design:
//  * the generator is a seeded xoshiro256** stream instead of MTRand seeded
//    from the clock (MersenneTwister.h:242-272), so runs are reproducible;
//  * particles draw in index order (the reference's random_shuffle only
//    permutes the order of draws);
//  * FCC lattice and uniform jitter are offered besides the SC lattice;
//  * storage is FP64.
#include <cmath>
#include <cstdint>

#include "lj_init.h"

namespace ljgb {

namespace {

constexpr double kPi = 3.141592653589793238462643;

struct Xoshiro256 {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  explicit Xoshiro256(uint64_t seed) {
    uint64_t x = seed;
    for (auto& w : s) w = splitmix(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // [0, 1) with 53 random bits
  double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
  // (0, 1): MTRand::randDblExc's open interval
  double uniform_open() {
    double u;
    do u = uniform();
    while (u == 0.0);
    return u;
  }
};

// MaxwellDistributionGenerator::prob (MDSystem.cpp:36-40): density of
// alpha = exp(-u) when u has density ~ u^2 exp(-u^2).
double maxwell_prob(double alpha) {
  const double tlog = -std::log(alpha);
  return tlog * tlog * std::exp(-tlog * tlog) / alpha;
}

}  // namespace

bool sample_initial_state(int n, double L, double T0, int lattice, double jitter, double sigma, uint64_t seed,
                          double* pos, double* vel) {
  if (n < 1 || !(L > 0) || !(T0 >= 0) || !pos || !vel) return false;
  Xoshiro256 rng(seed);
  // Lattice sites, first n in lattice order (x fastest), cell-centred.
  if (lattice == 0) {
    const int ns = (int)std::ceil(std::cbrt((double)n) - 1e-12);
    const int side = (ns * ns * ns < n) ? ns + 1 : ns;
    const double dL = L / side;
    for (int i = 0; i < n; ++i) {
      const int ix = i % side, iy = (i / side) % side, iz = i / (side * side);
      pos[3 * i + 0] = (ix + 0.5) * dL;
      pos[3 * i + 1] = (iy + 0.5) * dL;
      pos[3 * i + 2] = (iz + 0.5) * dL;
    }
  } else {
    int nc = (int)std::ceil(std::cbrt(n / 4.0) - 1e-12);
    while (4 * nc * nc * nc < n) ++nc;
    const double a = L / nc;
    static const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    for (int i = 0; i < n; ++i) {
      const int c = i / 4, b = i % 4;
      const int cx = c % nc, cy = (c / nc) % nc, cz = c / (nc * nc);
      pos[3 * i + 0] = (cx + basis[b][0] + 0.25) * a;
      pos[3 * i + 1] = (cy + basis[b][1] + 0.25) * a;
      pos[3 * i + 2] = (cz + basis[b][2] + 0.25) * a;
    }
  }
  if (jitter > 0) {
    for (int k = 0; k < 3 * n; ++k) pos[k] += (2.0 * rng.uniform() - 1.0) * jitter * sigma;
  }
  // Speeds and directions (MDSystem.cpp:171-177).
  const double probmax = 1.2;
  for (int i = 0; i < n; ++i) {
    double alpha = 0.0;
    while (true) {
      alpha = rng.uniform_open();
      const double eta = rng.uniform() * probmax;
      if (eta < maxwell_prob(alpha)) break;
    }
    const double speed = std::sqrt(2.0 * T0) * (-std::log(alpha));
    const double cth = 2.0 * rng.uniform() - 1.0;
    const double ph = 2.0 * kPi * rng.uniform();
    const double sth = std::sqrt(1.0 - cth * cth);
    vel[3 * i + 0] = speed * sth * std::cos(ph);
    vel[3 * i + 1] = speed * sth * std::sin(ph);
    vel[3 * i + 2] = speed * cth;
  }
  // Zero total momentum (m = 1).
  double P[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) P[c] += vel[3 * i + c];
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) vel[3 * i + c] -= P[c] / n;
  // Exact T0: Tkin = sum v^2 / (3N)  (KineticTemperature, MDSystem.cpp:361-373).
  double s2 = 0;
  for (int k = 0; k < 3 * n; ++k) s2 += vel[k] * vel[k];
  const double Tkin = s2 / 3.0 / n;
  if (Tkin > 0) {
    const double f = std::sqrt(T0 / Tkin);
    for (int k = 0; k < 3 * n; ++k) vel[k] *= f;
  }
  return true;
}

}  // namespace ljgb
