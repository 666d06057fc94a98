// MDSystem.cpp -- the reference's MDSystem class (src/library/MDSystem.h) as
// a facade over the lj_* C ABI.  Every method cites the reference method it
// stands in for; the physics runs in the sm_103a kernels behind lj_*.
#include "ljgb/MDSystem.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>

namespace {
constexpr double kPi = 3.141592653589793238462643;
}

bool MDSystem::check(int status) {
  m_status = status;
  if (status != LJ_OK) {
    m_error = lj_last_error(m_sys);
    std::fprintf(stderr, "MDSystem (lj_gb300): %s\n", m_error.c_str());
    return false;
  }
  return true;
}

void MDSystem::create(const MDSystemConfiguration& c) {
  m_config = c;
  lj_config lc;
  lj_config_default(&lc);
  lc.n = c.N;
  lc.temperature = c.T0;
  lc.density = c.rho;
  lc.canonical = c.canonical ? 1 : 0;
  lc.boundary = c.boundaryConditions;
  lc.precision = c.precision;
  lc.epsilon = c.epsilon;
  lc.sigma = c.sigma;
  lc.lattice = c.lattice;
  lc.jitter = c.jitter;
  lc.seed = c.seed;
  lc.block_hint = 0;
  lc.device = c.device;
  if (m_sys) {
    check(lj_reinitialize(m_sys, &lc));
  } else {
    m_status = lj_create(&lc, &m_sys);
    if (m_status != LJ_OK) {
      m_error = lj_last_error(nullptr);
      std::fprintf(stderr, "MDSystem (lj_gb300): %s\n", m_error.c_str());
      m_sys = nullptr;
    }
  }
  CUDAInit = m_sys != nullptr;
}

// MDSystem::MDSystem (MDSystem.cpp:55-64)
MDSystem::MDSystem(const MDSystemConfiguration& config)
    : U(0), T(0), K(0), V(0), P(0), Pshear(0), CUDAInit(false), h_Pos(nullptr), h_Vel(nullptr), h_Force(nullptr),
      t(0), L(0), veloIters(0), rdf_dr2(0), momN(0), momN2(0), momN3(0), momN4(0), momiters(0), av_U_tot(0),
      av_T_tot(0), av_p_tot(0), av_iters(0) {
  Reinitialize(config);
}

// MDSystem::~MDSystem (MDSystem.cpp:218-230)
MDSystem::~MDSystem() {
  delete[] h_Pos;
  delete[] h_Vel;
  delete[] h_Force;
  if (m_sys) lj_destroy(m_sys);
}

// MDSystem::Reinitialize (MDSystem.cpp:66-114): box, initial state, RDF bin
// width, forces, parameters, velocity histogram, averages reset.
void MDSystem::Reinitialize(const MDSystemConfiguration& config) {
  create(config);
  const int N = m_config.N;
  L = std::cbrt(N / m_config.rho);
  T = m_config.T0;
  t = 0;
  delete[] h_Pos;
  delete[] h_Vel;
  delete[] h_Force;
  h_Pos = new float[4 * (size_t)N]();
  h_Vel = new float[4 * (size_t)N]();
  h_Force = new float[4 * (size_t)N]();
  rdf_dr2 = lj_reference_rdf_dr2(N);
  NdNdr2.assign(256, 0);
  if (!m_sys) return;
  // lj_create already sampled the state and evaluated forces/observables.
  pullObservables(false);
  P = 0;
  {
    lj_observables o;
    if (check(lj_get_observables(m_sys, &o))) P = o.W / 6.0;
  }
  CalculateParameters();
  mirrorFromDevice();
  pullRDF();
  veloIters = 0;
  initvelo();
  momN = momN2 = momN3 = momN4 = 0.;
  momiters = 0;
  av_U_tot = av_T_tot = av_p_tot = 0.;
  av_iters = 0;
}

// MDSystem::ReallocateMemory (MDSystem.cpp:116-144): device memory is owned
// by the handle and sized at creation; this re-uploads the host mirrors.
void MDSystem::ReallocateMemory() {
  if (m_sys) pushArrays(true, true);
}

// MDSystem::SampleInitialConditions (MDSystem.cpp:147-181) with the seeded
// generator of lj_sample_initial_state.
void MDSystem::SampleInitialConditions() {
  if (!m_sys) return;
  lj_config lc;
  lj_config_default(&lc);
  lc.n = m_config.N;
  lc.temperature = m_config.T0;
  lc.density = m_config.rho;
  lc.lattice = m_config.lattice;
  lc.jitter = m_config.jitter;
  lc.sigma = m_config.sigma;
  lc.seed = m_config.seed;
  m_buf.resize(3 * (size_t)m_config.N);
  m_buf2.resize(3 * (size_t)m_config.N);
  if (!check(lj_sample_initial_state(&lc, m_buf.data(), m_buf2.data()))) return;
  check(lj_set_state(m_sys, m_buf.data(), m_buf2.data()));
  mirrorFromDevice();
}

// MDSystem::CorrectTotalMomentum (MDSystem.cpp:183-216) on the device state.
void MDSystem::CorrectTotalMomentum() {
  if (!m_sys) return;
  const int N = m_config.N;
  m_buf.resize(3 * (size_t)N);
  if (!check(lj_get_state(m_sys, nullptr, m_buf.data(), nullptr))) return;
  double p[3] = {0, 0, 0};
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 3; ++c) p[c] += m_buf[3 * (size_t)i + c];
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 3; ++c) m_buf[3 * (size_t)i + c] -= p[c] / N;
  check(lj_set_state(m_sys, nullptr, m_buf.data()));
  mirrorFromDevice();
}

void MDSystem::CalculateForces() { CalculateForces(h_Force); }

// MDSystem::CalculateForces (MDSystem.cpp:232-311): forces at the current
// positions, V, the virial part of P, and the r^2 RDF counts.
void MDSystem::CalculateForces(float* frc) {
  if (!m_sys) return;
  if (!check(lj_compute_forces(m_sys))) return;
  lj_observables o;
  if (!check(lj_get_observables(m_sys, &o))) return;
  V = o.V;
  P = o.W / 6.0;
  Pshear = 0.0;
  pullRDF();
  m_buf3.resize(3 * (size_t)m_config.N);
  std::vector<double> e(m_config.N);
  if (check(lj_get_state(m_sys, nullptr, nullptr, m_buf3.data())) && check(lj_get_pair_sums(m_sys, e.data(), nullptr)) &&
      frc) {
    for (int i = 0; i < m_config.N; ++i) {
      for (int c = 0; c < 3; ++c) frc[4 * (size_t)i + c] = (float)m_buf3[3 * (size_t)i + c];
      // Force.w of the GPU path: sum_j (r^-12 - r^-6) = e_i / (4 eps)
      frc[4 * (size_t)i + 3] = (float)(e[i] / (4.0 * m_config.epsilon));
    }
  }
}

// MDSystem::KineticTemperature (MDSystem.cpp:361-373), on a caller array.
double MDSystem::KineticTemperature(float* vel) {
  double r = 0.;
  for (int i = 0; i < 4 * m_config.N; i += 4) r += vel[i] * vel[i] + vel[i + 1] * vel[i + 1] + vel[i + 2] * vel[i + 2];
  return r / 3. / m_config.N;
}

// MDSystem::CalculateXi (MDSystem.cpp:313-323), on caller arrays.
double MDSystem::CalculateXi(float* frc, float* vel) {
  double num = 0., den = 0.;
  for (int i = 0; i < 4 * m_config.N; i += 4) {
    num += vel[i] * frc[i] + vel[i + 1] * frc[i + 1] + vel[i + 2] * frc[i + 2];
    den += vel[i] * vel[i] + vel[i + 1] * vel[i + 1] + vel[i + 2] * vel[i + 2];
  }
  return num / den;
}

// MDSystem::CalculateParameters (MDSystem.cpp:325-359): K from the device,
// then T, P (+= N T, / volume), U and the running averages, on the members.
void MDSystem::CalculateParameters() {
  const int N = m_config.N;
  if (m_sys) {
    lj_observables o;
    if (check(lj_get_observables(m_sys, &o))) {
      K = o.K;
      V = o.V;
    }
  }
  T = 2. * K / 3. / N;
  P += N * T;
  P /= (N / m_config.rho);
  U = K + V;
  Pshear /= (N / m_config.rho);
  av_iters++;
  av_U_tot += U;
  av_p_tot += P;
  av_T_tot += T;
}

// MDSystem::RenormalizeVelocities (MDSystem.cpp:375-389)
void MDSystem::RenormalizeVelocities(bool recalc) {
  if (!m_sys) return;
  if (!recalc) {
    // The device uses its last observable T; keep the facade's T in step.
    lj_observables o;
    if (check(lj_get_observables(m_sys, &o)) && o.T != T) {
      const double Tkin = T;
      const double f = std::sqrt(m_config.T0 / Tkin);
      m_buf.resize(3 * (size_t)m_config.N);
      if (!check(lj_get_state(m_sys, nullptr, m_buf.data(), nullptr))) return;
      for (auto& x : m_buf) x *= f;
      check(lj_set_state(m_sys, nullptr, m_buf.data()));
      K *= m_config.T0 / Tkin;
      T = m_config.T0;
      U = K + V;
      mirrorFromDevice();
      return;
    }
  }
  if (!check(lj_renormalize_velocities(m_sys, recalc ? 1 : 0))) return;
  lj_observables o;
  if (check(lj_get_observables(m_sys, &o))) {
    K = o.K;
    T = o.T;
    U = K + V;
  }
  mirrorFromDevice();
}

// MDSystem::RenormalizeVelocitiesToEnergy (MDSystem.cpp:391-404)
void MDSystem::RenormalizeVelocitiesToEnergy(double ust) {
  if (!m_sys) return;
  if (!check(lj_renormalize_velocities_to_energy(m_sys, ust))) return;
  K = ust * m_config.N - V;
  U = K + V;
  mirrorFromDevice();
}

// MDSystem::ApplyBoundaryConditions (MDSystem.cpp:406-436) on the device state.
void MDSystem::ApplyBoundaryConditions() {
  if (!m_sys || m_config.boundaryConditions == 2) return;
  const int N = m_config.N;
  m_buf.resize(3 * (size_t)N);
  m_buf2.resize(3 * (size_t)N);
  if (!check(lj_get_state(m_sys, m_buf.data(), m_buf2.data(), nullptr))) return;
  for (size_t k = 0; k < m_buf.size(); ++k) {
    if (m_config.boundaryConditions == 0) {
      if (m_buf[k] < 0.) m_buf[k] += L;
      if (m_buf[k] > L) m_buf[k] -= L;
    } else {
      if (m_buf[k] < 0. && m_buf2[k] < 0) m_buf2[k] = -m_buf2[k];
      if (m_buf[k] > L && m_buf2[k] > 0) m_buf2[k] = -m_buf2[k];
    }
  }
  check(lj_set_state(m_sys, m_buf.data(), m_buf2.data()));
  mirrorFromDevice();
}

// MDSystem::Integrate (MDSystem.cpp:438-583)
void MDSystem::Integrate(double dt) { Integrate(dt, 1); }

void MDSystem::Integrate(double dt, int nsteps) {
  if (!m_sys || nsteps < 1) return;
  // The device advances its own running sums every step; the facade's
  // averages (CalculateParameters, MDSystem.cpp:355-358) take the increments.
  lj_observables o0, o1;
  if (!check(lj_get_observables(m_sys, &o0))) return;
  if (!check(lj_step(m_sys, dt, nsteps))) return;
  // With host mirrors on, the state and the observables come back together.
  const bool mirrored = m_mirror && h_Pos;
  if (mirrored) {
    const int N = m_config.N;
    m_buf.resize(3 * (size_t)N);
    m_buf2.resize(3 * (size_t)N);
    m_buf3.resize(3 * (size_t)N);
    if (!check(lj_get_state_observables(m_sys, m_buf.data(), m_buf2.data(), m_buf3.data(), &o1))) return;
    fillMirrors();
  } else if (!check(lj_get_observables(m_sys, &o1))) {
    return;
  }
  K = o1.K;
  V = o1.V;
  T = o1.T;
  P = o1.P;
  U = o1.U;
  t = o1.t;
  Pshear = 0.0;
  av_iters += (int)(o1.av_iters - o0.av_iters);
  av_U_tot += o1.av_U_tot - o0.av_U_tot;
  av_p_tot += o1.av_p_tot - o0.av_p_tot;
  av_T_tot += o1.av_T_tot - o0.av_T_tot;
  if (m_rdf_every_step) pullRDF();
}

// MDSystem::getArray (MDSystem.cpp:586-613)
float* MDSystem::getArray(int type) {
  mirrorFromDevice();
  return type == 1 ? h_Vel : h_Pos;
}

// MDSystem::setArray (MDSystem.cpp:615-630): uploads float4 data as the
// device state of positions (0) or velocities (1).
void MDSystem::setArray(int type, const float* data) {
  if (!m_sys || !data) return;
  const int N = m_config.N;
  m_buf.resize(3 * (size_t)N);
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 3; ++c) m_buf[3 * (size_t)i + c] = data[4 * (size_t)i + c];
  if (type == 1) check(lj_set_state(m_sys, nullptr, m_buf.data()));
  else check(lj_set_state(m_sys, m_buf.data(), nullptr));
}

// MDSystem::initvelo (MDSystem.cpp:651-669)
void MDSystem::initvelo(double vmax, double step) {
  const int N = m_config.N;
  const int maxind = (int)(vmax / step) + 1;
  std::vector<uint64_t> dens(maxind, 0);
  if (m_sys) check(lj_velocity_counts(m_sys, step, maxind, dens.data()));
  curvelo = SplineFunction();
  for (int i = 0; i < maxind; ++i) curvelo.add_val(step * (0.5 + i), dens[i] / step / N);
  veloIters = 1;
}

SplineFunction MDSystem::getvelo() { return curvelo; }

// MDSystem::updatevelo (MDSystem.cpp:676-694): running mean of the histogram.
void MDSystem::updatevelo() {
  const int N = m_config.N;
  const int maxind = (int)curvelo.vals.size();
  if (maxind < 2) return;
  const double shag = curvelo.vals[1].first - curvelo.vals[0].first;
  std::vector<uint64_t> dens(maxind, 0);
  if (m_sys) check(lj_velocity_counts(m_sys, shag, maxind, dens.data()));
  for (int i = 0; i < maxind; ++i)
    curvelo.vals[i].second = (curvelo.vals[i].second * veloIters + dens[i] / shag / N) / (veloIters + 1);
  veloIters++;
}

// MDSystem::Maxwell (MDSystem.cpp:696-699)
double MDSystem::Maxwell(double v) {
  return 4 * kPi * std::pow(1. / 2. / kPi / T, 3. / 2.) * v * v * std::exp(-v * v / 2. / T);
}

// MDSystem::resetAveraging (MDSystem.cpp:701-705)
void MDSystem::resetAveraging() {
  av_U_tot = av_T_tot = av_p_tot = 0.;
  av_iters = 0;
  if (m_sys) check(lj_reset_averaging(m_sys));
}

// MDSystem::RDF (MDSystem.cpp:633-649): arguments ignored as in the
// reference; g(r_k) = C_k / (dr2 2 pi r_k n0 N) at r_k = sqrt((k+1/2) dr2).
SplineFunction MDSystem::RDF(double rmax, double shag) {
  (void)rmax;
  (void)shag;
  pullRDF();
  const int N = m_config.N;
  const double n0 = N / L / L / L;
  std::vector<double> x, y;
  for (size_t k = 0; k < NdNdr2.size(); ++k) {
    const double r2 = (k + 0.5) * rdf_dr2;
    const double r = std::sqrt(r2);
    x.push_back(r);
    y.push_back(NdNdr2[k] / rdf_dr2 / 2. / kPi / r / n0 / static_cast<double>(N));
  }
  return SplineFunction(x, y);
}

// MDSystem::Fluctuations (MDSystem.cpp:707-730): particles in the central
// sub-cube of volume fraction `fraction`, running moments, printed.
void MDSystem::Fluctuations(double fraction) {
  mirrorFromDevice();
  const int N = m_config.N;
  const double tsz = L * std::pow(fraction, 1. / 3.);
  long long tN = 0;
  for (int i = 0; i < 4 * N; i += 4) {
    bool in = true;
    for (int c = 0; c < 3; ++c) in = in && h_Pos[i + c] >= 0.5 * L - 0.5 * tsz && h_Pos[i + c] <= 0.5 * L + 0.5 * tsz;
    if (in) tN++;
  }
  momN += tN;
  momN2 += (double)tN * tN;
  momN3 += (double)tN * tN * tN;
  momN4 += (double)tN * tN * tN * tN;
  momiters++;
  const double mean = momN / momiters;
  const double ev = (1. - 2. * kPi / 3. * N / L / L / L);
  std::cout << "Iteration: " << momiters << "\t<N> = " << mean << "\tw[N] = " << (momN2 / momiters - mean * mean) / mean
            << "\tEV: " << ev * ev << "\tBinom: " << 1. - fraction << "\n";
}

// MDSystem::fast_round (MDSystem.cpp:732-739)
int MDSystem::fast_round(float x) { return x > 0 ? static_cast<int>(x + 0.5f) : static_cast<int>(x - 0.5f); }

// MDSystem::setHardwareMode (MDSystem.cpp:741-745): the GPU path is the only
// path; the flag is stored for callers that read it back.
void MDSystem::setHardwareMode(bool useCUDA) { m_config.useCUDA = useCUDA; }

void MDSystem::setCanonical(bool canonical) {
  m_config.canonical = canonical;
  if (m_sys) check(lj_set_canonical(m_sys, canonical ? 1 : 0));
}

void MDSystem::setBoundaryCondition(int cond) {
  m_config.boundaryConditions = cond;
  if (m_sys) check(lj_set_boundary(m_sys, cond));
}

void MDSystem::syncHost() { mirrorFromDevice(); }

// ---- private -----------------------------------------------------------

// After a device step: the device computed CalculateParameters' K, V, T, P, U;
// the facade's running averages advance like CalculateParameters does.
void MDSystem::pullObservables(bool parameters) {
  lj_observables o;
  if (!check(lj_get_observables(m_sys, &o))) return;
  K = o.K;
  V = o.V;
  t = o.t;
  if (parameters) {
    T = o.T;
    P = o.P;
    U = o.U;
    Pshear = 0.0;
    av_iters++;
    av_U_tot += U;
    av_p_tot += P;
    av_T_tot += T;
  }
}

void MDSystem::pullRDF() {
  if (!m_sys) return;
  std::vector<uint64_t> c(256);
  if (!check(lj_rdf_counts(m_sys, LJ_RDF_R2_CLAMP, 256, rdf_dr2, c.data()))) return;
  NdNdr2.resize(256);
  for (int b = 0; b < 256; ++b) NdNdr2[b] = (int)c[b];
}

void MDSystem::mirrorFromDevice() {
  if (!m_sys || !h_Pos) return;
  const int N = m_config.N;
  m_buf.resize(3 * (size_t)N);
  m_buf2.resize(3 * (size_t)N);
  m_buf3.resize(3 * (size_t)N);
  if (!check(lj_get_state(m_sys, m_buf.data(), m_buf2.data(), m_buf3.data()))) return;
  fillMirrors();
}

// h_Pos / h_Vel / h_Force from the FP64 buffers last read from the device.
void MDSystem::fillMirrors() {
  const int N = m_config.N;
  const float w = (float)(L / 150.f);
  for (int i = 0; i < N; ++i) {
    for (int c = 0; c < 3; ++c) {
      h_Pos[4 * (size_t)i + c] = (float)m_buf[3 * (size_t)i + c];
      h_Vel[4 * (size_t)i + c] = (float)m_buf2[3 * (size_t)i + c];
      h_Force[4 * (size_t)i + c] = (float)m_buf3[3 * (size_t)i + c];
    }
    h_Pos[4 * (size_t)i + 3] = w;
  }
}

void MDSystem::pushArrays(bool pos, bool vel) {
  const int N = m_config.N;
  m_buf.resize(3 * (size_t)N);
  m_buf2.resize(3 * (size_t)N);
  for (int i = 0; i < N; ++i)
    for (int c = 0; c < 3; ++c) {
      m_buf[3 * (size_t)i + c] = h_Pos[4 * (size_t)i + c];
      m_buf2[3 * (size_t)i + c] = h_Vel[4 * (size_t)i + c];
    }
  check(lj_set_state(m_sys, pos ? m_buf.data() : nullptr, vel ? m_buf2.data() : nullptr));
}
