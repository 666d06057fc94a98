// MDSystem.hpp -- the reference's MDSystem class over the lj_* C ABI.
//
// Same class name, configuration struct, public members and methods as
// vlvovch/lennard-jones-cuda's src/library/MDSystem.h:6-164, so callers (the
// GUI, run-isotherm, run-fluctuations, semiGCEfluctuations) compile against
// it unchanged.  The state lives on the GPU in FP64; the public float arrays
// h_Pos / h_Vel / h_Force are host mirrors.
//
// Differences from the reference, by design:
//  * always the GPU: useCUDA = false / setHardwareMode(false) keep the GPU
//    path (there is no CPU fallback); the flag is stored and reported;
//  * h_Pos / h_Vel / h_Force are refreshed after every Integrate /
//    CalculateForces while hostMirror() is on (default), and on getArray();
//    writes into them reach the device through setArray(type, data)
//    (MDSystem.cpp:615-630), SampleInitialConditions or
//    CorrectTotalMomentum;
//  * NdNdr2 (the r^2 RDF counts) is refreshed by CalculateForces() and RDF();
//    Integrate refreshes it only when setRDFEveryStep(true), since the
//    histogram costs an extra pair pass;
//  * the initial state comes from a seeded generator (config seed), not
//    MTRand seeded from the clock;
//  * Pshear is 0 (the reference's GPU mode never recomputes it).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../lj_gb300.h"
#include "splinefunction.hpp"

class MDSystem {
 public:
  // MDSystem.h:10-41, plus the parameters the reference hard-codes.
  struct MDSystemConfiguration {
    int N;
    double T0;
    double rho;
    bool canonical;
    int boundaryConditions;  // 0 periodic, 1 hard wall, 2 none
    bool useCUDA;
    int CUDABlockSize;
    // extensions
    double epsilon;
    double sigma;
    int lattice;     // LJ_LATTICE_SC (reference) or LJ_LATTICE_FCC
    double jitter;   // sigma units
    uint64_t seed;
    int precision;   // LJ_PREC_MIXED or LJ_PREC_FP64
    int device;

    MDSystemConfiguration()
        : N(128),
          T0(1.5),
          rho(0.2),
          canonical(false),
          boundaryConditions(0),
          useCUDA(false),
          CUDABlockSize(256),
          epsilon(1.0),
          sigma(1.0),
          lattice(LJ_LATTICE_SC),
          jitter(0.0),
          seed(1),
          precision(LJ_PREC_MIXED),
          device(0) {}
  };

  MDSystemConfiguration m_config;

  // Dynamical parameters (MDSystem.h:63-66)
  double U, T, K, V, P;
  double Pshear;

  bool CUDAInit;

  // Host mirrors (float4 per particle, w of h_Pos = L/150 as the reference)
  float* h_Pos;
  float* h_Vel;
  float* h_Force;

  double t;
  double L;

  SplineFunction curvelo;
  int veloIters;

  std::vector<int> NdNdr2;
  float rdf_dr2;

  double momN, momN2, momN3, momN4;
  int momiters;

  double av_U_tot, av_T_tot, av_p_tot;
  int av_iters;

  explicit MDSystem(const MDSystemConfiguration& config = MDSystemConfiguration());
  ~MDSystem();
  MDSystem(const MDSystem&) = delete;
  MDSystem& operator=(const MDSystem&) = delete;

  void Reinitialize(const MDSystemConfiguration& config);
  void ReallocateMemory();
  void SampleInitialConditions();
  void CorrectTotalMomentum();
  void CalculateForces();
  void CalculateForces(float* frc);
  double KineticTemperature(float* vel);
  double CalculateXi(float* frc, float* vel);
  void CalculateParameters();
  void RenormalizeVelocities(bool RecalculateTkin = false);
  void RenormalizeVelocitiesToEnergy(double ust);
  void ApplyBoundaryConditions();
  double getTime() { return t; }
  void Integrate(double dt);

  float* getArray(int type);
  void setArray(int type, const float* data);

  void initvelo(double vmax = 12., double shag = 0.12);
  void updatevelo();
  SplineFunction getvelo();
  double Maxwell(double v);

  void resetAveraging();
  SplineFunction RDF(double rmax = 5., double shag = 0.1);
  void Fluctuations(double fraction);
  int fast_round(float x);

  void setHardwareMode(bool useCUDA);
  void setCanonical(bool canonical);
  void setPeriodicBoundaryCondition(bool periodic) { setBoundaryCondition(!periodic); }
  void setBoundaryCondition(int cond);

  // ---- extensions ----
  // n steps in one call (one graph launch per step, observables read once).
  void Integrate(double dt, int nsteps);
  void setHostMirror(bool on) { m_mirror = on; }
  bool hostMirror() const { return m_mirror; }
  void setRDFEveryStep(bool on) { m_rdf_every_step = on; }
  // Refreshes h_Pos / h_Vel / h_Force from the device.
  void syncHost();
  // The underlying handle (lj_gb300.h) and the status of the last call.
  lj_system* handle() { return m_sys; }
  int lastStatus() const { return m_status; }
  const std::string& lastError() const { return m_error; }

 private:
  lj_system* m_sys = nullptr;
  bool m_mirror = true;
  bool m_rdf_every_step = false;
  int m_status = 0;
  std::string m_error;
  std::vector<double> m_buf, m_buf2, m_buf3;

  bool check(int status);
  void create(const MDSystemConfiguration& config);
  void pullObservables(bool parameters);
  void pullRDF();
  void mirrorFromDevice();
  void fillMirrors();
  void pushArrays(bool pos, bool vel);
};
