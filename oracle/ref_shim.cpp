// ref_shim.cpp -- C entry points around the reference's own CPU MDSystem.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh against the
// reference sources where they lie (src/library/MDSystem.cpp,
// src/library/splinefunction.cpp of vlvovch/lennard-jones-cuda, built without
// USE_CUDA_TOOLKIT so the CUDA entry points are the CPU stubs of
// MDSystem.cpp:26-34) into oracle/_ref/libmdsystem_ref.so.  Used to pin the
// oracle restatement and to generate the golden fixtures; the product never
// loads it.
//
// State injection follows the reference's public members: h_Pos/h_Vel are
// overwritten after construction (MDSystem.h:72-73), then CalculateForces /
// CalculateParameters / Integrate are called exactly as callers do.
#include <cstring>

#include "MDSystem.h"

extern "C" {

void* ref_create(int N, double T0, double rho, int canonical, int bc) {
  MDSystem::MDSystemConfiguration c;
  c.N = N;
  c.T0 = T0;
  c.rho = rho;
  c.canonical = canonical != 0;
  c.boundaryConditions = bc;
  c.useCUDA = false;
  return new MDSystem(c);
}

void ref_destroy(void* h) { delete static_cast<MDSystem*>(h); }

void ref_set_state(void* h, const float* pos4, const float* vel4) {
  MDSystem* s = static_cast<MDSystem*>(h);
  std::memcpy(s->h_Pos, pos4, sizeof(float) * 4 * s->m_config.N);
  std::memcpy(s->h_Vel, vel4, sizeof(float) * 4 * s->m_config.N);
}

void ref_set_forces(void* h, const float* frc4) {
  MDSystem* s = static_cast<MDSystem*>(h);
  std::memcpy(s->h_Force, frc4, sizeof(float) * 4 * s->m_config.N);
}

void ref_calculate_forces(void* h) { static_cast<MDSystem*>(h)->CalculateForces(); }

void ref_calculate_parameters(void* h) { static_cast<MDSystem*>(h)->CalculateParameters(); }

void ref_integrate(void* h, double dt, int nsteps) {
  MDSystem* s = static_cast<MDSystem*>(h);
  for (int k = 0; k < nsteps; ++k) s->Integrate(dt);
}

void ref_renormalize(void* h, int recalc) {
  static_cast<MDSystem*>(h)->RenormalizeVelocities(recalc != 0);
}

void ref_renormalize_to_energy(void* h, double ust) {
  static_cast<MDSystem*>(h)->RenormalizeVelocitiesToEnergy(ust);
}

void ref_reset_averaging(void* h) { static_cast<MDSystem*>(h)->resetAveraging(); }

void ref_set_canonical(void* h, int c) { static_cast<MDSystem*>(h)->setCanonical(c != 0); }

void ref_set_bc(void* h, int bc) { static_cast<MDSystem*>(h)->setBoundaryCondition(bc); }

void ref_set_time(void* h, double t) { static_cast<MDSystem*>(h)->t = t; }

// scalars: U T K V P Pshear t L av_U av_T av_p av_iters rdf_dr2
void ref_get(void* h, float* pos4, float* vel4, float* frc4, double* scalars, int* rdf256) {
  MDSystem* s = static_cast<MDSystem*>(h);
  const int n = s->m_config.N;
  if (pos4) std::memcpy(pos4, s->h_Pos, sizeof(float) * 4 * n);
  if (vel4) std::memcpy(vel4, s->h_Vel, sizeof(float) * 4 * n);
  if (frc4) std::memcpy(frc4, s->h_Force, sizeof(float) * 4 * n);
  if (scalars) {
    double v[13] = {s->U,        s->T,        s->K,        s->V,        s->P,
                    s->Pshear,   s->t,        s->L,        s->av_U_tot, s->av_T_tot,
                    s->av_p_tot, (double)s->av_iters, (double)s->rdf_dr2};
    std::memcpy(scalars, v, sizeof(v));
  }
  if (rdf256)
    for (int b = 0; b < 256; ++b) rdf256[b] = s->NdNdr2[b];
}

// RDF() spline (MDSystem.cpp:633-649): 256 (r, g) pairs.
void ref_rdf(void* h, double* x, double* y) {
  SplineFunction f = static_cast<MDSystem*>(h)->RDF();
  for (size_t k = 0; k < f.vals.size() && k < 256; ++k) {
    x[k] = f.vals[k].first;
    y[k] = f.vals[k].second;
  }
}

void ref_initvelo(void* h, double vmax, double step) { static_cast<MDSystem*>(h)->initvelo(vmax, step); }

void ref_updatevelo(void* h) { static_cast<MDSystem*>(h)->updatevelo(); }

// getvelo() spline: returns the number of points written (at most cap).
int ref_getvelo(void* h, double* x, double* y, int cap) {
  SplineFunction f = static_cast<MDSystem*>(h)->getvelo();
  int n = 0;
  for (; n < (int)f.vals.size() && n < cap; ++n) {
    x[n] = f.vals[n].first;
    y[n] = f.vals[n].second;
  }
  return n;
}

double ref_maxwell(void* h, double v) { return static_cast<MDSystem*>(h)->Maxwell(v); }

}  // extern "C"
