/*
 * lj_oracle.c -- CPU oracle for the Lennard-Jones MD hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, loads or
 * calls this file; only the tests, the package smoke check and the bench's
 * CPU-baseline leg do, and there only as the checker (or as the timed CPU
 * baseline), never as the thing that is measured or shipped.
 *
 * Two restatements of vlvovch/lennard-jones-cuda live here:
 *
 *   r32_*  A faithful restatement of the reference CPU path in
 *          src/library/MDSystem.cpp, reproducing its float storage of
 *          positions, velocities and forces and its double temporaries
 *          operation by operation.  Built with -ffp-contract=off it is
 *          bit-identical to the reference compiled from its own sources
 *          (pinned by the golden fixtures under tests/golden/).  With
 *          nthreads > 1 the i-loop is split over OpenMP threads; forces stay
 *          bit-identical, the scalar sums (V, P, Pshear) and the RDF are then
 *          combined per thread and differ from the serial order in the last
 *          bits only.  This is the CPU baseline ("port").
 *
 *   f64_*  A true-FP64 restatement of the same formulas (double storage
 *          everywhere, explicit epsilon and sigma) -- the accuracy oracle the
 *          mixed-precision GPU path is gated against.
 *
 *   emu_*  Bit-exact emulation of the integer/histogram decisions the device
 *          makes (fixed-point positions, FP32 r^2 bins, FP64 speed bins), so
 *          histogram counts can be compared exactly.
 *
 *   init_* The seeded initial state of the benchmark workloads (lattice,
 *          jitter, Maxwell speeds by the reference's rejection sampler
 *          MDSystem.cpp:36-53 and :147-181, zero momentum :183-216, exact T0
 *          :375-389, drawn from a xoshiro256** stream), so the CPU baseline
 *          starts from the same state as the GPU arm without loading the
 *          product library.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_PI 3.141592653589793238462643

/* ------------------------------------------------------------------------ */
/* Part 1: faithful float-storage restatement of MDSystem.cpp (CPU mode).    */
/* ------------------------------------------------------------------------ */

/* Mirrors the public state of class MDSystem (MDSystem.h:43-99) that the CPU
 * path reads and writes.  pos/vel/frc are caller-owned float[4N] arrays laid
 * out like h_Pos/h_Vel/h_Force (x, y, z, w per particle). */
typedef struct {
  int N;
  double T0, rho;
  int canonical;
  int bc; /* 0 periodic, 1 hard wall, 2 none (MDSystem.h:24) */
  double L, t;
  double U, T, K, V, P, Pshear;
  double av_U_tot, av_T_tot, av_p_tot;
  int av_iters;
  float rdf_dr2;
  int rdf[256];
  float *pos, *vel, *frc;
} r32_state;

/* MDSystem::fast_round, MDSystem.cpp:732-739 (float argument, half away from 0). */
static int r32_fast_round(float x) {
  if (x > 0) return (int)(x + 0.5f);
  return (int)(x - 0.5f);
}

/* Reinitialize's RDF bin width, MDSystem.cpp:93-95 (stored in a float member). */
float r32_rdf_dr2(int N) {
  double a = 0.2 * sqrt(100. / N);
  float dr2 = (float)(a > 0.05 ? a : 0.05);
  if (250 * dr2 < 25.0) dr2 = (float)(25.0 / 250);
  return dr2;
}

/* Inner j-loop of MDSystem::CalculateForces(float*) for one i (MDSystem.cpp:262-305).
 * V, P, Ps are running sums carried across i exactly like the reference's members. */
static void r32_force_row(const r32_state* s, float* frc, int i, double* V, double* P, double* Ps,
                          int* rdf) {
  const float* h_Pos = s->pos;
  const int N4 = 4 * s->N;
  const double L = s->L;
  double r2, r6;
  frc[i] = 0.;
  frc[i + 1] = 0.;
  frc[i + 2] = 0.;
  for (int j = 0; j < N4; j += 4) {
    if (j == i) continue;
    float rx = h_Pos[i] - h_Pos[j];
    float ry = h_Pos[i + 1] - h_Pos[j + 1];
    float rz = h_Pos[i + 2] - h_Pos[j + 2];
    if (s->bc == 0) {
      /* rx / L is a double division, fast_round takes it back as float (:274-276). */
      rx = (float)((double)rx - L * (double)r32_fast_round((float)((double)rx / L)));
      ry = (float)((double)ry - L * (double)r32_fast_round((float)((double)ry / L)));
      rz = (float)((double)rz - L * (double)r32_fast_round((float)((double)rz / L)));
    }
    /* float products and sum, then widened (:279) */
    r2 = (double)(rx * rx + ry * ry + rz * rz);
    {
      double q = floor(r2 / (double)s->rdf_dr2); /* :282-284, overflow bins dropped */
      if (q < 256.0) rdf[(int)q]++;
    }
    r2 = 1 / r2;
    r6 = r2 * r2 * r2;
    double fijx = r2 * (12 * r6 * r6 - 6 * r6) * (double)rx;
    double fijy = r2 * (12 * r6 * r6 - 6 * r6) * (double)ry;
    double fijz = r2 * (12 * r6 * r6 - 6 * r6) * (double)rz;
    frc[i] = (float)((double)frc[i] + fijx);
    frc[i + 1] = (float)((double)frc[i + 1] + fijy);
    frc[i + 2] = (float)((double)frc[i + 2] + fijz);
    *V += (1 * r6 * r6 - 1 * r6);
    *P += (double)rx * fijx + (double)ry * fijy + (double)rz * fijz;
    *Ps += (double)(-rx) * fijy;
  }
  frc[i] *= 4;
  frc[i + 1] *= 4;
  frc[i + 2] *= 4;
}

/* The same j-loop for rows [i0, i1) only, split over nthreads OpenMP threads:
 * a bounded sample of one force evaluation ((i1 - i0)(N - 1) ordered pairs)
 * for timing.  Writes those rows of frc; returns sum_i V_i of the rows. */
double r32_force_rows(const r32_state* s, float* frc, int i0, int i1, int nthreads) {
  double Vsum = 0.;
  int nt = nthreads > 1 ? nthreads : 1;
#pragma omp parallel for num_threads(nt) schedule(static) reduction(+ : Vsum)
  for (int p = i0; p < i1; ++p) {
    double V = 0., P = 0., Ps = 0.;
    int hist[256] = {0};
    r32_force_row(s, frc, 4 * p, &V, &P, &Ps, hist);
    Vsum += V;
  }
  return Vsum;
}

/* MDSystem::CalculateForces(float*), CPU branch (MDSystem.cpp:252-310). */
void r32_calculate_forces(r32_state* s, float* frc, int nthreads) {
  const int N = s->N;
  memset(s->rdf, 0, sizeof(s->rdf));
  s->V = 0.;
  s->P = 0.;
  s->Pshear = 0.;
  if (nthreads <= 1) {
    double V = 0., P = 0., Ps = 0.;
    for (int i = 0; i < 4 * N; i += 4) r32_force_row(s, frc, i, &V, &P, &Ps, s->rdf);
    s->V = V;
    s->P = P;
    s->Pshear = Ps;
  } else {
    /* Contiguous i-chunks per thread, partial sums combined in chunk order. */
    int nt = nthreads;
    double* part = (double*)calloc((size_t)nt * 3, sizeof(double));
    int* hist = (int*)calloc((size_t)nt * 256, sizeof(int));
#pragma omp parallel for num_threads(nt) schedule(static, 1)
    for (int c = 0; c < nt; ++c) {
      int lo = (int)((long long)N * c / nt), hi = (int)((long long)N * (c + 1) / nt);
      double V = 0., P = 0., Ps = 0.;
      for (int p = lo; p < hi; ++p) r32_force_row(s, frc, 4 * p, &V, &P, &Ps, hist + 256 * c);
      part[3 * c] = V;
      part[3 * c + 1] = P;
      part[3 * c + 2] = Ps;
    }
    double V = 0., P = 0., Ps = 0.;
    for (int c = 0; c < nt; ++c) {
      V += part[3 * c];
      P += part[3 * c + 1];
      Ps += part[3 * c + 2];
      for (int b = 0; b < 256; ++b) s->rdf[b] += hist[256 * c + b];
    }
    s->V = V;
    s->P = P;
    s->Pshear = Ps;
    free(part);
    free(hist);
  }
  s->P *= 4. / 3. / 2.;
  s->V *= 4. / 2.;
  s->Pshear *= 4. / 2.;
}

/* MDSystem::CalculateParameters, CPU branch (MDSystem.cpp:325-359). */
void r32_calculate_parameters(r32_state* s) {
  const int N = s->N;
  const float* v = s->vel;
  s->K = 0.;
  for (int i = 0; i < 4 * N; i += 4) {
    s->K += (double)(v[i] * v[i] + v[i + 1] * v[i + 1] + v[i + 2] * v[i + 2]) / 2.;
    s->Pshear += (double)(-v[i] * v[i + 1]);
  }
  s->T = 2. * s->K / 3. / N;
  s->P += N * s->T;
  s->P /= (N / s->rho);
  s->U = s->K + s->V;
  s->Pshear /= (N / s->rho);
  s->av_iters++;
  s->av_U_tot += s->U;
  s->av_p_tot += s->P;
  s->av_T_tot += s->T;
}

/* MDSystem::KineticTemperature (MDSystem.cpp:361-373). */
double r32_kinetic_temperature(const r32_state* s, const float* vel) {
  double ret = 0.;
  for (int i = 0; i < 4 * s->N; i += 4)
    ret += (double)(vel[i] * vel[i] + vel[i + 1] * vel[i + 1] + vel[i + 2] * vel[i + 2]);
  ret *= 1. / 3. / s->N;
  return ret;
}

/* MDSystem::RenormalizeVelocities (MDSystem.cpp:375-389). */
void r32_renormalize_velocities(r32_state* s, int recalc) {
  double Tkin = s->T;
  if (recalc) Tkin = r32_kinetic_temperature(s, s->vel);
  for (int i = 0; i < 4 * s->N; i += 4) {
    s->vel[i] = (float)((double)s->vel[i] * sqrt(s->T0 / Tkin));
    s->vel[i + 1] = (float)((double)s->vel[i + 1] * sqrt(s->T0 / Tkin));
    s->vel[i + 2] = (float)((double)s->vel[i + 2] * sqrt(s->T0 / Tkin));
  }
  s->K *= s->T0 / Tkin;
  s->T = s->T0;
  s->U = s->K + s->V;
}

/* MDSystem::RenormalizeVelocitiesToEnergy (MDSystem.cpp:391-404). */
void r32_renormalize_velocities_to_energy(r32_state* s, double ust) {
  double Kold = s->K;
  double Udes = ust * s->N;
  double Kdes = Udes - s->V;
  for (int i = 0; i < 4 * s->N; i += 4) {
    s->vel[i] = (float)((double)s->vel[i] * sqrt(Kdes / Kold));
    s->vel[i + 1] = (float)((double)s->vel[i + 1] * sqrt(Kdes / Kold));
    s->vel[i + 2] = (float)((double)s->vel[i + 2] * sqrt(Kdes / Kold));
  }
  s->K = Kdes;
  s->U = s->K + s->V;
}

/* MDSystem::ApplyBoundaryConditions (MDSystem.cpp:406-436). */
void r32_apply_boundary_conditions(r32_state* s) {
  float* p = s->pos;
  float* v = s->vel;
  const double L = s->L;
  if (s->bc == 2) return;
  if (s->bc == 0) {
    for (int i = 0; i < 4 * s->N; i += 4)
      for (int d = 0; d < 3; ++d) {
        if ((double)p[i + d] < 0.) p[i + d] = (float)((double)p[i + d] + L);
        if ((double)p[i + d] > L) p[i + d] = (float)((double)p[i + d] - L);
      }
  } else {
    for (int i = 0; i < 4 * s->N; i += 4)
      for (int d = 0; d < 3; ++d) {
        if ((double)p[i + d] < 0. && v[i + d] < 0) v[i + d] = -v[i + d];
        if ((double)p[i + d] > L && v[i + d] > 0) v[i + d] = -v[i + d];
      }
  }
}

/* MDSystem::Integrate (MDSystem.cpp:438-510, 578-582): EVN or TVN branch. */
void r32_integrate(r32_state* s, double dt, int nthreads) {
  const int N = s->N;
  float* p = s->pos;
  float* v = s->vel;
  float* f = s->frc;
  if (!s->canonical) {
    for (int i = 0; i < 4 * N; i += 4) {
      float fx = f[i], fy = f[i + 1], fz = f[i + 2];
      p[i] = (float)((double)p[i] + (dt * (double)v[i] + dt * dt * (double)fx / 2.));
      p[i + 1] = (float)((double)p[i + 1] + (dt * (double)v[i + 1] + dt * dt * (double)fy / 2.));
      p[i + 2] = (float)((double)p[i + 2] + (dt * (double)v[i + 2] + dt * dt * (double)fz / 2.));
      v[i] = (float)((double)v[i] + dt * (double)fx / 2.);
      v[i + 1] = (float)((double)v[i + 1] + dt * (double)fy / 2.);
      v[i + 2] = (float)((double)v[i + 2] + dt * (double)fz / 2.);
    }
    r32_calculate_forces(s, f, nthreads);
    for (int i = 0; i < 4 * N; i += 4) {
      v[i] = (float)((double)v[i] + dt * (double)f[i] / 2.);
      v[i + 1] = (float)((double)v[i + 1] + dt * (double)f[i + 1] / 2.);
      v[i + 2] = (float)((double)v[i + 2] + dt * (double)f[i + 2] / 2.);
    }
  } else {
    float* tF = (float*)malloc(sizeof(float) * 4 * (size_t)N);
    float* tV = (float*)malloc(sizeof(float) * 4 * (size_t)N);
    for (int i = 0; i < 4 * N; i += 4) {
      float fx = f[i], fy = f[i + 1], fz = f[i + 2];
      p[i] = (float)((double)p[i] + (dt * (double)v[i] + dt * dt * (double)fx / 2.));
      p[i + 1] = (float)((double)p[i + 1] + (dt * (double)v[i + 1] + dt * dt * (double)fy / 2.));
      p[i + 2] = (float)((double)p[i + 2] + (dt * (double)v[i + 2] + dt * dt * (double)fz / 2.));
      tF[i] = 0.5f * f[i];
      tF[i + 1] = 0.5f * f[i + 1];
      tF[i + 2] = 0.5f * f[i + 2];
      tF[i + 3] = 0.f;
    }
    r32_calculate_forces(s, f, nthreads);
    for (int i = 0; i < 4 * N; i += 4) {
      tF[i] += 0.5f * f[i];
      tF[i + 1] += 0.5f * f[i + 1];
      tF[i + 2] += 0.5f * f[i + 2];
    }
    for (int i = 0; i < 4 * N; i += 4) {
      tV[i] = (float)((double)v[i] + dt * (double)tF[i] / 2.);
      tV[i + 1] = (float)((double)v[i + 1] + dt * (double)tF[i + 1] / 2.);
      tV[i + 2] = (float)((double)v[i + 2] + dt * (double)tF[i + 2] / 2.);
      tV[i + 3] = 0.f;
    }
    double Tkin = r32_kinetic_temperature(s, tV);
    double chi = sqrt(s->T0 / Tkin);
    for (int i = 0; i < 4 * N; i += 4) {
      v[i] = (float)((2. * chi - 1.) * (double)v[i] + chi * dt * (double)tF[i]);
      v[i + 1] = (float)((2. * chi - 1.) * (double)v[i + 1] + chi * dt * (double)tF[i + 1]);
      v[i + 2] = (float)((2. * chi - 1.) * (double)v[i + 2] + chi * dt * (double)tF[i + 2]);
    }
    free(tF);
    free(tV);
  }
  r32_apply_boundary_conditions(s);
  r32_calculate_parameters(s);
  s->t += dt;
}

/* MDSystem::initvelo / updatevelo (MDSystem.cpp:651-694): counts of |v|/step bins.
 * sqrt of the float sum is the C double sqrt (no std:: overload is in scope there). */
void r32_velocity_counts(const r32_state* s, double step, int nbins, int* dens) {
  memset(dens, 0, sizeof(int) * (size_t)nbins);
  const float* v = s->vel;
  for (int i = 0; i < 4 * s->N; i += 4) {
    int tind = (int)(sqrt((double)(v[i] * v[i] + v[i + 1] * v[i + 1] + v[i + 2] * v[i + 2])) / step);
    if (tind < nbins) dens[tind]++;
  }
}

/* ------------------------------------------------------------------------ */
/* Part 2: true-FP64 restatement (accuracy oracle).                          */
/* ------------------------------------------------------------------------ */

/* All-pairs LJ with minimum image, double storage, explicit epsilon/sigma:
 *   u(r) = 4 eps [(s/r)^12 - (s/r)^6],  F_i = sum_j 24 eps/r^2 [2(s/r)^12 - (s/r)^6] (x_i - x_j)
 * Same pair set as MDSystem.cpp:260-306 (ordered pairs, j != i, minimum image
 * only for periodic boxes, no cutoff).
 *   pos  : double[3N] interleaved x,y,z
 *   frc  : double[3N] out (may be NULL)
 *   epair: double[N]  out, per-particle sum_j 4 eps[(s/r)^12-(s/r)^6] (may be NULL)
 *   wpair: double[N]  out, per-particle sum_j r_ij . f_ij (may be NULL)
 *   out3 : V (= 1/2 sum_i epair), W (= sum over ordered pairs r.f), Pshear_pair (-sum x f_y / 2 ordered)
 * Rows [i0, i1) only when i0/i1 select a subset (forces for those rows only; out3 then covers them). */
void f64_forces_rows(int N, const double* pos, double L, int periodic, double eps, double sigma,
                     int i0, int i1, double* frc, double* epair, double* wpair, double* out3,
                     int nthreads) {
  const double s2 = sigma * sigma;
  double V = 0., W = 0., Ps = 0.;
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16) reduction(+ : V, W, Ps)
  for (int i = i0; i < i1; ++i) {
    double fx = 0., fy = 0., fz = 0., e = 0., w = 0., ps = 0.;
    const double xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      double rx = xi - pos[3 * j], ry = yi - pos[3 * j + 1], rz = zi - pos[3 * j + 2];
      if (periodic) {
        rx -= L * round(rx / L);
        ry -= L * round(ry / L);
        rz -= L * round(rz / L);
      }
      double r2 = rx * rx + ry * ry + rz * rz;
      double q2 = s2 / r2;
      double q6 = q2 * q2 * q2;
      double sfac = 24. * eps / r2 * (2. * q6 * q6 - q6);
      fx += sfac * rx;
      fy += sfac * ry;
      fz += sfac * rz;
      e += 4. * eps * (q6 * q6 - q6);
      w += sfac * r2;
      ps += -rx * sfac * ry;
    }
    if (frc) {
      frc[3 * i] = fx;
      frc[3 * i + 1] = fy;
      frc[3 * i + 2] = fz;
    }
    if (epair) epair[i] = e;
    if (wpair) wpair[i] = w;
    V += 0.5 * e;
    W += w;
    Ps += 0.5 * ps;
  }
  if (out3) {
    out3[0] = V;
    out3[1] = W;
    out3[2] = Ps;
  }
}

void f64_forces(int N, const double* pos, double L, int periodic, double eps, double sigma,
                double* frc, double* epair, double* wpair, double* out3, int nthreads) {
  f64_forces_rows(N, pos, L, periodic, eps, sigma, 0, N, frc, epair, wpair, out3, nthreads);
}

/* FP64 state for the integrator restatement. */
typedef struct {
  int N;
  double T0, rho, L, eps, sigma;
  int canonical, bc;
  double t;
  double U, T, K, V, P, W; /* W = sum over ordered pairs r.f */
  double *pos, *vel, *frc; /* double[3N] each, caller-owned */
  int nthreads;
} f64_state;

/* Observables as MDSystem::CalculateParameters (MDSystem.cpp:325-359) with the
 * reference's pressure normalisation P = (W/3 + N T)/(N/rho) (W/3 = virial sum
 * scaled as MDSystem.cpp:307 does: 4/3/2 over ordered pairs of r.f/4). */
void f64_parameters(f64_state* s) {
  double K = 0.;
  for (int i = 0; i < s->N; ++i) {
    const double* v = s->vel + 3 * i;
    K += (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) / 2.;
  }
  s->K = K;
  s->T = 2. * K / 3. / s->N;
  s->P = (s->W / 6. + s->N * s->T) / (s->N / s->rho);
  s->U = s->K + s->V;
}

void f64_compute_forces(f64_state* s) {
  double out3[3];
  f64_forces(s->N, s->pos, s->L, s->bc == 0, s->eps, s->sigma, s->frc, NULL, NULL, out3,
             s->nthreads);
  s->V = out3[0];
  s->W = out3[1];
}

/* Boundary handling (MDSystem.cpp:406-436) in double. */
void f64_apply_boundary_conditions(f64_state* s) {
  if (s->bc == 2) return;
  const double L = s->L;
  for (int k = 0; k < 3 * s->N; ++k) {
    if (s->bc == 0) {
      if (s->pos[k] < 0.) s->pos[k] += L;
      if (s->pos[k] > L) s->pos[k] -= L;
    } else {
      if (s->pos[k] < 0. && s->vel[k] < 0) s->vel[k] = -s->vel[k];
      if (s->pos[k] > L && s->vel[k] > 0) s->vel[k] = -s->vel[k];
    }
  }
}

/* One velocity-Verlet step, EVN (MDSystem.cpp:442-464) or TVN (:465-510), in double. */
void f64_step(f64_state* s, double dt) {
  const int n3 = 3 * s->N;
  double* p = s->pos;
  double* v = s->vel;
  double* f = s->frc;
  if (!s->canonical) {
    for (int k = 0; k < n3; ++k) {
      p[k] += dt * v[k] + dt * dt * f[k] / 2.;
      v[k] += dt * f[k] / 2.;
    }
    f64_compute_forces(s);
    for (int k = 0; k < n3; ++k) v[k] += dt * f[k] / 2.;
  } else {
    double* tF = (double*)malloc(sizeof(double) * (size_t)n3);
    for (int k = 0; k < n3; ++k) {
      p[k] += dt * v[k] + dt * dt * f[k] / 2.;
      tF[k] = 0.5 * f[k];
    }
    f64_compute_forces(s);
    double sum = 0.;
    for (int k = 0; k < n3; ++k) {
      tF[k] += 0.5 * f[k];
      double tv = v[k] + dt * tF[k] / 2.;
      sum += tv * tv;
    }
    double Tkin = sum / 3. / s->N;
    double chi = sqrt(s->T0 / Tkin);
    for (int k = 0; k < n3; ++k) v[k] = (2. * chi - 1.) * v[k] + chi * dt * tF[k];
    free(tF);
  }
  f64_apply_boundary_conditions(s);
  f64_parameters(s);
  s->t += dt;
}

/* ------------------------------------------------------------------------ */
/* Part 3: emulation of the device's integer decisions (exact histograms).   */
/* ------------------------------------------------------------------------ */

/* Device shadow: a periodic coordinate as the low 32 bits of
 * llrint(x * 2^32 / L), moved to the nearest multiple of 3 -- the device's
 * arithmetic (one double multiply by invL * 2^32, round to nearest even). */
uint32_t emu_fixed_coord(double x, double invL) {
  const double t = x * (invL * 4294967296.0);
  const uint32_t u = (uint32_t)(unsigned long long)llrint(t);
  const uint32_t r = u % 3u;
  return r == 0u ? u : (r == 1u ? u - 1u : u + 1u);
}

/* r^2 of a pair in box units^2 exactly as the device forms it in FP32:
 * d = (int32)(qj - qi); dx = (float)d; r2 = fma(dz,dz,fma(dy,dy,dx*dx)) * k2
 * where k2 = (float)((L/2^32)^2) [sigma = 1 units]. */
static float emu_r2(const uint32_t* qi, const uint32_t* qj, float k2) {
  float dx = (float)(int32_t)(qj[0] - qi[0]);
  float dy = (float)(int32_t)(qj[1] - qi[1]);
  float dz = (float)(int32_t)(qj[2] - qi[2]);
  float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
  return r2 * k2;
}

/* RDF counts of ordered pairs over r^2 bins, device binning rule:
 *   mode 0 (reference GPU rule, MDSystem.cu:39): b = min(floor(r2 * inv_dr2), nb-1)
 *   mode 1 (reference CPU rule, MDSystem.cpp:282-284): drop b >= nb
 * q: uint32[3N] fixed-point coordinates.  k2 and inv_dr2 are the FP32 constants
 * the device uses.  counts: uint64[nb]. */
void emu_rdf_r2(int N, const uint32_t* q, float k2, float inv_dr2, int nb, int mode,
                uint64_t* counts, int nthreads) {
  memset(counts, 0, sizeof(uint64_t) * (size_t)nb);
  if (nthreads < 1) nthreads = 1;
  uint64_t* part = (uint64_t*)calloc((size_t)nthreads * nb, sizeof(uint64_t));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int i = 0; i < N; ++i) {
#ifdef _OPENMP
    uint64_t* h = part + (size_t)omp_get_thread_num() * nb;
#else
    uint64_t* h = part;
#endif
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      float r2 = emu_r2(q + 3 * i, q + 3 * j, k2);
      float fb = floorf(r2 * inv_dr2);
      if (mode == 0) {
        int b = fb < (float)(nb - 1) ? (int)fb : nb - 1;
        h[b]++;
      } else if (fb < (float)nb) {
        h[(int)fb]++;
      }
    }
  }
  for (int t = 0; t < nthreads; ++t)
    for (int b = 0; b < nb; ++b) counts[b] += part[(size_t)t * nb + b];
  free(part);
}

/* RDF counts over linear r bins up to rmax (ordered pairs, r >= rmax dropped):
 * b = floor(sqrt(r2) * inv_dr) with the device's FP32 sqrt (correctly rounded). */
void emu_rdf_r(int N, const uint32_t* q, float k2, float inv_dr, float rmax2, int nb,
               uint64_t* counts, int nthreads) {
  memset(counts, 0, sizeof(uint64_t) * (size_t)nb);
  if (nthreads < 1) nthreads = 1;
  uint64_t* part = (uint64_t*)calloc((size_t)nthreads * nb, sizeof(uint64_t));
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
  for (int i = 0; i < N; ++i) {
#ifdef _OPENMP
    uint64_t* h = part + (size_t)omp_get_thread_num() * nb;
#else
    uint64_t* h = part;
#endif
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      float r2 = emu_r2(q + 3 * i, q + 3 * j, k2);
      if (!(r2 < rmax2)) continue;
      int b = (int)floorf(sqrtf(r2) * inv_dr);
      if (b > nb - 1) b = nb - 1;
      h[b]++;
    }
  }
  for (int t = 0; t < nthreads; ++t)
    for (int b = 0; b < nb; ++b) counts[b] += part[(size_t)t * nb + b];
  free(part);
}

/* Speed histogram (MDSystem.cpp:658-662 rule) over FP64 velocities:
 * b = (int)(sqrt(vx*vx + vy*vy + vz*vz) / step), dropped if b >= nb.
 * Products and sums are rounded separately (no fused multiply-add). */
void emu_velocity_counts(int N, const double* vel, double step, int nb, uint64_t* counts) {
  memset(counts, 0, sizeof(uint64_t) * (size_t)nb);
  for (int i = 0; i < N; ++i) {
    const double* v = vel + 3 * i;
    double s = v[0] * v[0];
    s = s + v[1] * v[1];
    s = s + v[2] * v[2];
    double b = floor(sqrt(s) / step);
    if (b < (double)nb) counts[(int)b]++;
  }
}

/* ------------------------------------------------------------------------ */
/* init_*: seeded initial state (the draws lj_sample_initial_state makes)   */
/* ------------------------------------------------------------------------ */
typedef struct {
  uint64_t s[4];
} init_rng;

static uint64_t init_splitmix(uint64_t* x) {
  uint64_t z = (*x += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

static uint64_t init_rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

/* xoshiro256** (Blackman & Vigna) */
static uint64_t init_next(init_rng* r) {
  uint64_t* s = r->s;
  const uint64_t out = init_rotl(s[1] * 5, 7) * 9;
  const uint64_t t = s[1] << 17;
  s[2] ^= s[0];
  s[3] ^= s[1];
  s[1] ^= s[2];
  s[0] ^= s[3];
  s[2] ^= t;
  s[3] = init_rotl(s[3], 45);
  return out;
}

static double init_uniform(init_rng* r) { return (double)(init_next(r) >> 11) * (1.0 / 9007199254740992.0); }

/* pos, vel: (n, 3) doubles; *L_out = cbrt(n / density).  lattice 0: simple
 * cubic, 1: FCC; sites filled in lattice order (x fastest), cell-centred;
 * uniform jitter of +-jitter. */
int init_sample_state(int n, double density, double T0, int lattice, double jitter, uint64_t seed, double* pos,
                      double* vel, double* L_out) {
  if (n < 1 || !(density > 0) || !(T0 >= 0)) return 1;
  const double L = cbrt((double)n / density);
  *L_out = L;
  init_rng rng;
  uint64_t x = seed;
  for (int k = 0; k < 4; ++k) rng.s[k] = init_splitmix(&x);
  if (lattice == 0) {
    const int ns = (int)ceil(cbrt((double)n) - 1e-12);
    const int side = (ns * ns * ns < n) ? ns + 1 : ns;
    const double dL = L / side;
    for (int i = 0; i < n; ++i) {
      pos[3 * i + 0] = (i % side + 0.5) * dL;
      pos[3 * i + 1] = ((i / side) % side + 0.5) * dL;
      pos[3 * i + 2] = (i / (side * side) + 0.5) * dL;
    }
  } else {
    static const double basis[4][3] = {{0, 0, 0}, {0.5, 0.5, 0}, {0.5, 0, 0.5}, {0, 0.5, 0.5}};
    int nc = (int)ceil(cbrt(n / 4.0) - 1e-12);
    while (4 * nc * nc * nc < n) ++nc;
    const double a = L / nc;
    for (int i = 0; i < n; ++i) {
      const int c = i / 4, b = i % 4;
      pos[3 * i + 0] = (c % nc + basis[b][0] + 0.25) * a;
      pos[3 * i + 1] = ((c / nc) % nc + basis[b][1] + 0.25) * a;
      pos[3 * i + 2] = (c / (nc * nc) + basis[b][2] + 0.25) * a;
    }
  }
  if (jitter > 0)
    for (int k = 0; k < 3 * n; ++k) pos[k] += (2.0 * init_uniform(&rng) - 1.0) * jitter;
  /* speed u = -ln(alpha), alpha accepted with probability
     prob(alpha) / probmax, prob(alpha) = ln^2(alpha) exp(-ln^2 alpha) / alpha */
  for (int i = 0; i < n; ++i) {
    double alpha;
    for (;;) {
      do alpha = init_uniform(&rng);
      while (alpha == 0.0);
      const double eta = init_uniform(&rng) * 1.2;
      const double tl = -log(alpha);
      if (eta < tl * tl * exp(-tl * tl) / alpha) break;
    }
    const double speed = sqrt(2.0 * T0) * (-log(alpha));
    const double cth = 2.0 * init_uniform(&rng) - 1.0;
    const double ph = 2.0 * ORACLE_PI * init_uniform(&rng);
    const double sth = sqrt(1.0 - cth * cth);
    vel[3 * i + 0] = speed * sth * cos(ph);
    vel[3 * i + 1] = speed * sth * sin(ph);
    vel[3 * i + 2] = speed * cth;
  }
  double P[3] = {0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) P[c] += vel[3 * i + c];
  for (int i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) vel[3 * i + c] -= P[c] / n;
  double s2 = 0;
  for (int k = 0; k < 3 * n; ++k) s2 += vel[k] * vel[k];
  const double Tkin = s2 / 3.0 / n;
  if (Tkin > 0) {
    const double f = sqrt(T0 / Tkin);
    for (int k = 0; k < 3 * n; ++k) vel[k] *= f;
  }
  return 0;
}
