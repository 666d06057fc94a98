// ljgb-run-isotherm -- equation of state along an isotherm (TVN runs over a
// density grid), the task of the reference's src/tasks/run-isotherm/
// run-isotherm.cpp:10-170 on the lj_* API.
//
// Same parameters and defaults (run-isotherm-aux.h:30-45; sample file
// input/N400.Tst1.4.isotherm), same loop per density (equilibrate until
// t >= teq, then observe u* = U/N and p* before every step until t >= tfin),
// same time averages with statistical-inefficiency errors, same console
// lines every 1000 observations and the same <prefix>.dat columns, including
// the isothermal compressibility w[N] = T0 / (dp*/drho*) from neighbouring
// densities.
//
// The steps run on the GPU in chunks of up to 1000 with the per-step
// observables recorded on the device (lj_set_recording), instead of a host
// round trip per step.  useCUDA is accepted and ignored (there is no CPU
// path).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <vector>

#include "lj_gb300.h"
#include "ljgb/Parameters.hpp"
#include "ljgb/Statistics.hpp"

namespace {

bool check(lj_status st, lj_system* s, const char* what) {
  if (st == LJ_OK) return true;
  std::cerr << what << " failed (" << (int)st << "): " << lj_last_error(s) << "\n";
  return false;
}

void row(std::ostream& o, const std::vector<double>& v) {
  for (double x : v) o << std::setw(15) << x << " ";
}

}  // namespace

int main(int argc, char* argv[]) {
  ljgb::TaskParameters params("isotherm.run", {{"N", 400},
                                               {"T*", 1.4},
                                               {"rho*_min", 0.60},
                                               {"rho*_max", 0.60},
                                               {"drho*", 0.01},
                                               {"teq", 10.},
                                               {"tfin", 5000.},
                                               {"dt*", 0.004},
                                               {"useCUDA", 1}});
  if (argc > 1) {
    std::cout << "Reading parameters from file " << argv[1] << std::endl;
    if (!params.ReadParametersFromFile(argv[1])) return 2;
  }
  params.output_prefix = params.GetFullPrefix(false, true, false);
  params.OutputParameters("Lennard-Jones Molecular Dynamics isotherm run parameter list:");

  const int N = (int)std::lround(params.get("N"));
  const double Tst = params.get("T*");
  const double rhomin = params.get("rho*_min"), rhomax = params.get("rho*_max"), drho = params.get("drho*");
  const double dt = params.get("dt*"), teq = params.get("teq"), tfin = params.get("tfin");

  const char* cols[] = {"rho*", "t*", "T*", "<u*>", "d<u*>", "teq_u*", "<p*>", "d<p*>", "teq_p*", "<Z>", "d<Z>"};
  for (const char* c : cols) std::cout << std::setw(15) << c << " ";
  std::cout << std::endl;
  std::ofstream fout(params.output_prefix + ".dat");
  for (const char* c : cols) fout << std::setw(15) << c << " ";
  fout << std::setw(15) << "w[N]"
       << " " << std::setw(15) << "dw[N]"
       << " " << std::endl;

  double Pprev = 0., Ppreverr = 0.;
  const int kChunk = 1000;
  std::vector<lj_observables> rec(kChunk);
  for (double rho = rhomin; rho <= rhomax; rho += drho) {
    std::cout << std::endl;
    lj_config c;
    lj_config_default(&c);
    c.n = N;
    c.temperature = Tst;
    c.density = rho;
    c.canonical = 1;
    lj_system* s = nullptr;
    if (!check(lj_create(&c, &s), nullptr, "lj_create")) return 1;

    // equilibration: the reference's loop while (t < teq) { step; t += dt; }
    double t = 0.;
    long long neq = 0;
    while (t < teq) {
      t += dt;
      ++neq;
    }
    for (long long done = 0; done < neq;) {
      const int k = (int)std::min<long long>(neq - done, 100000);
      if (!check(lj_step(s, dt, k), s, "lj_step")) return 1;
      done += k;
    }
    // production: observe, then step, while t < tfin
    long long nprod = 0;
    for (double tp = t; tp < tfin; tp += dt) ++nprod;
    ljgb::TimeAverage uav, Pav;
    lj_observables o;
    if (!check(lj_get_observables(s, &o), s, "lj_get_observables")) return 1;
    long long iters = 0;
    double T = o.T;
    auto observe = [&](const lj_observables& ob) {
      uav.AddObservation(ob.U / N);
      Pav.AddObservation(ob.P);
      T = ob.T;
      ++iters;
      if (iters % 1000 == 0)
        row(std::cout, {rho, t, T, uav.GetMean(), uav.GetMeanError(), uav.GetS() * dt, Pav.GetMean(),
                        Pav.GetMeanError(), Pav.GetS() * dt, Pav.GetMean() / rho / Tst, Pav.GetMeanError() / rho / Tst}),
            std::cout << std::endl;
    };
    if (nprod > 0) observe(o);
    lj_set_recording(s, kChunk);
    for (long long done = 0; done < nprod;) {
      // the last production step is taken but not observed
      const int k = (int)std::min<long long>(nprod - done, kChunk);
      if (!check(lj_step(s, dt, k), s, "lj_step")) return 1;
      int32_t cnt = 0;
      if (!check(lj_get_records(s, rec.data(), kChunk, &cnt), s, "lj_get_records")) return 1;
      for (int r = 0; r < cnt; ++r) {
        t += dt;
        if (done + r + 1 < nprod) observe(rec[r]);
      }
      done += k;
      lj_set_recording(s, kChunk);  // consumed
    }
    if (!check(lj_get_observables(s, &o), s, "lj_get_observables")) return 1;

    row(fout, {rho, t - dt, o.T, uav.GetMean(), uav.GetMeanError(), uav.GetS() * dt, Pav.GetMean(),
               Pav.GetMeanError(), Pav.GetS() * dt, Pav.GetMean() / rho / Tst, Pav.GetMeanError() / rho / Tst});
    const double Pcur = Pav.GetMean(), Pcurerr = Pav.GetMeanError();
    const double tdrho = (rho == rhomin) ? rhomin : drho;
    const double w = Tst / ((Pcur - Pprev) / tdrho);
    const double werr = Tst * tdrho * std::sqrt(Pcurerr * Pcurerr + Ppreverr * Ppreverr) / std::abs(Pcur - Pprev);
    row(fout, {w, werr});
    fout << std::endl;
    fout.flush();
    Pprev = Pcur;
    Ppreverr = Pcurerr;
    lj_destroy(s);
  }
  return 0;
}
