// ljgb-semiGCEfluctuations -- particle-number fluctuations in central cubes of
// one periodic box, the task of the reference's
// src/tasks/semiGCEfluctuations/semiGCEfluctuations.cpp:27-106 on the lj_* API.
//
// Same run: N=512, T*=1.312, rho*=0.316, dt=0.005; 10000 TVN equilibration
// steps, then EVN production of 10000 events of 200 steps.  After each event
// it counts the particles in the cube of volume fraction f around the box
// centre, for f = 0.05, 0.10, ... <= 1 accumulated as the reference's loop
// does (GetNsub, :7-25).  Every 10 events it prints one line per f with the
// reference's format (:86-101): <N> +- err, the scaled variance
// w = kappa_2/<N> +- err, w/(1 - f) +- err/(1 - f) and
// (kappa_3/kappa_2)/(1 - 2f) +- err/(1 - 2f).
//
// The counts are made on the GPU: a type-3 counter (lj_counters_configure)
// counted after every 200th step (lj_counters_set_interval), instead of
// copying all positions to the host after every event.  The reference's
// hard-coded values are the defaults.  An optional parameter file in the task
// parameter format overrides them: N, T*, rho*, dt*, equilibration_steps,
// steps_per_event, events, print_every.  dump_counts 1 also writes the
// per-event counts to <output_prefix>.counts.dat (one row per event, one
// column per f).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
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

}  // namespace

int main(int argc, char* argv[]) {
  ljgb::TaskParameters params("semiGCE", {{"N", 512},
                                          {"T*", 1.312},
                                          {"rho*", 0.316},
                                          {"dt*", 0.005},
                                          {"equilibration_steps", 10000},
                                          {"steps_per_event", 200},
                                          {"events", 10000},
                                          {"print_every", 10},
                                          {"dump_counts", 0}});
  if (argc > 1 && !params.ReadParametersFromFile(argv[1], std::cerr)) return 2;
  const int N = (int)std::lround(params.get("N"));
  const double Tst = params.get("T*"), rhost = params.get("rho*"), dt = params.get("dt*");
  const long long iterspreeq = std::llround(params.get("equilibration_steps"));
  const int itersstep = (int)std::lround(params.get("steps_per_event"));
  const int nev = (int)std::lround(params.get("events"));
  const int print_every = (int)std::lround(params.get("print_every"));
  if (N < 2 || itersstep < 1 || nev < 0 || print_every < 1 || iterspreeq < 0) {
    std::cerr << "invalid parameters\n";
    return 2;
  }

  // the reference's fraction loop, accumulated in floating point
  std::vector<double> fracs;
  for (double tfr = 0.05; tfr <= 1.; tfr += 0.05) fracs.push_back(tfr);
  std::vector<ljgb::NumberStatistics> stats(fracs.size());

  lj_config c;
  lj_config_default(&c);
  c.n = N;
  c.temperature = Tst;
  c.density = rhost;
  c.canonical = 0;
  lj_system* s = nullptr;
  if (!check(lj_create(&c, &s), nullptr, "lj_create")) return 1;

  // equilibration: TVN
  if (!check(lj_set_canonical(s, 1), s, "lj_set_canonical")) return 1;
  for (long long done = 0; done < iterspreeq;) {
    const int k = (int)std::min<long long>(iterspreeq - done, 100000);
    if (!check(lj_step(s, dt, k), s, "lj_step")) return 1;
    done += k;
  }

  // production: EVN, the central cubes counted after every itersstep-th step
  if (!check(lj_set_canonical(s, 0), s, "lj_set_canonical")) return 1;
  const lj_counter cube = {3, (int32_t)fracs.size(), 0.05, 0.0};
  if (!check(lj_counters_configure(s, &cube, 1, print_every), s, "lj_counters_configure")) return 1;
  if (!check(lj_counters_set_interval(s, itersstep), s, "lj_counters_set_interval")) return 1;
  std::ofstream dump;
  if (std::lround(params.get("dump_counts")) != 0) dump.open(params.output_prefix + ".counts.dat");

  std::vector<int32_t> rows((size_t)print_every * fracs.size());
  for (int iN = 1; iN <= nev;) {
    // events up to the next output point
    const int k = std::min(print_every - (iN - 1) % print_every, nev - iN + 1);
    if (!check(lj_step(s, dt, k * itersstep), s, "lj_step")) return 1;
    int32_t got = 0;
    if (!check(lj_counters_read(s, rows.data(), k, &got), s, "lj_counters_read")) return 1;
    if (got != k) {
      std::cerr << "expected " << k << " counted steps, got " << got << "\n";
      return 1;
    }
    for (int r = 0; r < got; ++r, ++iN) {
      const int32_t* row = rows.data() + (size_t)r * fracs.size();
      for (size_t i = 0; i < fracs.size(); ++i) stats[i].AddObservation(static_cast<double>(row[i]));
      if (dump.is_open()) {
        for (size_t i = 0; i < fracs.size(); ++i) dump << row[i] << (i + 1 < fracs.size() ? " " : "\n");
      }
      if (iN % print_every == 0) {
        for (size_t i = 0; i < fracs.size(); ++i) {
          const ljgb::NumberStatistics& st = stats[i];
          std::printf("%15d %10lf +- %-10lf %10lf +- %-10lf %10lf +- %-10lf %10lf +- %-10lf\n", iN, st.GetMean(),
                      st.GetMeanError(), st.GetScaledVariance(), st.GetScaledVarianceError(),
                      st.GetScaledVariance() / (1. - fracs[i]), st.GetScaledVarianceError() / (1. - fracs[i]),
                      st.GetSkewness() / (1. - 2. * fracs[i]), st.GetSkewnessError() / (1. - 2. * fracs[i]));
        }
        std::printf("\n");
        std::fflush(stdout);
      }
    }
  }
  lj_destroy(s);
  return 0;
}
