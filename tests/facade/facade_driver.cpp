// facade_driver.cpp -- a task-style caller of the MDSystem class, written the
// way the reference's drivers use it (src/tasks/semiGCEfluctuations/
// semiGCEfluctuations.cpp:7-104, run-isotherm.cpp:84-133): configure,
// equilibrate in TVN, switch to EVN, read h_Pos every step, print averages,
// the RDF and the velocity distribution.  Built and run by
// tests/test_facade_gpu.py against include/ljgb/MDSystem.hpp + liblj_gb300.so.
#include <cmath>
#include <cstdio>
#include <cstdlib>

#include "ljgb/MDSystem.hpp"

static int GetNsub(const MDSystem& syst, double fraction) {
  const double L = syst.L;
  const double tL = L * std::pow(fraction, 1. / 3.);
  int ret = 0;
  for (int i = 0; i < 4 * syst.m_config.N; i += 4) {
    const double dx = syst.h_Pos[i] - 0.5 * L, dy = syst.h_Pos[i + 1] - 0.5 * L, dz = syst.h_Pos[i + 2] - 0.5 * L;
    if (std::fabs(dx) < 0.5 * tL && std::fabs(dy) < 0.5 * tL && std::fabs(dz) < 0.5 * tL) ret++;
  }
  return ret;
}

int main(int argc, char** argv) {
  const int steps = argc > 1 ? std::atoi(argv[1]) : 200;
  MDSystem::MDSystemConfiguration config;
  config.N = 512;
  config.T0 = 1.312;
  config.rho = 0.316;
  config.useCUDA = true;
  MDSystem syst(config);
  if (!syst.CUDAInit) {
    std::printf("init failed: %s\n", syst.lastError().c_str());
    return 2;
  }
  std::printf("init U=%.10g T=%.10g P=%.10g K=%.10g V=%.10g L=%.10g\n", syst.U, syst.T, syst.P, syst.K, syst.V, syst.L);
  syst.m_config.canonical = true;  // as semiGCEfluctuations.cpp:57 does
  syst.setCanonical(true);
  for (int i = 0; i < steps; ++i) syst.Integrate(0.005);
  std::printf("tvn T=%.10g t=%.10g av_iters=%d\n", syst.T, syst.getTime(), syst.av_iters);
  syst.setCanonical(false);
  syst.resetAveraging();
  double nsum = 0;
  for (int i = 0; i < steps; ++i) {
    syst.Integrate(0.005);
    nsum += GetNsub(syst, 0.5);
  }
  std::printf("evn U/N=%.10g <U>/N=%.10g <P>=%.10g <T>=%.10g av_iters=%d <Nsub>=%.6g\n", syst.U / config.N,
              syst.av_U_tot / syst.av_iters / config.N, syst.av_p_tot / syst.av_iters, syst.av_T_tot / syst.av_iters,
              syst.av_iters, nsum / steps);
  SplineFunction g = syst.RDF();
  // The last r^2 bin collects every pair beyond the histogram (the
  // reference GPU rule, MDSystem.cu:39), so the peak search skips it.
  double gmax = 0, rmax = 0;
  for (size_t k = 0; k + 1 < g.vals.size(); ++k)
    if (g.vals[k].second > gmax) {
      gmax = g.vals[k].second;
      rmax = g.vals[k].first;
    }
  long long total = 0;
  for (int c : syst.NdNdr2) total += c;
  std::printf("rdf bins=%zu peak_r=%.4f peak_g=%.4f total=%lld\n", g.vals.size(), rmax, gmax, total);
  syst.updatevelo();
  SplineFunction v = syst.getvelo();
  double norm = 0;
  for (auto& p : v.vals) norm += p.second * 0.12;
  std::printf("velo bins=%zu norm=%.6f maxwell(1)=%.6f\n", v.vals.size(), norm, syst.Maxwell(1.0));
  syst.Integrate(0.005, 50);
  std::printf("multi t=%.10g av_iters=%d status=%d\n", syst.getTime(), syst.av_iters, syst.lastStatus());
  return syst.lastStatus();
}
