// golden_driver.cpp -- feeds a golden state (written by the reference's own
// MDSystem, tests/golden/make_golden.py) through the MDSystem facade
// (include/ljgb/MDSystem.hpp) in the order the fixture generator called the
// reference: setArray, CalculateForces, CalculateParameters, initvelo(12,
// 0.12), RDF(), getvelo(); `steps` calls of Integrate(dt); updatevelo(),
// getvelo().  Prints every value the reference's RDF() / getvelo() return
// (MDSystem.cpp:633-694) so tests/test_facade_gpu.py can compare them with
// the fixture.
//
// usage: golden_driver N T0 rho canonical bc dt steps pos.f32 vel.f32
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "ljgb/MDSystem.hpp"

static bool read_f32(const char* path, std::vector<float>& out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(out.data(), sizeof(float), out.size(), f);
  std::fclose(f);
  return got == out.size();
}

static void print_row(const char* name, const std::vector<double>& v) {
  std::printf("%s", name);
  for (double x : v) std::printf(" %.17g", x);
  std::printf("\n");
}

static void print_spline(const char* xname, const char* yname, const SplineFunction& f) {
  std::vector<double> x, y;
  for (const auto& p : f.vals) {
    x.push_back(p.first);
    y.push_back(p.second);
  }
  print_row(xname, x);
  print_row(yname, y);
}

int main(int argc, char** argv) {
  if (argc != 10) {
    std::fprintf(stderr, "usage: %s N T0 rho canonical bc dt steps pos.f32 vel.f32\n", argv[0]);
    return 2;
  }
  MDSystem::MDSystemConfiguration config;
  config.N = std::atoi(argv[1]);
  config.T0 = std::atof(argv[2]);
  config.rho = std::atof(argv[3]);
  config.canonical = std::atoi(argv[4]) != 0;
  config.boundaryConditions = std::atoi(argv[5]);
  config.useCUDA = true;
  const double dt = std::atof(argv[6]);
  const int steps = std::atoi(argv[7]);
  std::vector<float> pos(4 * (size_t)config.N), vel(4 * (size_t)config.N);
  if (!read_f32(argv[8], pos) || !read_f32(argv[9], vel)) {
    std::fprintf(stderr, "cannot read the state files\n");
    return 2;
  }
  MDSystem syst(config);
  if (!syst.CUDAInit) {
    std::printf("init failed: %s\n", syst.lastError().c_str());
    return 2;
  }
  syst.setArray(0, pos.data());
  syst.setArray(1, vel.data());
  syst.CalculateForces();
  syst.CalculateParameters();
  syst.initvelo(12., 0.12);
  std::printf("scalars U=%.17g T=%.17g K=%.17g V=%.17g P=%.17g L=%.17g rdf_dr2=%.17g\n", syst.U, syst.T, syst.K,
              syst.V, syst.P, syst.L, syst.rdf_dr2);
  print_spline("rdf_x", "rdf_y", syst.RDF());
  std::vector<double> counts(syst.NdNdr2.begin(), syst.NdNdr2.end());
  print_row("rdf_counts", counts);
  print_spline("velo_x", "velo_y", syst.getvelo());
  for (int i = 0; i < steps; ++i) syst.Integrate(dt);
  syst.updatevelo();
  print_spline("velo_upd_x", "velo_upd_y", syst.getvelo());
  std::printf("status %d\n", syst.lastStatus());
  return syst.lastStatus();
}
