// ljgb-run-fluctuations -- particle-number fluctuations in coordinate and
// momentum subsystems of one box, the task of the reference's
// src/tasks/run-fluctuations/run-fluctuations.cpp:10-202 on the lj_* API.
//
// Same parameters and defaults (run-fluctuations-aux.h:30-47; sample files
// input/N400.Tst1.4.rhost0.05, input/N400.ust1.708.rhost0.05), same run
// (TVN at T*, or EVN renormalised to u* per particle; equilibrate until
// t >= teq; then step and sample until t >= tfin, or forever if tfin < 0),
// same counters (slabs x, y, z < alpha L and the central cube of volume
// fraction alpha, alpha = spacing, 2 spacing, ... < 1; |v_z| < alpha
// 3 sqrt(T*), alpha up to 1; N(z < L/2)), same time-averaged RDF (the
// reference's 256 r^2 bins, normalised as MDSystem::RDF), and the same
// output every 1000 steps: console line, <prefix>.TimeDep.txt,
// <prefix>.RDF.dat, <prefix>.flucs{X,Y,Z,Cube,Vz}.dat.
//
// The counts are made on the GPU after every step (lj_counters_configure)
// and the RDF is summed there (lj_rdf_accumulate); the host reads both every
// 1000 steps instead of copying all positions and velocities every step.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "lj_gb300.h"
#include "ljgb/Parameters.hpp"
#include "ljgb/Statistics.hpp"

namespace {

constexpr double kPi = 3.14159265358979323846;

bool check(lj_status st, lj_system* s, const char* what) {
  if (st == LJ_OK) return true;
  std::cerr << what << " failed (" << (int)st << "): " << lj_last_error(s) << "\n";
  return false;
}

// The reference's alpha loops (run-fluctuations-aux.h:336, :444): alpha
// accumulated from step, < 1 - 1e-9 (coordinates) or <= 1 + 1e-9 (momenta).
std::vector<double> alphas(double step, bool up_to_one) {
  std::vector<double> a;
  for (double x = step; up_to_one ? x <= 1. + 1.e-9 : x < 1. - 1.e-9; x += step) a.push_back(x);
  return a;
}

struct FlucAverage {  // one counter: per alpha, TimeAverage of N(alpha)
  std::vector<double> alpha;
  std::vector<ljgb::TimeAverage> stats;
  explicit FlucAverage(std::vector<double> a) : alpha(std::move(a)), stats(alpha.size()) {}
  void add(const int32_t* n) {
    for (size_t k = 0; k < alpha.size(); ++k) stats[k].AddObservation(n[k]);
  }
  // CoordFlucsAverage::PrintToFile (run-fluctuations-aux.h:388-423)
  void print_coord(const std::string& fn) const {
    std::ofstream f(fn);
    for (const char* c : {"alpha", "<N>", "w[N]", "w[N]/(1-alpha)", "error", "s"}) f << std::setw(15) << c << " ";
    f << std::endl;
    for (size_t k = 0; k < alpha.size(); ++k) {
      const auto& st = stats[k];
      const double w = st.stats.GetScaledVariance(), s = st.GetS(), a = alpha[k];
      f << std::setw(15) << a << " " << std::setw(15) << st.GetMean() << " " << std::setw(15) << w << " "
        << std::setw(15) << w / (1. - a) << " " << std::setw(15)
        << st.stats.GetScaledVarianceError() * std::sqrt(s) / (1. - a) << " " << std::setw(15) << s << " "
        << std::endl;
    }
  }
  // MomentumFlucsAverage::PrintToFile (run-fluctuations-aux.h:487-524)
  void print_momentum(const std::string& fn, const std::vector<double>& vcut, int N) const {
    std::ofstream f(fn);
    for (const char* c : {"vcut", "<N>", "alpha", "w[N]", "w[N]/(1-alpha)", "error", "s"})
      f << std::setw(15) << c << " ";
    f << std::endl;
    for (size_t k = 0; k < alpha.size(); ++k) {
      const auto& st = stats[k];
      const double w = st.stats.GetScaledVariance(), s = st.GetS(), a = st.GetMean() / N;
      f << std::setw(15) << vcut[k] << " " << std::setw(15) << st.GetMean() << " " << std::setw(15) << a << " "
        << std::setw(15) << w << " " << std::setw(15) << w / (1. - a) << " " << std::setw(15)
        << st.stats.GetScaledVarianceError() * std::sqrt(s) / (1. - a) << " " << std::setw(15) << s << " "
        << std::endl;
    }
  }
};

}  // namespace

int main(int argc, char* argv[]) {
  ljgb::TaskParameters params("run", {{"N", 400},
                                      {"T*", 1.4},
                                      {"u*", 1.708},
                                      {"rho*", 0.60},
                                      {"teq", 10.},
                                      {"tfin", 1000.},
                                      {"dt*", 0.004},
                                      {"canonical", 1},
                                      {"subvolume_spacing", 0.05},
                                      {"useCUDA", 1}});
  if (argc > 1) {
    std::cout << "Reading parameters from file " << argv[1] << std::endl;
    if (!params.ReadParametersFromFile(argv[1])) return 2;
  }
  const bool canonical = std::lround(params.get("canonical")) != 0;
  params.output_prefix = params.GetFullPrefix(true, canonical, true);
  params.OutputParameters("Lennard-Jones Molecular Dynamics fluctuations run parameter list:");

  const int N = (int)std::lround(params.get("N"));
  const double rho = params.get("rho*"), Tst = params.get("T*"), ust = params.get("u*");
  const double dt = params.get("dt*"), teq = params.get("teq"), tfin = params.get("tfin");
  const double dalpha = params.get("subvolume_spacing");
  const std::string& pre = params.output_prefix;

  lj_config c;
  lj_config_default(&c);
  c.n = N;
  c.temperature = Tst;
  c.density = rho;
  c.canonical = canonical ? 1 : 0;
  lj_system* s = nullptr;
  if (!check(lj_create(&c, &s), nullptr, "lj_create")) return 1;
  if (!canonical && !check(lj_renormalize_velocities_to_energy(s, ust), s, "renormalize")) return 1;
  int32_t n_out = 0;
  double L = 0;
  lj_get_info(s, &n_out, &L);

  // counters: slabs x, y, z and cube (coordinate alphas), |v_z| (momentum
  // alphas, vmax = 3 sqrt(T*)), and N(z < L/2)
  const std::vector<double> ac = alphas(dalpha, false), am = alphas(dalpha, true);
  const double vmax = std::sqrt(Tst) * 3.0;
  std::vector<lj_counter> cs;
  for (int t = 0; t < 4; ++t) cs.push_back({t, (int32_t)ac.size(), dalpha, 0.0});
  cs.push_back({6, (int32_t)am.size(), dalpha, vmax});
  cs.push_back({2, 1, 0.5, 0.0});
  const int kChunk = 1000;
  const int bins = 4 * (int)ac.size() + (int)am.size() + 1;
  const double rdf_dr2 = lj_reference_rdf_dr2(N);

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
  if (!check(lj_counters_configure(s, cs.data(), (int32_t)cs.size(), kChunk), s, "lj_counters_configure")) return 1;

  const char* cols[] = {"t*", "u*", "T*", "Z", "<u*>", "<T*>", "<Z>"};
  for (const char* cc : cols) std::cout << std::setw(15) << cc << " ";
  std::cout << std::setw(15) << "<w>/(1-x)"
            << " " << std::endl;
  std::ofstream fout(pre + ".TimeDep.txt");
  for (const char* cc : cols) fout << std::setw(15) << cc << " ";
  for (const char* cc : {"<wx>/(1-x)", "<wy>/(1-x)", "<wz>/(1-x)", "<vx>", "<vy>", "<vz>"})
    fout << std::setw(15) << cc << " ";
  fout << std::endl;

  // production
  if (!check(lj_reset_averaging(s), s, "lj_reset_averaging")) return 1;
  if (!check(lj_rdf_accumulate(s, 1, LJ_RDF_R2_CLAMP, 256, rdf_dr2), s, "lj_rdf_accumulate")) return 1;
  FlucAverage fx(ac), fy(ac), fz(ac), fcube(ac), fvz(am);
  std::vector<double> vcut;
  for (double a : am) vcut.push_back(std::sqrt(Tst) * a * 3.0);
  double totN = 0, totN2 = 0;
  long long iters = 0;
  std::vector<int32_t> rows((size_t)kChunk * bins);
  std::vector<double> pos(3 * (size_t)N), vel(3 * (size_t)N);
  while (t < tfin || tfin < 0.) {
    // steps until the next output point (every 1000 steps) or the end
    long long k = kChunk - iters % kChunk;
    if (tfin >= 0.) {
      long long left = 0;
      for (double tt = t; tt < tfin && left < k; tt += dt) ++left;
      k = std::min(k, left);
    }
    if (!check(lj_step(s, dt, (int32_t)k), s, "lj_step")) return 1;
    int32_t got = 0;
    if (!check(lj_counters_read(s, rows.data(), kChunk, &got), s, "lj_counters_read")) return 1;
    for (int r = 0; r < got; ++r) {
      const int32_t* row = rows.data() + (size_t)r * bins;
      const size_t na = ac.size();
      fx.add(row);
      fy.add(row + na);
      fz.add(row + 2 * na);
      fcube.add(row + 3 * na);
      fvz.add(row + 4 * na);
      const double tN = row[4 * na + am.size()];
      totN += tN;
      totN2 += tN * tN;
      t += dt;
    }
    iters += got;
    if (iters % 1000 != 0) {
      if (t < tfin || tfin < 0.) continue;
      break;  // the reference writes output every 1000 steps only
    }
    lj_observables o;
    if (!check(lj_get_observables(s, &o), s, "lj_get_observables")) return 1;
    const double Tav = o.av_T_tot / o.av_iters;
    const double Nav = totN / iters, N2av = totN2 / iters;
    std::cout << std::setw(15) << t << " " << std::setw(15) << o.U / N << " " << std::setw(15) << o.T << " "
              << std::setw(15) << o.P / (rho * o.T) << " " << std::setw(15) << o.av_U_tot / o.av_iters / N << " "
              << std::setw(15) << Tav << " " << std::setw(15) << o.av_p_tot / o.av_iters / (rho * Tav) << " "
              << std::setw(15) << (N2av - Nav * Nav) / Nav / (1. - 0.5) << " " << std::endl;
    fout << std::setw(15) << t << " " << std::setw(15) << o.U / N << " " << std::setw(15) << o.T << " "
         << std::setw(15) << o.P / (rho * o.T) << " " << std::setw(15) << o.av_U_tot / o.av_iters / N << " "
         << std::setw(15) << Tav << " " << std::setw(15) << o.av_p_tot / o.av_iters / (rho * Tav) << " ";
    for (const FlucAverage* f : {&fx, &fy, &fz}) {  // the middle alpha (run-fluctuations.cpp:170-183)
      const size_t ti = f->alpha.size() / 2;
      const double a = f->alpha[ti];
      fout << std::setw(15) << f->stats[ti].stats.GetScaledVariance() / (1. - a) << " ";
    }
    if (!check(lj_get_state(s, pos.data(), vel.data(), nullptr), s, "lj_get_state")) return 1;
    double v[3] = {0, 0, 0};
    for (int i = 0; i < N; ++i)
      for (int cc = 0; cc < 3; ++cc) v[cc] += vel[3 * (size_t)i + cc];
    for (int cc = 0; cc < 3; ++cc) fout << std::setw(15) << v[cc] / N << " ";
    fout << std::endl;
    fout.flush();

    // time-averaged RDF: the mean of the per-step normalised RDFs
    // (MDSystem::RDF, MDSystem.cpp:633-649) = the normalised sum / steps
    std::vector<uint64_t> rc(256);
    int64_t ns = 0;
    if (!check(lj_rdf_accumulated(s, rc.data(), &ns, 0), s, "lj_rdf_accumulated")) return 1;
    {
      std::ofstream f(pre + ".RDF.dat");
      f << std::setw(15) << "r*"
        << " " << std::setw(15) << "G(r)"
        << " " << std::endl;
      const double n0 = N / L / L / L;
      for (int b = 0; b < 256; ++b) {
        const double r = std::sqrt((b + 0.5) * rdf_dr2);
        const double g = (double)rc[b] / (double)std::max<int64_t>(ns, 1) / rdf_dr2 / 2. / kPi / r / n0 / N;
        f << std::setw(15) << r << " " << std::setw(15) << g << " " << std::endl;
      }
    }
    fx.print_coord(pre + ".flucsX.dat");
    fy.print_coord(pre + ".flucsY.dat");
    fz.print_coord(pre + ".flucsZ.dat");
    fcube.print_coord(pre + ".flucsCube.dat");
    fvz.print_momentum(pre + ".flucsVz.dat", vcut, N);
    if (!(t < tfin || tfin < 0.)) break;
  }
  lj_destroy(s);
  return 0;
}
