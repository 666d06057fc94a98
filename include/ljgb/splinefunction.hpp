// splinefunction.hpp -- tabulated function with linear interpolation, the
// return type of MDSystem::RDF() and MDSystem::getvelo().
//
// Same interface as the reference's SplineFunction
// (src/library/splinefunction.h:7-79): a sorted vector of (x, y) pairs in the
// public member `vals`, evaluated by linear interpolation inside the table and
// linear extrapolation from the end intervals outside it.
#pragma once

#include <algorithm>
#include <fstream>
#include <utility>
#include <vector>

class SplineFunction {
 public:
  std::vector<std::pair<double, double> > vals;

  SplineFunction() = default;
  SplineFunction(const std::vector<double>& x, const std::vector<double>& y) { fill(x, y); }

  void add_val(double x, double y) {
    vals.emplace_back(x, y);
    std::sort(vals.begin(), vals.end());
  }

  // Linear interpolation on the interval containing arg (the first or last
  // interval when arg lies outside the table).  Needs at least two points.
  double f(double arg) const {
    const size_t n = vals.size();
    size_t hi = std::lower_bound(vals.begin(), vals.end(), std::make_pair(arg, 0.0)) - vals.begin();
    if (hi == 0) hi = 1;
    if (hi >= n) hi = n - 1;
    const auto& a = vals[hi - 1];
    const auto& b = vals[hi];
    return a.second + (arg - a.first) * (b.second - a.second) / (b.first - a.first);
  }

  double fsquare(double arg) const {
    const double v = f(arg);
    return v * v;
  }

  // Two-point zero table on [0, 1].
  void clear() {
    vals.assign(2, std::make_pair(0.0, 0.0));
    vals[1].first = 1.0;
  }

  void clearall() { vals.clear(); }

  void fill(const std::vector<double>& x, const std::vector<double>& y) {
    vals.clear();
    for (size_t k = 0; k < x.size() && k < y.size(); ++k) vals.emplace_back(x[k], y[k]);
    std::sort(vals.begin(), vals.end());
  }

  void setConstant(double v) {
    vals.clear();
    vals.emplace_back(0.0, v);
    vals.emplace_back(1.0, v);
  }

  // Whitespace-separated "x y" pairs.
  void loadFromFile(const char* file) {
    vals.clear();
    std::ifstream in(file);
    double x, y;
    while (in >> x >> y) vals.emplace_back(x, y);
    std::sort(vals.begin(), vals.end());
  }
};
