// ljgb/Statistics.hpp -- sample statistics of the task drivers.
//
// Restates the parts of the reference's statistics that its task drivers
// use:
//  * NumberStatistics (src/extra/sample-moments/NumberStatistics.h):
//    mean, biased variance <(x - <x>)^2>, error of the mean sqrt(var / n),
//    central moments up to the 4th, the scaled variance kappa_2 / <x> and
//    its large-sample error (Kendall & Stuart: var(m2) = (mu4 - mu2^2)/n,
//    cov(m2, <x>) = mu3/n);
//  * TimeAverage (src/tasks/auxiliary/time-average-aux.h:27-67): the
//    statistical inefficiency s = 2 / ln(var / (<x_t x_{t-1}> - <x>^2)) of a
//    time series with exponentially decaying correlations (Allen &
//    Tildesley, Computer Simulation of Liquids, pp. 194-195), s = 1 where the
//    logarithm is negative, and the error of the mean scaled by sqrt(s).
// NumberStatistics sums its moments about the first observation, which
// keeps the variance of a series like U/N ~ -5 +- 1e-2 free of cancellation.
#pragma once

#include <cmath>
#include <cstdint>

namespace ljgb {

class NumberStatistics {
 public:
  void AddObservation(double x) {
    if (n_ == 0) shift_ = x;
    const double d = x - shift_;
    double p = 1.0;
    for (int k = 1; k <= 4; ++k) {
      p *= d;
      sums_[k] += p;
    }
    ++n_;
  }
  int64_t GetNumberOfObservations() const { return n_; }
  double GetMean() const { return n_ ? shift_ + sums_[1] / n_ : 0.0; }
  // <(x - <x>)^r>, r = 0..4 (biased, 1/n)
  double GetCentralMoment(int r) const {
    if (!n_ || r < 0 || r > 4) return 0.0;
    const double m[5] = {1.0, sums_[1] / n_, sums_[2] / n_, sums_[3] / n_, sums_[4] / n_};
    const double a = m[1];
    switch (r) {
      case 0: return 1.0;
      case 1: return 0.0;
      case 2: return m[2] - a * a;
      case 3: return m[3] - 3 * a * m[2] + 2 * a * a * a;
      default: return m[4] - 4 * a * m[3] + 6 * a * a * m[2] - 3 * a * a * a * a;
    }
  }
  double GetVariance() const { return GetCentralMoment(2); }
  double GetMeanError() const { return n_ ? std::sqrt(GetVariance() / n_) : 0.0; }
  double GetScaledVariance() const { return GetVariance() / GetMean(); }
  double GetScaledVarianceError() const {
    const double c1 = GetVariance(), c2 = GetMean();
    const double c1dev = (GetCentralMoment(4) - c1 * c1) / n_;
    const double c2dev = GetMeanError() * GetMeanError();
    const double c12 = GetCentralMoment(3) / n_;
    return std::fabs(c1 / c2) * std::sqrt(c1dev / c1 / c1 + c2dev / c2 / c2 - 2.0 * c12 / c1 / c2);
  }

 private:
  double shift_ = 0.0;
  double sums_[5] = {0, 0, 0, 0, 0};
  int64_t n_ = 0;
};

class TimeAverage {
 public:
  NumberStatistics stats;

  void AddObservation(double x) {
    stats.AddObservation(x);
    if (iters_ > 0) lag_sum_ += last_ * x;
    last_ = x;
    ++iters_;
  }
  // statistical inefficiency (in units of the sampling interval); the lag
  // product is summed over the raw values as in the reference.  Where the
  // lag-1 covariance is not positive or not below the variance (no
  // exponential decay to fit), s = 1; the reference's formula gives NaN or
  // infinity there.
  double GetS() const {
    const double mean = stats.GetMean();
    const double corr = lag_sum_ / (iters_ - 1) - mean * mean;
    const double ratio = stats.GetVariance() / corr;
    if (!(corr > 0.0) || !(ratio > 1.0)) return 1.0;
    const double s = 2.0 / std::log(ratio);
    return s < 0.0 ? 1.0 : s;
  }
  double GetMean() const { return stats.GetMean(); }
  double GetMeanError() const { return stats.GetMeanError() * std::sqrt(GetS()); }
  int64_t GetNumberOfObservations() const { return iters_; }

 private:
  double last_ = 0.0, lag_sum_ = 0.0;
  int64_t iters_ = 0;
};

}  // namespace ljgb
