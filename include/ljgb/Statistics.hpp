// ljgb/Statistics.hpp -- sample statistics of the task drivers.
//
// Restates the parts of the reference's statistics that its task drivers
// use:
//  * NumberStatistics (src/extra/sample-moments/NumberStatistics.h):
//    mean, biased central moments <(x - <x>)^r> up to r = 4 with errors up
//    to r = 4 (moments to the 8th order are summed), error of the mean
//    sqrt(var / n), the central-moment sample covariances of Kendall &
//    Stuart (NumberStatistics.h:208-225), the scaled variance kappa_2 / <x>
//    and its error (:276-291), and the skewness kappa_3 / kappa_2 and
//    kurtosis kappa_4 / kappa_2 with the delta-method errors of a cumulant
//    ratio (:304-310 with :470-560);
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
  static constexpr int kOrder = 8;  // highest moment summed (errors of 4th-order cumulants)

  void AddObservation(double x) {
    if (n_ == 0) shift_ = x;
    const double d = x - shift_;
    double p = 1.0;
    for (int k = 1; k <= kOrder; ++k) {
      p *= d;
      sums_[k] += p;
    }
    ++n_;
  }
  int64_t GetNumberOfObservations() const { return n_; }
  double GetMean() const { return n_ ? shift_ + sums_[1] / n_ : 0.0; }
  // mu_r = <(x - <x>)^r>, r = 0..kOrder (biased, 1/n): the binomial
  // expansion of the moments about the first observation
  double GetCentralMoment(int r) const {
    if (!n_ || r < 0 || r > kOrder) return 0.0;
    if (r == 0) return 1.0;
    if (r == 1) return 0.0;
    const double a = sums_[1] / n_;
    double mu = 0.0, pa = 1.0, binom = 1.0;
    for (int i = 0; i <= r; ++i) {  // C(r, i) m_{r-i} (-a)^i
      const double m = (r - i == 0) ? 1.0 : sums_[r - i] / n_;
      mu += binom * m * pa;
      pa *= -a;
      binom = binom * (r - i) / (i + 1);
    }
    return mu;
  }
  // cov(mu_r, mu_q) of the sample central moments (NumberStatistics.h:208-225)
  double GetCentralMomentsSampleCovariance(int r, int q) const {
    if (r <= 1 || q <= 1 || r + q > kOrder || !n_) return 0.0;
    const double m2 = GetCentralMoment(2);
    double c = GetCentralMoment(r + q) - GetCentralMoment(r) * GetCentralMoment(q);
    c += r * q * m2 * GetCentralMoment(r - 1) * GetCentralMoment(q - 1);
    c -= r * GetCentralMoment(r - 1) * GetCentralMoment(q + 1);
    c -= q * GetCentralMoment(r + 1) * GetCentralMoment(q - 1);
    return c / n_;
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
  // kappa_3 / kappa_2 = mu_3 / mu_2
  double GetSkewness() const { return GetCentralMoment(3) / GetCentralMoment(2); }
  double GetSkewnessError() const {
    // gradient of mu3 / mu2 in (mu2, mu3)
    const double m2 = GetCentralMoment(2), m3 = GetCentralMoment(3);
    const double g[2] = {-m3 / (m2 * m2), 1.0 / m2};
    return delta_error(g, 2);
  }
  // kappa_4 / kappa_2 = (mu_4 - 3 mu_2^2) / mu_2
  double GetKurtosis() const {
    const double m2 = GetCentralMoment(2);
    return (GetCentralMoment(4) - 3.0 * m2 * m2) / m2;
  }
  double GetKurtosisError() const {
    // gradient of (mu4 - 3 mu2^2) / mu2 in (mu2, mu3, mu4)
    const double m2 = GetCentralMoment(2), m4 = GetCentralMoment(4);
    const double k4 = m4 - 3.0 * m2 * m2;
    const double g[3] = {-6.0 - k4 / (m2 * m2), 0.0, 1.0 / m2};
    return delta_error(g, 3);
  }

 private:
  // sqrt(g^T C g) with C the sample covariance of (mu_2, ..., mu_{2+ng-1})
  double delta_error(const double* g, int ng) const {
    double v = 0.0;
    for (int a = 0; a < ng; ++a)
      for (int b = 0; b < ng; ++b) v += g[a] * g[b] * GetCentralMomentsSampleCovariance(2 + a, 2 + b);
    return std::sqrt(v);
  }

  double shift_ = 0.0;
  double sums_[kOrder + 1] = {};
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
