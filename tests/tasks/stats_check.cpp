// Reads numbers from stdin and prints ljgb::NumberStatistics / TimeAverage
// of the series (include/ljgb/Statistics.hpp), for comparison with the
// numpy restatement in oracle/tasks.py.
#include <cstdio>
#include <iostream>

#include "ljgb/Statistics.hpp"

int main() {
  ljgb::TimeAverage ta;
  double x;
  while (std::cin >> x) ta.AddObservation(x);
  const ljgb::NumberStatistics& s = ta.stats;
  std::printf("n=%lld mean=%.17g var=%.17g mean_err=%.17g w=%.17g w_err=%.17g s=%.17g ta_err=%.17g "
              "skew=%.17g skew_err=%.17g kurt=%.17g kurt_err=%.17g\n",
              (long long)s.GetNumberOfObservations(), s.GetMean(), s.GetVariance(), s.GetMeanError(),
              s.GetScaledVariance(), s.GetScaledVarianceError(), ta.GetS(), ta.GetMeanError(), s.GetSkewness(),
              s.GetSkewnessError(), s.GetKurtosis(), s.GetKurtosisError());
  return 0;
}
