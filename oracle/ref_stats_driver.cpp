// ref_stats_driver.cpp -- runs the reference's own TimeAverage /
// NumberStatistics (src/tasks/auxiliary/time-average-aux.h:27-67 over
// src/extra/sample-moments/NumberStatistics.h of vlvovch/lennard-jones-cuda,
// compiled where they lie by oracle/build_ref.sh) on a series read from
// stdin, and prints the statistics the task drivers use.
//
// TEST INFRASTRUCTURE ONLY: tests/golden/make_stats_golden.py runs it to
// write the fixtures that pin oracle/tasks.py and include/ljgb/Statistics.hpp.
//
// argv[1], if given, is passed to NumberStatistics::SetMeanShift before the
// first observation (the reference's own guard against round-off in the
// power sums of a series with a large mean).
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "time-average-aux.h"

int main(int argc, char** argv) {
  TimeAverage ta;
  if (argc > 1) ta.stats.SetMeanShift(std::atof(argv[1]));
  double x;
  while (std::cin >> x) ta.AddObservation(x);
  SampleMoments::NumberStatistics& s = ta.stats;
  std::printf("n=%lld mean=%.17g var=%.17g mean_err=%.17g w=%.17g w_err=%.17g s=%.17g ta_err=%.17g "
              "skew=%.17g skew_err=%.17g kurt=%.17g kurt_err=%.17g\n",
              (long long)s.GetNumberOfObservations(), s.GetMean(), s.GetVariance(), s.GetMeanError(),
              s.GetScaledVariance(), s.GetScaledVarianceError(), ta.GetS(), ta.GetMeanError(), s.GetSkewness(),
              s.GetSkewnessError(), s.GetKurtosis(), s.GetKurtosisError());
  return 0;
}
