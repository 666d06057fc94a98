// Reads a task parameter file with ljgb::TaskParameters
// (include/ljgb/Parameters.hpp) over the isotherm defaults and prints
// name=value lines; exit status 2 when the file does not parse.
#include <cstdio>

#include "ljgb/Parameters.hpp"

int main(int argc, char** argv) {
  ljgb::TaskParameters p("isotherm.run", {{"N", 400}, {"T*", 1.4}, {"teq", 10.}, {"useCUDA", 1}});
  std::ostringstream log;
  if (argc < 2 || !p.ReadParametersFromFile(argv[1], log)) return 2;
  std::printf("output_prefix=%s\n", p.output_prefix.c_str());
  for (const auto& kv : p.parameters) std::printf("%s=%.17g\n", kv.first.c_str(), kv.second);
  std::printf("full=%s\n", p.GetFullPrefix(true, false, true).c_str());
  return 0;
}
