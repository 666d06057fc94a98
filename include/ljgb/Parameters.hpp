// ljgb/Parameters.hpp -- parameter files of the task drivers.
//
// The reference's task drivers read `name value` pairs, whitespace
// separated, where a token starting with '#' comments out the rest of its
// line and `output_prefix <string>` names the output files
// (src/tasks/run-fluctuations/include/run-fluctuations-aux.h:54-85,
// src/tasks/run-isotherm/include/run-isotherm-aux.h:50-81; samples under
// input/).  Output files are named <prefix>.<dd-mm-YYYY-THH-MM-SS>.N<N>...
// (GetFullPrefix, run-fluctuations-aux.h:101-118).  This reader keeps that
// format and its defaults-then-file semantics, and reports a value that does
// not parse instead of reading on.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <ctime>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <map>
#include <sstream>
#include <string>

namespace ljgb {

struct TaskParameters {
  std::string output_prefix;
  std::map<std::string, double> parameters;

  TaskParameters(std::string prefix, std::map<std::string, double> defaults)
      : output_prefix(std::move(prefix)), parameters(std::move(defaults)) {}

  // Reads name/value pairs over the defaults; false if the file cannot be
  // opened or a value is not a number (parameters read up to then are kept).
  bool ReadParametersFromFile(const std::string& filename, std::ostream& log = std::cout) {
    std::ifstream fin(filename);
    if (!fin.is_open()) {
      log << "Cannot open parameters file " << filename << "\n";
      return false;
    }
    log << "Reading input parameters from file " << filename << "\n";
    std::string var;
    while (fin >> var) {
      if (var[0] == '#') {
        fin.ignore(std::numeric_limits<std::streamsize>::max(), '\n');
        continue;
      }
      if (var == "output_prefix") {
        fin >> output_prefix;
        log << "Reading input parameter output_prefix = " << output_prefix << "\n";
        continue;
      }
      std::string tok;
      if (!(fin >> tok)) {
        log << "Parameter " << var << " has no value\n";
        return false;
      }
      char* end = nullptr;
      const double val = std::strtod(tok.c_str(), &end);
      if (end == tok.c_str() || *end != '\0') {
        log << "Parameter " << var << ": value '" << tok << "' is not a number\n";
        return false;
      }
      log << "Reading input parameter " << var << " = " << val << "\n";
      parameters[var] = val;
    }
    return true;
  }

  void OutputParameters(const std::string& title, std::ostream& out = std::cout) const {
    const int tabsize = 25;
    out << title << "\n";
    for (const auto& el : parameters) out << std::setw(tabsize) << el.first << " = " << el.second << "\n";
    out << std::setw(tabsize) << "output_prefix"
        << " = " << output_prefix << "\n\n";
  }

  // <prefix>.<dd-mm-YYYY-THH-MM-SS>.N<N>[.Tst<T*> | .ust<u*>][.rhost<rho*>]
  std::string GetFullPrefix(bool with_ensemble_key, bool canonical, bool with_density) const {
    std::time_t t = std::time(nullptr);
    std::tm tm = *std::localtime(&t);
    std::stringstream ss;
    ss << std::put_time(&tm, "%d-%m-%Y-T%H-%M-%S");
    ss << ".N" << get("N");
    if (!with_ensemble_key || canonical)
      ss << ".Tst" << get("T*");
    else
      ss << ".ust" << get("u*");
    if (with_density) ss << ".rhost" << get("rho*");
    return output_prefix + "." + ss.str();
  }

  double get(const std::string& k) const {
    auto it = parameters.find(k);
    return it == parameters.end() ? 0.0 : it->second;
  }
};

}  // namespace ljgb
