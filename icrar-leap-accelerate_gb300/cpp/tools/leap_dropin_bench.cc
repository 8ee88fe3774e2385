// Timing of the C++ drop-in call: LeapCalibratorFactory::Create(gb300)->Calibrate(...)
// (the call the reference CLI makes, LA/../leap-accelerate-cli/main.cc:120-128) on a
// ".leapms" file loaded once, repeated, with a steady clock around each call.
//   leap_dropin_bench -f file.leapms -d '[[ra, dec], ...]' [-s interval] [-p fp64|mixed]
//                     [--warmup W] [--repeat K] [--out result.json]
// Every timed call builds the MetaData, moves each solution interval's visibilities
// from host memory to the device, calibrates all directions and returns the
// CalibrationCollection on the host.  Prints one JSON line: per-call milliseconds,
// the solution count and the visibility bytes one call moves.
#include <chrono>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "icrar/LeapCalibratorFactory.h"
#include "icrar/exception.h"

namespace {

// [[ra, dec], ...] as written by json.dumps.
std::vector<icrar::SphericalDirection> parse_directions(const std::string& s) {
  std::vector<double> v;
  std::string num;
  for (char c : s) {
    if ((c >= '0' && c <= '9') || c == '.' || c == '-' || c == '+' || c == 'e' || c == 'E') {
      num += c;
    } else if (!num.empty()) {
      v.push_back(std::stod(num));
      num.clear();
    }
  }
  if (!num.empty()) v.push_back(std::stod(num));
  if (v.empty() || v.size() % 2)
    throw icrar::invalid_argument_exception("expected [[ra, dec], ...]", "directions", __FILE__, __LINE__);
  std::vector<icrar::SphericalDirection> d;
  for (size_t i = 0; i < v.size(); i += 2) d.emplace_back(v[i], v[i + 1]);
  return d;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    std::string file, dirs, interval = "-1", precision = "mixed", out;
    int warmup = 1, repeat = 3;
    for (int i = 1; i < argc; ++i) {
      const std::string a = argv[i];
      auto next = [&]() -> std::string {
        if (i + 1 >= argc) throw icrar::invalid_argument_exception("missing value", a, __FILE__, __LINE__);
        return argv[++i];
      };
      if (a == "-f") file = next();
      else if (a == "-d") dirs = next();
      else if (a == "-s") interval = next();
      else if (a == "-p") precision = next();
      else if (a == "--warmup") warmup = std::stoi(next());
      else if (a == "--repeat") repeat = std::stoi(next());
      else if (a == "--out") out = next();
      else throw icrar::invalid_argument_exception("unknown option", a, __FILE__, __LINE__);
    }
    if (file.empty() || dirs.empty() || repeat < 1 || warmup < 0)
      throw icrar::invalid_argument_exception("need -f, -d and --repeat >= 1", "arguments", __FILE__, __LINE__);
    icrar::gb300::GpuOptions opt;
    if (precision == "mixed") opt.precision = LEAP_PRECISION_MIXED;
    else if (precision != "fp64") throw icrar::invalid_argument_exception("precision must be fp64 or mixed", "precision", __FILE__, __LINE__);
    const auto directions = parse_directions(dirs);
    const icrar::Slice slice = icrar::ParseSlice(interval);
    const icrar::MeasurementSet ms(file);
    auto calibrator = icrar::LeapCalibratorFactory::Create(icrar::ComputeImplementation::gb300, opt);
    std::vector<double> ms_per_call;
    size_t solutions = 0;
    for (int k = 0; k < warmup + repeat; ++k) {
      const auto t0 = std::chrono::steady_clock::now();
      const auto result = calibrator->Calibrate(ms, directions, slice, 0.0, std::nullopt, false);
      const auto t1 = std::chrono::steady_clock::now();
      if (k >= warmup) ms_per_call.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
      solutions = result.GetCalibrations().size();
      if (k == warmup + repeat - 1 && !out.empty()) {
        std::ofstream f(out);
        result.Serialize(f);
      }
    }
    const double vis_bytes = static_cast<double>(ms.GetNumRows()) * ms.GetNumChannels() * ms.GetNumPols() *
                             (ms.HasFloatData() ? 8.0 : 16.0);
    std::ostringstream o;
    o.precision(17);
    o << "{\"ms_per_call\": [";
    for (size_t i = 0; i < ms_per_call.size(); ++i) o << (i ? ", " : "") << ms_per_call[i];
    o << "], \"solutions\": " << solutions << ", \"directions\": " << directions.size()
      << ", \"visibility_bytes\": " << vis_bytes << "}";
    std::cout << o.str() << std::endl;
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return -1;
  }
}
