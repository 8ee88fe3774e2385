// Test driver for the C++ drop-in layer: the calibration call of the
// reference CLI (LA/../leap-accelerate-cli/main.cc:78-141) on a ".leapms" file.
//   leap_calibrate_driver [--config file.json] [-f file.leapms] [-i impl] [-d directions]
//                         [-s interval] [-a refAnt] [-m minBL] [-p fp64|mixed] [--cache]
// Precedence: defaults < config file < command line (Arguments.cc:96-118).
// Config keys: filePath, computeImplementation, directions, solutionInterval,
// referenceAntenna, minimumBaselineThreshold, useFileSystemCache, precision.
// Prints the CalibrationCollection JSON; on error prints it and returns -1.
#include <cctype>
#include <cstring>
#include <optional>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "icrar/LeapCalibratorFactory.h"
#include "icrar/exception.h"

namespace {

// Minimal JSON value: enough for the config keys above.
struct Json {
  enum Kind { Null, Number, String, Bool, Array, Object } kind = Null;
  double num = 0;
  std::string str;
  bool b = false;
  std::vector<Json> arr;
  std::map<std::string, Json> obj;
  std::string raw;  // source text of this value
};

struct Parser {
  const std::string& s;
  size_t i = 0;
  void ws() { while (i < s.size() && std::isspace(static_cast<unsigned char>(s[i]))) ++i; }
  Json value() {
    ws();
    const size_t start = i;
    Json v;
    if (i >= s.size()) throw std::runtime_error("unexpected end of JSON");
    const char c = s[i];
    if (c == '{') {
      v.kind = Json::Object;
      ++i;
      ws();
      while (i < s.size() && s[i] != '}') {
        Json k = value();
        ws();
        if (s[i] != ':') throw std::runtime_error("expected ':' in JSON");
        ++i;
        v.obj[k.str] = value();
        ws();
        if (s[i] == ',') ++i;
        ws();
      }
      ++i;
    } else if (c == '[') {
      v.kind = Json::Array;
      ++i;
      ws();
      while (i < s.size() && s[i] != ']') {
        v.arr.push_back(value());
        ws();
        if (s[i] == ',') ++i;
        ws();
      }
      ++i;
    } else if (c == '"') {
      v.kind = Json::String;
      ++i;
      while (i < s.size() && s[i] != '"') v.str += s[i++];
      ++i;
    } else if (s.compare(i, 4, "true") == 0 || s.compare(i, 5, "false") == 0) {
      v.kind = Json::Bool;
      v.b = s[i] == 't';
      i += v.b ? 4 : 5;
    } else if (s.compare(i, 4, "null") == 0) {
      i += 4;
    } else {
      v.kind = Json::Number;
      size_t j = i;
      while (j < s.size() && (std::isdigit(static_cast<unsigned char>(s[j])) || std::strchr("+-.eE", s[j]))) ++j;
      v.num = std::strtod(s.substr(i, j - i).c_str(), nullptr);
      i = j;
    }
    v.raw = s.substr(start, i - start);
    return v;
  }
};

Json parse(const std::string& text) {
  Parser p{text};
  return p.value();
}

std::vector<icrar::SphericalDirection> directions_from(const Json& v) {
  std::vector<icrar::SphericalDirection> d;
  for (const auto& e : v.arr) {
    if (e.kind != Json::Array || e.arr.size() != 2) throw icrar::invalid_argument_exception("expected [ra, dec]", "directions", __FILE__, __LINE__);
    d.emplace_back(e.arr[0].num, e.arr[1].num);
  }
  return d;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    std::string file, impl = "gb300", interval = "-1", precision = "fp64", directions;
    std::optional<unsigned int> refAnt;
    double minBL = 0.0;
    bool cache = false;
    std::map<std::string, std::string> cli;
    for (int i = 1; i < argc; ++i) {
      const std::string a = argv[i];
      auto next = [&]() -> std::string {
        if (i + 1 >= argc) throw icrar::invalid_argument_exception("missing value", a, __FILE__, __LINE__);
        return argv[++i];
      };
      if (a == "--cache") cli["cache"] = "1";
      else if (a == "--config" || a == "-c") cli["config"] = next();
      else if (a == "-f" || a == "--filePath") cli["file"] = next();
      else if (a == "-i" || a == "--implementation") cli["impl"] = next();
      else if (a == "-d" || a == "--directions") cli["directions"] = next();
      else if (a == "-s" || a == "--solutionInterval") cli["interval"] = next();
      else if (a == "-a" || a == "--referenceAntenna") cli["refAnt"] = next();
      else if (a == "-m" || a == "--minimumBaselineThreshold") cli["minBL"] = next();
      else if (a == "-p" || a == "--precision") cli["precision"] = next();
      else throw icrar::invalid_argument_exception("unknown option", a, __FILE__, __LINE__);
    }
    if (cli.count("config")) {
      std::ifstream f(cli["config"]);
      if (!f) throw icrar::file_exception(cli["config"], "cannot open config", __FILE__, __LINE__);
      std::stringstream ss;
      ss << f.rdbuf();
      const Json cfg = parse(ss.str());
      auto has = [&](const char* k) { return cfg.obj.count(k) != 0; };
      if (has("filePath")) file = cfg.obj.at("filePath").str;
      if (has("computeImplementation")) impl = cfg.obj.at("computeImplementation").str;
      if (has("directions")) directions = cfg.obj.at("directions").raw;
      if (has("solutionInterval")) interval = cfg.obj.at("solutionInterval").raw;
      if (has("referenceAntenna")) refAnt = static_cast<unsigned int>(cfg.obj.at("referenceAntenna").num);
      if (has("minimumBaselineThreshold")) minBL = cfg.obj.at("minimumBaselineThreshold").num;
      if (has("useFileSystemCache")) cache = cfg.obj.at("useFileSystemCache").b;
      if (has("precision")) precision = cfg.obj.at("precision").str;
    }
    if (cli.count("file")) file = cli["file"];
    if (cli.count("impl")) impl = cli["impl"];
    if (cli.count("directions")) directions = cli["directions"];
    if (cli.count("interval")) interval = cli["interval"];
    if (cli.count("refAnt")) refAnt = static_cast<unsigned int>(std::stoul(cli["refAnt"]));
    if (cli.count("minBL")) minBL = std::stod(cli["minBL"]);
    if (cli.count("precision")) precision = cli["precision"];
    if (cli.count("cache")) cache = true;

    icrar::ComputeImplementation ci;
    if (!icrar::TryParseComputeImplementation(impl, ci))
      throw icrar::invalid_argument_exception("unknown compute implementation " + impl, "implementation", __FILE__, __LINE__);
    icrar::gb300::GpuOptions opt;
    if (precision == "mixed") opt.precision = LEAP_PRECISION_MIXED;
    else if (precision != "fp64") throw icrar::invalid_argument_exception("precision must be fp64 or mixed", "precision", __FILE__, __LINE__);
    if (file.empty()) throw icrar::invalid_argument_exception("no measurement set given", "filePath", __FILE__, __LINE__);
    if (directions.empty()) throw icrar::invalid_argument_exception("no directions given", "directions", __FILE__, __LINE__);

    // Arguments are validated and the measurement set opened before the
    // calibrator is created, as in the reference CLI (main.cc:120-125).
    const auto dirs = directions_from(parse(directions));
    const icrar::Slice slice = icrar::ParseSlice(interval);
    const icrar::MeasurementSet ms(file);
    auto calibrator = icrar::LeapCalibratorFactory::Create(ci, opt);
    const auto result = calibrator->Calibrate(ms, dirs, slice, minBL, refAnt, cache);
    result.Serialize(std::cout);
    return 0;
  } catch (const std::exception& e) {
    std::cerr << e.what() << std::endl;
    return -1;
  }
}
