#include "calibration.h"

#include <cctype>
#include <charconv>
#include <cmath>
#include <cstdlib>

#include "Slice.h"
#include "exception.h"

namespace icrar {
namespace cpu {

std::string FormatDouble(double v) {
  if (!std::isfinite(v)) return std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity");
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), v);
  std::string s(buf, r.ptr);
  if (s.find_first_of(".eE") == std::string::npos) s += ".0";
  return s;
}

void BeamCalibration::Write(std::string& out) const {
  out += "{\"direction\":[";
  out += FormatDouble(m_direction(0)) + "," + FormatDouble(m_direction(1));
  out += "],\"beamCalibration\":[";
  for (size_t i = 0; i < m_calibration.size(); ++i) {
    if (i) out += ",";
    out += FormatDouble(m_calibration[i]);
  }
  out += "]}";
}

void BeamCalibration::Serialize(std::ostream& os) const {
  std::string s;
  Write(s);
  os << s << std::endl;
}

void Calibration::Write(std::string& out) const {
  out += "{\"epoch\":{\"start\":" + FormatDouble(m_startEpoch) + ",\"end\":" + FormatDouble(m_endEpoch) + "},";
  out += "\"calibration\":[";
  for (size_t i = 0; i < m_beamCalibrations.size(); ++i) {
    if (i) out += ",";
    m_beamCalibrations[i].Write(out);
  }
  out += "]}";
}

void Calibration::Serialize(std::ostream& os) const {
  std::string s;
  Write(s);
  os << s << std::endl;
}

void CalibrationCollection::Serialize(std::ostream& os) const {
  std::string s = "[";
  for (size_t i = 0; i < m_calibrations.size(); ++i) {
    if (i) s += ",";
    m_calibrations[i].Write(s);
  }
  s += "]";
  os << s << std::endl;
}

}  // namespace cpu

// ParseSlice (LA/common/Slice.cc:65-110): an integer is an interval; an array of
// two or three integers is [start, end] or [start, interval, end]; null is -1.
Slice ParseSlice(const std::string& json) {
  std::vector<int> v;
  size_t i = 0;
  auto skip = [&] { while (i < json.size() && std::isspace(static_cast<unsigned char>(json[i]))) ++i; };
  auto number = [&]() -> int {
    skip();
    if (json.compare(i, 4, "null") == 0) {
      i += 4;
      return -1;
    }
    size_t j = i;
    if (j < json.size() && (json[j] == '-' || json[j] == '+')) ++j;
    while (j < json.size() && std::isdigit(static_cast<unsigned char>(json[j]))) ++j;
    if (j == i) throw icrar::exception("expected an integer in slice: " + json, __FILE__, __LINE__);
    const int x = std::atoi(json.substr(i, j - i).c_str());
    i = j;
    return x;
  };
  skip();
  if (i < json.size() && json[i] == '[') {
    ++i;
    skip();
    while (i < json.size() && json[i] != ']') {
      v.push_back(number());
      skip();
      if (i < json.size() && json[i] == ',') ++i;
      skip();
    }
    if (v.size() == 2) return Slice(v[0], v[1]);
    if (v.size() == 3) return Slice(v[0], v[1], v[2]);
    throw icrar::exception("expected 2 or 3 elements in slice array", __FILE__, __LINE__);
  }
  return Slice(number());
}

}  // namespace icrar
