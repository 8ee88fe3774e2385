#include "MeasurementSet.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iostream>

#include "exception.h"

// ".leapms" file: little-endian
//   char[8]  "LEAPMS01"
//   uint32   stations, totalAntennas, rows, channels, pols, isDouble
//   double   refFrequency, chanWidth, phaseCentreRa, phaseCentreDec
//   int32    antenna1[rows], antenna2[rows]
//   uint8    flag[rows]
//   double   time[rows], uvw[rows*3]
//   complex  data[rows*channels*pols]  (float pairs, or double pairs if isDouble)

namespace icrar {

namespace {
template <typename T>
void read_vec(std::ifstream& f, std::vector<T>& v, size_t n, const std::string& path) {
  v.resize(n);
  if (n && !f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(sizeof(T) * n)))
    throw file_exception(path, "truncated file", __FILE__, __LINE__);
}
template <typename T>
void write_vec(std::ofstream& f, const std::vector<T>& v) {
  if (!v.empty()) f.write(reinterpret_cast<const char*>(v.data()), static_cast<std::streamsize>(sizeof(T) * v.size()));
}
}  // namespace

MeasurementSet::MeasurementSet(const std::string& filepath, std::optional<int> overrideNStations,
                               bool readAutocorrelations)
    : m_readAutocorrelations(readAutocorrelations), m_filepath(filepath) {
  std::ifstream f(filepath, std::ios::binary);
  if (!f) throw file_exception(filepath, "cannot open", __FILE__, __LINE__);
  char magic[8];
  f.read(magic, 8);
  if (!f || std::memcmp(magic, "LEAPMS01", 8) != 0) throw file_exception(filepath, "not a .leapms file", __FILE__, __LINE__);
  uint32_t hdr[6];
  double hd[4];
  f.read(reinterpret_cast<char*>(hdr), sizeof(hdr));
  f.read(reinterpret_cast<char*>(hd), sizeof(hd));
  if (!f) throw file_exception(filepath, "truncated header", __FILE__, __LINE__);
  MeasurementSetData& d = m_data;
  d.stations = hdr[0];
  d.totalAntennas = hdr[1];
  const uint32_t rows = hdr[2];
  d.channels = hdr[3];
  d.pols = hdr[4];
  const bool isDouble = hdr[5] != 0;
  d.refFrequency = hd[0];
  d.chanWidth = hd[1];
  d.phaseCentreRa = hd[2];
  d.phaseCentreDec = hd[3];
  read_vec(f, d.antenna1, rows, filepath);
  read_vec(f, d.antenna2, rows, filepath);
  read_vec(f, d.flag, rows, filepath);
  read_vec(f, d.time, rows, filepath);
  read_vec(f, d.uvw, static_cast<size_t>(rows) * 3, filepath);
  const size_t n = static_cast<size_t>(rows) * d.channels * d.pols;
  if (isDouble) read_vec(f, d.data64, n, filepath);
  else read_vec(f, d.data32, n, filepath);
  m_stations = overrideNStations ? static_cast<uint32_t>(*overrideNStations) : d.stations;
  Validate();
}

MeasurementSet::MeasurementSet(MeasurementSetData data, bool readAutocorrelations)
    : m_data(std::move(data)), m_readAutocorrelations(readAutocorrelations) {
  m_stations = m_data.stations;
  Validate();
}

// MeasurementSet::Validate (LA/ms/MeasurementSet.cc:64-103).
void MeasurementSet::Validate() const {
  const uint32_t nbl = GetNumBaselines();
  const size_t rows = m_data.antenna1.size();
  if (m_data.antenna2.size() != rows || m_data.flag.size() != rows || m_data.time.size() != rows ||
      m_data.uvw.size() != rows * 3)
    throw exception("inconsistent column lengths", __FILE__, __LINE__);
  const size_t nvis = m_data.data32.empty() ? m_data.data64.size() : m_data.data32.size();
  if (nvis != rows * m_data.channels * m_data.pols) throw exception("DATA size does not match rows x channels x pols", __FILE__, __LINE__);
  if (rows) {
    const double epoch = m_data.time[0];
    const size_t epochRows = static_cast<size_t>(std::count(m_data.time.begin(), m_data.time.end(), epoch));
    if (epochRows != nbl)
      throw exception("visibilities at first epoch does not match number of baselines", __FILE__, __LINE__);
  }
  if (rows < nbl)
    throw file_exception(m_filepath.value_or("unknown"), "invalid number of rows, expected >=" + std::to_string(nbl),
                         __FILE__, __LINE__);
  if (nbl == 0 || rows % nbl != 0) throw exception("number of rows not an integer multiple of baselines", __FILE__, __LINE__);
}

uint32_t MeasurementSet::GetNumBaselines(bool useAutocorrelations) const {
  const uint32_t s = GetNumStations();
  return useAutocorrelations ? s * (s + 1) / 2 : s * (s - 1) / 2;
}

std::vector<double> MeasurementSet::GetEpochs() const {
  std::vector<double> e;
  const uint32_t nbl = GetNumBaselines();
  for (uint32_t t = 0; t < GetNumTimesteps(); ++t) e.push_back(m_data.time[static_cast<size_t>(t) * nbl]);
  return e;
}

std::vector<int32_t> MeasurementSet::GetAntenna1() const {
  return std::vector<int32_t>(m_data.antenna1.begin(), m_data.antenna1.begin() + GetNumBaselines());
}
std::vector<int32_t> MeasurementSet::GetAntenna2() const {
  return std::vector<int32_t>(m_data.antenna2.begin(), m_data.antenna2.begin() + GetNumBaselines());
}

std::vector<bool> MeasurementSet::GetFlaggedBaselines() const {
  const uint32_t nbl = GetNumBaselines();
  std::vector<bool> f(nbl);
  for (uint32_t i = 0; i < nbl; ++i) f[i] = m_data.flag[i] != 0;
  return f;
}

uint32_t MeasurementSet::GetNumFlaggedBaselines() const {
  const auto f = GetFlaggedBaselines();
  return static_cast<uint32_t>(std::count(f.begin(), f.end(), true));
}

std::vector<bool> MeasurementSet::GetShortBaselines(double minimumBaselineThreshold) const {
  const uint32_t nbl = GetNumBaselines();
  std::vector<bool> f(nbl, false);
  if (minimumBaselineThreshold > 0.0) {
    for (uint32_t i = 0; i < nbl; ++i) {
      const double u = m_data.uvw[3 * static_cast<size_t>(i)], v = m_data.uvw[3 * static_cast<size_t>(i) + 1];
      if (std::sqrt(u * u + v * v) < minimumBaselineThreshold) f[i] = true;
    }
  }
  return f;
}

uint32_t MeasurementSet::GetNumShortBaselines(double minimumBaselineThreshold) const {
  const auto f = GetShortBaselines(minimumBaselineThreshold);
  return static_cast<uint32_t>(std::count(f.begin(), f.end(), true));
}

std::vector<bool> MeasurementSet::GetFilteredBaselines(double minimumBaselineThreshold) const {
  auto a = GetFlaggedBaselines();
  const auto b = GetShortBaselines(minimumBaselineThreshold);
  for (size_t i = 0; i < a.size(); ++i) a[i] = a[i] || b[i];
  return a;
}

uint32_t MeasurementSet::GetNumFilteredBaselines(double minimumBaselineThreshold) const {
  const auto f = GetFilteredBaselines(minimumBaselineThreshold);
  return static_cast<uint32_t>(std::count(f.begin(), f.end(), true));
}

std::vector<double> MeasurementSet::GetCoords(uint32_t startRow, uint32_t n) const {
  const uint32_t rows = GetNumRows();
  if (startRow >= rows) throw exception("ms out of range", __FILE__, __LINE__);
  n = std::min(n, rows - startRow);
  return std::vector<double>(m_data.uvw.begin() + 3 * static_cast<size_t>(startRow),
                             m_data.uvw.begin() + 3 * (static_cast<size_t>(startRow) + n));
}

namespace {
template <typename Out, typename In>
std::vector<Out> transpose_vis(const std::vector<In>& data, uint32_t rowsTotal, uint32_t channels, uint32_t pols,
                               uint32_t startRow, uint32_t startChannel, uint32_t nChannels, uint32_t nRows,
                               uint32_t nPols) {
  if (startRow >= rowsTotal) throw exception("ms out of range", __FILE__, __LINE__);
  if (startRow + nRows > rowsTotal) throw exception("row selection exceeds total range", __FILE__, __LINE__);
  if (startChannel + nChannels > channels || nPols > pols) throw exception("channel or pol selection out of range", __FILE__, __LINE__);
  std::vector<Out> out(static_cast<size_t>(nChannels) * nRows * nPols);
  for (uint32_t c = 0; c < nChannels; ++c)
    for (uint32_t r = 0; r < nRows; ++r)
      for (uint32_t p = 0; p < nPols; ++p)
        out[p + static_cast<size_t>(nPols) * (r + static_cast<size_t>(nRows) * c)] =
            Out(data[(static_cast<size_t>(startRow + r) * channels + startChannel + c) * pols + p]);
  return out;
}
}  // namespace

std::vector<std::complex<double>> MeasurementSet::GetVis(uint32_t startRow, uint32_t startChannel, uint32_t nChannels,
                                                         uint32_t nRows, uint32_t nPols) const {
  if (HasFloatData())
    return transpose_vis<std::complex<double>>(m_data.data32, GetNumRows(), m_data.channels, m_data.pols, startRow,
                                               startChannel, nChannels, nRows, nPols);
  return transpose_vis<std::complex<double>>(m_data.data64, GetNumRows(), m_data.channels, m_data.pols, startRow,
                                             startChannel, nChannels, nRows, nPols);
}

std::vector<std::complex<float>> MeasurementSet::GetVisF32(uint32_t startRow, uint32_t startChannel, uint32_t nChannels,
                                                           uint32_t nRows, uint32_t nPols) const {
  if (!HasFloatData()) throw exception("DATA is complex<double>", __FILE__, __LINE__);
  return transpose_vis<std::complex<float>>(m_data.data32, GetNumRows(), m_data.channels, m_data.pols, startRow,
                                            startChannel, nChannels, nRows, nPols);
}

void WriteMeasurementSet(const std::string& filepath, const MeasurementSetData& d) {
  std::ofstream f(filepath, std::ios::binary);
  if (!f) throw file_exception(filepath, "cannot create", __FILE__, __LINE__);
  f.write("LEAPMS01", 8);
  const uint32_t hdr[6] = {d.stations, d.totalAntennas, static_cast<uint32_t>(d.antenna1.size()), d.channels, d.pols,
                           d.data32.empty() ? 1u : 0u};
  const double hd[4] = {d.refFrequency, d.chanWidth, d.phaseCentreRa, d.phaseCentreDec};
  f.write(reinterpret_cast<const char*>(hdr), sizeof(hdr));
  f.write(reinterpret_cast<const char*>(hd), sizeof(hd));
  write_vec(f, d.antenna1);
  write_vec(f, d.antenna2);
  write_vec(f, d.flag);
  write_vec(f, d.time);
  write_vec(f, d.uvw);
  if (d.data32.empty()) write_vec(f, d.data64);
  else write_vec(f, d.data32);
}

}  // namespace icrar
