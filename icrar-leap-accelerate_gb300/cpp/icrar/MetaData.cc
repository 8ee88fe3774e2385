#include "MetaData.h"

#include <cstring>
#include <fstream>
#include <iostream>
#include <string>

#include "exception.h"

namespace icrar {
namespace cpu {

leap_constants Constants::ToAbi() const {
  leap_constants k{};
  k.nbaselines = nbaselines;
  k.referenceAntenna = referenceAntenna;
  k.channels = channels;
  k.num_pols = num_pols;
  k.stations = stations;
  k.rows = rows;
  k.freq_start_hz = freq_start_hz;
  k.freq_inc_hz = freq_inc_hz;
  k.phase_centre_ra_rad = phase_centre_ra_rad;
  k.phase_centre_dec_rad = phase_centre_dec_rad;
  k.dlm_ra = dlm_ra;
  k.dlm_dec = dlm_dec;
  return k;
}

namespace {

void throw_status(int rc, const std::string& what) {
  const char* msg = leap_last_error(nullptr);
  if (rc == LEAP_ERR_INVALID_ARGUMENT) throw invalid_argument_exception(msg ? msg : "", what, __FILE__, __LINE__);
  throw icrar::exception(what + ": " + (msg ? msg : ""), __FILE__, __LINE__);
}

void phase_matrix(const std::vector<int32_t>& a1, const std::vector<int32_t>& a2, const std::vector<uint8_t>& fg,
                  std::optional<unsigned int> ref, std::vector<double>& A, std::vector<int32_t>& I, int32_t& rows,
                  int32_t& cols) {
  const int32_t n = static_cast<int32_t>(a1.size());
  int32_t maxc = 0;
  for (int32_t i = 0; i < n; ++i) maxc = std::max(maxc, std::max(a1[i], a2[i]));
  A.assign(static_cast<size_t>(n + 1) * (maxc + 1), 0.0);
  I.assign(std::max(n, 1), 0);
  const int rc = leap_phase_matrix(a1.data(), a2.data(), fg.data(), n, ref ? static_cast<int32_t>(*ref) : -1, A.data(),
                                   I.data(), &rows, &cols);
  if (rc != LEAP_OK) throw_status(rc, "refAnt");
  A.resize(static_cast<size_t>(rows) * cols);
  I.resize(rows - 1);
}

std::vector<double> pinv(const std::vector<double>& A, int32_t rows, int32_t cols) {
  std::vector<double> Ad(static_cast<size_t>(rows) * cols);
  const int rc = leap_pseudo_inverse(A.data(), rows, cols, Ad.data());
  if (rc != LEAP_OK) throw_status(rc, "A");
  return Ad;
}

// FNV-1a of the matrix bytes and shape: the cache key (the reference uses a
// hash of A, LA/common/eigen_extensions.h:48-64).
uint64_t matrix_hash(const std::vector<double>& A, int32_t rows, int32_t cols) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  };
  mix(&rows, sizeof(rows));
  mix(&cols, sizeof(cols));
  mix(A.data(), A.size() * sizeof(double));
  return h;
}

}  // namespace

void MetaData::SetConstants(const MeasurementSet& ms, std::optional<unsigned int> refAnt,
                            double minimumBaselineThreshold) {
  m_constants.nbaselines = ms.GetNumBaselines();
  m_constants.referenceAntenna = refAnt ? *refAnt : ms.GetTotalAntennas() - 1;
  m_constants.channels = ms.GetNumChannels();
  m_constants.freq_start_hz = ms.GetRefFrequency();
  m_constants.freq_inc_hz = ms.GetChanWidth();
  m_constants.rows = ms.GetNumRows();
  m_constants.num_pols = ms.GetNumPols();
  m_constants.stations = ms.GetNumStations();
  m_constants.phase_centre_ra_rad = ms.GetPhaseCentreRa();
  m_constants.phase_centre_dec_rad = ms.GetPhaseCentreDec();

  const auto filtered = ms.GetFilteredBaselines(minimumBaselineThreshold);
  m_fg.assign(filtered.begin(), filtered.end());
  m_a1 = ms.GetAntenna1();
  m_a2 = ms.GetAntenna2();
}

MetaData::MetaData(const MeasurementSet& ms, std::optional<unsigned int> refAnt, double minimumBaselineThreshold,
                   ConstantsOnly) {
  SetConstants(ms, refAnt, minimumBaselineThreshold);
}

MetaData::MetaData(const MeasurementSet& ms, std::optional<unsigned int> refAnt, double minimumBaselineThreshold,
                   bool useCache) {
  SetConstants(ms, refAnt, minimumBaselineThreshold);
  const auto& fg = m_fg;
  const auto& a1 = m_a1;
  const auto& a2 = m_a2;
  int32_t cols1 = 0, cols = 0;
  phase_matrix(a1, a2, fg, m_constants.referenceAntenna, m_A1, m_I1, m_A1rows, cols1);
  phase_matrix(a1, a2, fg, std::nullopt, m_A, m_I, m_Arows, cols);
  m_S = cols;
  m_Ad1 = pinv(m_A1, m_A1rows, cols1);
  if (useCache) {
    const uint64_t h = matrix_hash(m_A, m_Arows, cols);
    uint64_t cached = 0;
    std::ifstream fh("A.hash", std::ios::binary);
    bool hit = fh && fh.read(reinterpret_cast<char*>(&cached), sizeof(cached)) && cached == h;
    if (hit) {
      std::ifstream fc("Ad.cache", std::ios::binary);
      m_Ad.resize(static_cast<size_t>(m_Arows) * cols);
      hit = fc && fc.read(reinterpret_cast<char*>(m_Ad.data()), static_cast<std::streamsize>(m_Ad.size() * sizeof(double)));
    }
    if (!hit) {
      m_Ad = pinv(m_A, m_Arows, cols);
      std::ofstream oh("A.hash", std::ios::binary);
      oh.write(reinterpret_cast<const char*>(&h), sizeof(h));
      std::ofstream oc("Ad.cache", std::ios::binary);
      oc.write(reinterpret_cast<const char*>(m_Ad.data()), static_cast<std::streamsize>(m_Ad.size() * sizeof(double)));
    }
  } else {
    m_Ad = pinv(m_A, m_Arows, cols);
  }
}

std::array<double, 9> MetaData::GenerateDDMatrix(const SphericalDirection& direction) const {
  std::array<double, 9> dd{};
  leap_dd_matrix(m_constants.phase_centre_ra_rad, m_constants.phase_centre_dec_rad, direction(0), direction(1), dd.data());
  return dd;
}

void MetaData::SetDirection(const SphericalDirection& direction) {
  m_constants.dlm_ra = direction(0) - m_constants.phase_centre_ra_rad;
  m_constants.dlm_dec = direction(1) - m_constants.phase_centre_dec_rad;
}

}  // namespace cpu
}  // namespace icrar
