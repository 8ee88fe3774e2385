// Host-side calibration metadata: cpu::Constants and the phase matrices with
// their pseudoinverses (cpu::MetaData, LA/model/cpu/MetaData.h:76-221,
// MetaData.cc:42-137).  Matrices are column-major std::vector<double>.
#pragma once

#include <array>
#include <cstdint>
#include <optional>
#include <vector>

#include "MeasurementSet.h"
#include "SphericalDirection.h"
#include "leap_gb300.h"

namespace icrar {
namespace cpu {

struct Constants {
  uint32_t nbaselines = 0;
  uint32_t referenceAntenna = 0;
  uint32_t channels = 0;
  uint32_t num_pols = 0;
  uint32_t stations = 0;
  uint32_t rows = 0;
  double freq_start_hz = 0.0;
  double freq_inc_hz = 0.0;
  double phase_centre_ra_rad = 0.0;
  double phase_centre_dec_rad = 0.0;
  double dlm_ra = 0.0;
  double dlm_dec = 0.0;
  double GetChannelWavelength(int i) const { return 299792458.0 / (freq_start_hz + i * freq_inc_hz); }
  leap_constants ToAbi() const;
};

class MetaData {
 public:
  // refAnt default: the last antenna (MetaData.cc:51); useCache: pseudoinverse of
  // A read from / written to "A.hash" + "Ad.cache" in the working directory
  // (ProcessCache, LA/common/eigen_extensions.h:164-199).
  MetaData(const MeasurementSet& ms, std::optional<unsigned int> refAnt, double minimumBaselineThreshold, bool useCache);

  // Constants and the first-epoch baseline columns only (antenna1, antenna2 and the
  // filtered-baseline flags); the matrices are then built on the device
  // (leap_build_metadata).
  struct ConstantsOnly {};
  MetaData(const MeasurementSet& ms, std::optional<unsigned int> refAnt, double minimumBaselineThreshold,
           ConstantsOnly);
  const std::vector<int32_t>& GetAntenna1() const { return m_a1; }
  const std::vector<int32_t>& GetAntenna2() const { return m_a2; }
  const std::vector<uint8_t>& GetBaselineFlags() const { return m_fg; }

  const Constants& GetConstants() const { return m_constants; }
  int32_t GetARows() const { return m_Arows; }
  int32_t GetA1Rows() const { return m_A1rows; }
  int32_t GetStations() const { return m_S; }
  const std::vector<double>& GetA() const { return m_A; }
  const std::vector<int32_t>& GetI() const { return m_I; }
  const std::vector<double>& GetAd() const { return m_Ad; }
  const std::vector<double>& GetA1() const { return m_A1; }
  const std::vector<int32_t>& GetI1() const { return m_I1; }
  const std::vector<double>& GetAd1() const { return m_Ad1; }

  // MetaData::GenerateDDMatrix (MetaData.cc:166-203), row-major 3x3.
  std::array<double, 9> GenerateDDMatrix(const SphericalDirection& direction) const;
  // MetaData::SetDirection (MetaData.cc:205-213): dlm offsets of the direction.
  void SetDirection(const SphericalDirection& direction);

 private:
  Constants m_constants;
  int32_t m_S = 0, m_Arows = 0, m_A1rows = 0;
  std::vector<double> m_A, m_Ad, m_A1, m_Ad1;
  std::vector<int32_t> m_I, m_I1;
  std::vector<int32_t> m_a1, m_a2;
  std::vector<uint8_t> m_fg;
  void SetConstants(const MeasurementSet& ms, std::optional<unsigned int> refAnt, double minimumBaselineThreshold);
};

}  // namespace cpu
}  // namespace icrar
