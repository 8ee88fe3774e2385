// A MeasurementSet stand-in exposing the accessors the calibration path uses
// (icrar::MeasurementSet, LA/ms/MeasurementSet.h:54-224).  casacore is not
// available, so the data comes from memory or from a ".leapms" file (see
// MeasurementSet.cc for the format).  Rows are timestep-major (row = t*nbl + b)
// with the same baseline order in every timestep, as the reference assumes;
// DATA is stored as the MS stores it, [row][channel][pol] complex values.
#pragma once

#include <complex>
#include <cstdint>
#include <optional>
#include <string>
#include <vector>

namespace icrar {

struct MeasurementSetData {
  uint32_t stations = 0;        // number of stations (unique antennas)
  uint32_t totalAntennas = 0;   // rows of the ANTENNA table
  uint32_t channels = 0;
  uint32_t pols = 0;
  double refFrequency = 0.0;    // SPECTRAL_WINDOW REF_FREQUENCY (Hz)
  double chanWidth = 0.0;       // SPECTRAL_WINDOW CHAN_WIDTH[0] (Hz)
  double phaseCentreRa = 0.0;   // FIELD PHASE_DIR (rad)
  double phaseCentreDec = 0.0;
  std::vector<int32_t> antenna1, antenna2;  // per row
  std::vector<uint8_t> flag;                // per row: FLAG of channel 0, pol 0
  std::vector<double> time;                 // per row (s)
  std::vector<double> uvw;                  // per row: u, v, w (m)
  std::vector<std::complex<float>> data32;  // [row][channel][pol] when stored as complex<float>
  std::vector<std::complex<double>> data64; // [row][channel][pol] when stored as complex<double>
};

class MeasurementSet {
 public:
  // Load a ".leapms" file.  overrideNStations and readAutocorrelations have the
  // reference's meaning (LA/ms/MeasurementSet.cc:33-62).
  MeasurementSet(const std::string& filepath, std::optional<int> overrideNStations = std::nullopt,
                 bool readAutocorrelations = true);
  MeasurementSet(MeasurementSetData data, bool readAutocorrelations = true);

  uint32_t GetNumStations() const { return m_stations; }
  uint32_t GetTotalAntennas() const { return m_data.totalAntennas; }
  uint32_t GetNumPols() const { return m_data.pols; }
  uint32_t GetNumChannels() const { return m_data.channels; }
  uint32_t GetNumRows() const { return static_cast<uint32_t>(m_data.antenna1.size()); }
  uint32_t GetNumBaselines() const { return GetNumBaselines(m_readAutocorrelations); }
  uint32_t GetNumBaselines(bool useAutocorrelations) const;
  uint32_t GetNumTimesteps() const { return GetNumRows() / GetNumBaselines(); }
  std::vector<double> GetEpochs() const;
  double GetRefFrequency() const { return m_data.refFrequency; }
  double GetChanWidth() const { return m_data.chanWidth; }
  double GetPhaseCentreRa() const { return m_data.phaseCentreRa; }
  double GetPhaseCentreDec() const { return m_data.phaseCentreDec; }
  const std::optional<std::string>& GetFilepath() const { return m_filepath; }

  // First-epoch antenna columns (rows [0, nbl)).
  std::vector<int32_t> GetAntenna1() const;
  std::vector<int32_t> GetAntenna2() const;

  std::vector<bool> GetFlaggedBaselines() const;                          // MeasurementSet.cc:181-197
  uint32_t GetNumFlaggedBaselines() const;
  std::vector<bool> GetShortBaselines(double minimumBaselineThreshold) const;  // :205-228
  uint32_t GetNumShortBaselines(double minimumBaselineThreshold) const;
  std::vector<bool> GetFilteredBaselines(double minimumBaselineThreshold) const;  // :236-240
  uint32_t GetNumFilteredBaselines(double minimumBaselineThreshold) const;

  // UVW of rows [startRow, startRow + n), n x 3 row-major (ms_read_coords, LA/ms/utils.h:44-78).
  std::vector<double> GetCoords(uint32_t startRow, uint32_t n) const;

  // Visibilities of rows [startRow, startRow + nRows), channels [startChannel,
  // startChannel + nChannels), pols [0, nPols), transposed to the Integration
  // layout (pol, row, channel) column-major (ms_read_vis, LA/ms/utils.h:81-146).
  std::vector<std::complex<double>> GetVis(uint32_t startRow, uint32_t startChannel, uint32_t nChannels,
                                           uint32_t nRows, uint32_t nPols) const;
  // The same without widening, for complex<float> DATA.
  std::vector<std::complex<float>> GetVisF32(uint32_t startRow, uint32_t startChannel, uint32_t nChannels,
                                             uint32_t nRows, uint32_t nPols) const;
  bool HasFloatData() const { return !m_data.data32.empty(); }
  // DATA in the MeasurementSet's own order, [row][channel][pol], from row startRow
  // (what casacore hands out for the DATA column); the device transposes it.
  const void* GetRawVis(uint32_t startRow) const {
    const size_t off = static_cast<size_t>(startRow) * m_data.channels * m_data.pols;
    return HasFloatData() ? static_cast<const void*>(m_data.data32.data() + off)
                          : static_cast<const void*>(m_data.data64.data() + off);
  }

  const MeasurementSetData& GetData() const { return m_data; }

 private:
  void Validate() const;
  MeasurementSetData m_data;
  uint32_t m_stations = 0;
  bool m_readAutocorrelations = true;
  std::optional<std::string> m_filepath;
};

// Write a ".leapms" file (used by tests and tools to hand data to the C++ path).
void WriteMeasurementSet(const std::string& filepath, const MeasurementSetData& data);

}  // namespace icrar
