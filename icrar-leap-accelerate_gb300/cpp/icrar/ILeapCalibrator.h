// icrar::ILeapCalibrator (LA/algorithm/ILeapCalibrator.h:46-69): the interface a
// LEAP calibration implementation sits behind.  Same arguments and meaning;
// boost::optional becomes std::optional.
#pragma once

#include <optional>
#include <vector>

#include "MeasurementSet.h"
#include "Slice.h"
#include "SphericalDirection.h"
#include "calibration.h"

namespace icrar {

class ILeapCalibrator {
 public:
  virtual ~ILeapCalibrator() = default;
  ILeapCalibrator() = default;
  ILeapCalibrator(const ILeapCalibrator&) = delete;
  ILeapCalibrator& operator=(const ILeapCalibrator&) = delete;

  // ms: the measurements; directions: the directions to calibrate for;
  // solutionInterval: timesteps per solution; minimumBaselineThreshold: the
  // shortest baseline (metres) used; referenceAntenna: the reference antenna of
  // matrix A1 (default: the last antenna); isFileSystemCacheEnabled: cache the
  // pseudoinverse of A in the working directory.
  virtual cpu::CalibrationCollection Calibrate(const MeasurementSet& ms, const std::vector<SphericalDirection>& directions,
                                               const Slice& solutionInterval, double minimumBaselineThreshold,
                                               std::optional<unsigned int> referenceAntenna,
                                               bool isFileSystemCacheEnabled) = 0;
};

}  // namespace icrar
