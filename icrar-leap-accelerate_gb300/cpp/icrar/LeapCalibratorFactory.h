// icrar::LeapCalibratorFactory (LA/algorithm/LeapCalibratorFactory.cc:30-48) with
// the gb300 value.  cpu and cuda name the reference's own implementations,
// which are not part of this library: asking for them throws
// invalid_argument_exception, as the reference does for a build without CUDA.
#pragma once

#include <memory>

#include "GpuLeapCalibrator.h"
#include "ILeapCalibrator.h"
#include "compute_implementation.h"

namespace icrar {

class LeapCalibratorFactory {
 public:
  static std::unique_ptr<ILeapCalibrator> Create(ComputeImplementation impl);
  static std::unique_ptr<ILeapCalibrator> Create(ComputeImplementation impl, const gb300::GpuOptions& options);
};

}  // namespace icrar
