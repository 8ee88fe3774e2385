#include "LeapCalibratorFactory.h"

#include "exception.h"

namespace icrar {

std::unique_ptr<ILeapCalibrator> LeapCalibratorFactory::Create(ComputeImplementation impl) {
  return Create(impl, gb300::GpuOptions{});
}

std::unique_ptr<ILeapCalibrator> LeapCalibratorFactory::Create(ComputeImplementation impl,
                                                               const gb300::GpuOptions& options) {
  switch (impl) {
    case ComputeImplementation::gb300:
      return std::make_unique<gb300::GpuLeapCalibrator>(options);
    case ComputeImplementation::cpu:
      throw invalid_argument_exception("cpu implementation not built in this library", "impl", __FILE__, __LINE__);
    case ComputeImplementation::cuda:
      throw invalid_argument_exception("cuda build option not enabled", "impl", __FILE__, __LINE__);
  }
  throw invalid_argument_exception("invalid argument", "impl", __FILE__, __LINE__);
}

}  // namespace icrar
