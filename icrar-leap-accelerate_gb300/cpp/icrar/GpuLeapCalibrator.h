// GB300 implementation of ILeapCalibrator: the reference's calibration loop
// (CudaLeapCalibrator::Calibrate, LA/algorithm/cuda/CudaLeapCalibrator.cu:94-233)
// on the leap_gb300 C ABI.  MetaData once; then per solution interval one
// resident integration and ONE call for all directions (the reference
// re-uploads the integration and launches per direction).
#pragma once

#include "ILeapCalibrator.h"
#include "leap_gb300.h"

namespace icrar {
namespace gb300 {

struct GpuOptions {
  int device = 0;
  int precision = LEAP_PRECISION_FP64;  // LEAP_PRECISION_FP64 (reference-faithful) or LEAP_PRECISION_MIXED
  // Build A, A1 and their pseudo-inverses on the device (leap_build_metadata) unless the
  // file cache is requested, which keeps the host path and its A.hash / Ad.cache files.
  bool deviceMetadata = true;
};

class GpuLeapCalibrator : public ILeapCalibrator {
 public:
  explicit GpuLeapCalibrator(GpuOptions options = {});
  ~GpuLeapCalibrator() override;

  cpu::CalibrationCollection Calibrate(const MeasurementSet& ms, const std::vector<SphericalDirection>& directions,
                                       const Slice& solutionInterval, double minimumBaselineThreshold,
                                       std::optional<unsigned int> referenceAntenna,
                                       bool isFileSystemCacheEnabled) override;

 private:
  GpuOptions m_options;
  leap_ctx* m_ctx = nullptr;
};

}  // namespace gb300
}  // namespace icrar
