#include "GpuLeapCalibrator.h"

#include <complex>
#include <string>

#include "MetaData.h"
#include "exception.h"

namespace icrar {
namespace gb300 {

namespace {
void check(int rc, leap_ctx* ctx, const char* what) {
  if (rc == LEAP_OK) return;
  const std::string msg = std::string(what) + ": " + leap_last_error(ctx);
  if (rc == LEAP_ERR_INVALID_ARGUMENT) throw invalid_argument_exception(msg, what, __FILE__, __LINE__);
  throw icrar::exception(msg, __FILE__, __LINE__);
}
}  // namespace

GpuLeapCalibrator::GpuLeapCalibrator(GpuOptions options) : m_options(options) {
  check(leap_create(options.device, &m_ctx), nullptr, "leap_create");
}

GpuLeapCalibrator::~GpuLeapCalibrator() { leap_destroy(m_ctx); }

cpu::CalibrationCollection GpuLeapCalibrator::Calibrate(const MeasurementSet& ms,
                                                        const std::vector<SphericalDirection>& directions,
                                                        const Slice& solutionInterval, double minimumBaselineThreshold,
                                                        std::optional<unsigned int> referenceAntenna,
                                                        bool isFileSystemCacheEnabled) {
  const int timesteps = static_cast<int>(ms.GetNumTimesteps());
  const Range interval = solutionInterval.Evaluate(timesteps);
  const std::vector<double> epochs = ms.GetEpochs();
  const bool onDevice = m_options.deviceMetadata && !isFileSystemCacheEnabled;
  const cpu::MetaData metadata =
      onDevice ? cpu::MetaData(ms, referenceAntenna, minimumBaselineThreshold, cpu::MetaData::ConstantsOnly{})
               : cpu::MetaData(ms, referenceAntenna, minimumBaselineThreshold, isFileSystemCacheEnabled);
  const leap_constants k = metadata.GetConstants().ToAbi();
  int32_t S = 0;
  if (onDevice) {
    int32_t hostPath = 0;
    check(leap_build_metadata(m_ctx, &k, metadata.GetAntenna1().data(), metadata.GetAntenna2().data(),
                              metadata.GetBaselineFlags().data(), static_cast<int32_t>(k.nbaselines), &hostPath),
          m_ctx, "leap_build_metadata");
    check(leap_get_metadata_matrix(m_ctx, 0, nullptr, 0, &S, nullptr), m_ctx, "leap_get_metadata_matrix");
  } else {
    check(leap_set_metadata(m_ctx, &k, metadata.GetA().data(), metadata.GetARows(), metadata.GetStations(),
                            metadata.GetI().data(), metadata.GetAd().data(), metadata.GetA1().data(),
                            metadata.GetA1Rows(), metadata.GetI1().data(), metadata.GetAd1().data()),
          m_ctx, "leap_set_metadata");
    S = metadata.GetStations();
  }

  std::vector<double> dd(9 * directions.size());
  for (size_t i = 0; i < directions.size(); ++i) {
    const auto m = metadata.GenerateDDMatrix(directions[i]);
    std::copy(m.begin(), m.end(), dd.begin() + 9 * i);
  }
  const uint32_t nbl = ms.GetNumBaselines();
  const uint32_t C = ms.GetNumChannels(), P = ms.GetNumPols();
  const int32_t visType = ms.HasFloatData() ? LEAP_VIS_C64 : LEAP_VIS_C128;
  const int solutions = interval.GetSize();
  // Solution intervals go up double-buffered: interval s + 1 is queued on the library's copy
  // stream (slot (s + 1) % 2) while interval s calibrates, as the reference's loop would if it
  // overlapped its per-interval uploads (CudaLeapCalibrator.cu:159-227).  The transpose from
  // MeasurementSet order runs on the device; the UVWs of an interval stay alive in uvw[slot]
  // until the call that reads the slot has returned.  A library that cannot queue an upload from
  // this memory (pageable memory on a device that does not read it in place) takes each interval
  // synchronously instead.
  std::vector<double> uvw[2];
  bool overlap = solutions > 1;
  auto upload = [&](int s, int slot, bool async) -> int32_t {
    // Integration start row ignores Slice.start, as the reference does (CpuLeapCalibrator.cc:116).
    const uint32_t startRow = static_cast<uint32_t>(s) * interval.interval * nbl;
    const uint32_t rows = static_cast<uint32_t>(interval.interval) * nbl;
    uvw[slot] = ms.GetCoords(startRow, rows);
    return (async ? leap_set_integration_ms_async : leap_set_integration_ms)(
        m_ctx, slot, visType, ms.GetRawVis(startRow), C, 0, uvw[slot].data(), rows, C, P, LEAP_MEMORY_HOST);
  };
  if (overlap) {
    const int32_t rc = upload(0, 0, true);
    if (rc == LEAP_ERR_INVALID_ARGUMENT) overlap = false;
    else check(rc, m_ctx, "leap_set_integration_ms_async");
  }
  std::vector<cpu::Calibration> output;
  std::vector<double> cal(static_cast<size_t>(S) * directions.size());
  for (int s = 0; s < solutions; ++s) {
    output.emplace_back(epochs[static_cast<size_t>(s) * interval.interval],
                        epochs[static_cast<size_t>(s + 1) * interval.interval - 1]);
    const int slot = overlap ? s % 2 : 0;
    if (!overlap) check(upload(s, 0, false), m_ctx, "leap_set_integration_ms");
    // The next interval's slot was last read by calibration s - 1, which has returned.
    if (overlap && s + 1 < solutions) check(upload(s + 1, (s + 1) % 2, true), m_ctx, "leap_set_integration_ms_async");
    check(leap_calibrate(m_ctx, slot, dd.data(), static_cast<int32_t>(directions.size()), m_options.precision,
                         cal.data()),
          m_ctx, "leap_calibrate");
    for (size_t i = 0; i < directions.size(); ++i)
      output.back().GetBeamCalibrations().emplace_back(
          directions[i], std::vector<double>(cal.begin() + static_cast<std::ptrdiff_t>(S * i),
                                             cal.begin() + static_cast<std::ptrdiff_t>(S * (i + 1))));
  }
  if (overlap && solutions > 1) leap_release_integration(m_ctx, 1);
  leap_release_integration(m_ctx, 0);
  return cpu::CalibrationCollection(std::move(output));
}

}  // namespace gb300
}  // namespace icrar
