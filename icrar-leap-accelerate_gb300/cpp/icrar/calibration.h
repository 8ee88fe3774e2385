// Calibration result types (LA/model/cpu/calibration/BeamCalibration.h:45-124,
// Calibration.h:42-111, CalibrationCollection.h:41-82) and their JSON form:
//   [{"epoch":{"start":s,"end":e},"calibration":[{"direction":[ra,dec],"beamCalibration":[...]}]}]
#pragma once

#include <ostream>
#include <string>
#include <vector>

#include "SphericalDirection.h"

namespace icrar {
namespace cpu {

class BeamCalibration {
 public:
  BeamCalibration(SphericalDirection direction, std::vector<double> calibration)
      : m_direction(direction), m_calibration(std::move(calibration)) {}
  const SphericalDirection& GetDirection() const { return m_direction; }
  // Phase calibration of each antenna for the direction (the reference's S x 1 matrix).
  const std::vector<double>& GetPhaseCalibration() const { return m_calibration; }
  void Write(std::string& out) const;
  void Serialize(std::ostream& os) const;

 private:
  SphericalDirection m_direction;
  std::vector<double> m_calibration;
};

class Calibration {
 public:
  Calibration(double startEpoch, double endEpoch) : m_startEpoch(startEpoch), m_endEpoch(endEpoch) {}
  double GetStartEpoch() const { return m_startEpoch; }
  double GetEndEpoch() const { return m_endEpoch; }
  const std::vector<BeamCalibration>& GetBeamCalibrations() const { return m_beamCalibrations; }
  std::vector<BeamCalibration>& GetBeamCalibrations() { return m_beamCalibrations; }
  void Write(std::string& out) const;
  void Serialize(std::ostream& os) const;

 private:
  double m_startEpoch;
  double m_endEpoch;
  std::vector<BeamCalibration> m_beamCalibrations;
};

class CalibrationCollection {
 public:
  explicit CalibrationCollection(std::vector<Calibration> calibrations) : m_calibrations(std::move(calibrations)) {}
  const std::vector<Calibration>& GetCalibrations() const { return m_calibrations; }
  void Serialize(std::ostream& os) const;

 private:
  std::vector<Calibration> m_calibrations;
};

// Shortest decimal text that reads back to the same double (what RapidJSON's
// Writer::Double emits for the reference's output).
std::string FormatDouble(double v);

}  // namespace cpu
}  // namespace icrar
