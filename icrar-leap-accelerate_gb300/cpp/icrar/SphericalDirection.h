// Calibration direction (ra, dec) in radians: icrar::SphericalDirection
// (LA/common/SphericalDirection.h:32, an Eigen::Vector2d in the reference).
#pragma once

#include <array>

namespace icrar {

class SphericalDirection {
 public:
  SphericalDirection() = default;
  SphericalDirection(double ra, double dec) : m_v{ra, dec} {}
  double operator()(int i) const { return m_v[i]; }
  double& operator()(int i) { return m_v[i]; }
  const double* begin() const { return m_v.data(); }
  const double* end() const { return m_v.data() + 2; }
  bool operator==(const SphericalDirection& o) const { return m_v == o.m_v; }

 private:
  std::array<double, 2> m_v{0.0, 0.0};
};

}  // namespace icrar
