// geometry.cpp — scalar delay laws and arrival times (behaviour of the
// reference's core/src/geometry.cpp:17-130). Host bookkeeping only: transmit
// delay laws are computed once per transmit, and the per-pixel geometry runs
// inside the CUDA kernels.
#include "usx/geometry.hpp"

#include <algorithm>
#include <cmath>

namespace usx {

void compute_transmit_delays(const Probe& probe, const Medium& medium, Transmit& tx,
                             Window apod_window, real f_number, real* t0_offset) {
  const real c = medium.speed_of_sound;
  const int n = probe.n_elements;
  tx.delays.assign(static_cast<std::size_t>(n), 0.0f);
  tx.apodization.assign(static_cast<std::size_t>(n), 0.0f);
  const Vec3 origin(tx.origin.x, 0.0f, 0.0f);
  // Active half-aperture: f-number limited for focused beams, whole array otherwise.
  real half = 0.5f * probe.aperture_width();
  if (tx.type == TransmitType::Focused)
    half = 0.5f * std::abs(tx.focus.z - origin.z) / std::max(f_number, 0.1f);
  half = std::min(half, 0.5f * probe.aperture_width());

  bool any = false;
  real tmin = 0.0f;
  for (int i = 0; i < n; ++i) {
    const Vec3 p = probe.element_position(i);
    const real w = window_value(apod_window, (p.x - origin.x) / std::max(half, 1e-9f));
    if (w <= 0.0f) continue;
    tx.apodization[static_cast<std::size_t>(i)] = w;
    real d = 0.0f;
    if (tx.type == TransmitType::PlaneWave)
      d = (p.x - origin.x) * std::sin(tx.angle) / c;
    else if (tx.type == TransmitType::Focused)
      d = (distance(tx.focus, origin) - distance(tx.focus, p)) / c;
    else
      d = (distance(p, tx.focus) - distance(origin, tx.focus)) / c;
    tx.delays[static_cast<std::size_t>(i)] = d;
  }
  for (int i = 0; i < n; ++i) {
    if (tx.apodization[static_cast<std::size_t>(i)] == 0.0f) continue;
    tmin = any ? std::min(tmin, tx.delays[static_cast<std::size_t>(i)]) : tx.delays[static_cast<std::size_t>(i)];
    any = true;
  }
  if (t0_offset) *t0_offset = any ? tmin : 0.0f;
}

real transmit_arrival_time(const Transmit& tx, const Vec3& point, real c) {
  const Vec3 origin(tx.origin.x, 0.0f, 0.0f);
  switch (tx.type) {
    case TransmitType::PlaneWave: {
      const real s = std::sin(tx.angle), k = std::cos(tx.angle);
      return ((point.x - origin.x) * s + (point.z - origin.z) * k) / c;
    }
    case TransmitType::Focused: {
      const Vec3 axis = tx.focus - origin;
      const real len = axis.norm();
      if (len < 1e-9f) return point.norm() / c;
      const Vec3 dir(axis.x / len, axis.y / len, axis.z / len);
      const Vec3 rel = point - tx.focus;
      const real proj = rel.x * dir.x + rel.y * dir.y + rel.z * dir.z;
      return (len + (proj >= 0.0f ? 1.0f : -1.0f) * rel.norm()) / c;
    }
    case TransmitType::Diverging:
      return (distance(point, tx.focus) - distance(origin, tx.focus)) / c;
  }
  return 0.0f;
}

real element_directivity(real element_width, real wavelength, real sin_theta) {
  const real st = std::clamp(sin_theta, -1.0f, 1.0f);
  const real ct = std::sqrt(std::max(0.0f, 1.0f - st * st));
  const real x = kPi * element_width * st / wavelength;
  const real s = std::abs(x) < 1e-6f ? 1.0f - x * x / 6.0f : std::sin(x) / x;
  return ct * s;
}

real dynamic_aperture_weight(const Vec3& element, const Vec3& point, real f_number, Window w,
                             real tukey_alpha) {
  const real depth = point.z - element.z;
  if (depth <= 0.0f) return 0.0f;
  const real half = 0.5f * depth / std::max(f_number, 1e-3f);
  return window_value(w, (element.x - point.x) / std::max(half, 1e-9f), tukey_alpha);
}

}  // namespace usx
