// usx/geometry.hpp — transmit delay laws and arrival times (drop-in for the
// reference's core/include/usx/geometry.hpp:14-58). Scalar host utilities;
// the per-pixel versions used by the beamformer live in the CUDA kernels.
#pragma once

#include "usx/types.hpp"

namespace usx {

void compute_transmit_delays(const Probe& probe, const Medium& medium, Transmit& tx,
                             Window apod_window, real f_number, real* t0_offset);
real transmit_arrival_time(const Transmit& tx, const Vec3& point, real c);
inline real receive_arrival_time(const Vec3& element, const Vec3& point, real c) {
  return distance(element, point) / c;
}
real element_directivity(real element_width, real wavelength, real sin_theta);
real dynamic_aperture_weight(const Vec3& element, const Vec3& point, real f_number, Window w,
                             real tukey_alpha = 0.5f);

}  // namespace usx
