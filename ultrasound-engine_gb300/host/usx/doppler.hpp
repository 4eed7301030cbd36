// usx/doppler.hpp — wall filter, colour/power Doppler, speckle tracking and
// strain (drop-in for the reference's core/include/usx/doppler.hpp:19-144);
// runs on the GPU.
#pragma once

#include <cstdint>
#include <vector>

#include "usx/types.hpp"

namespace usx {

enum class WallFilter : std::uint8_t { None = 0, PolynomialRegression = 1, MeanSubtraction = 2 };

struct DopplerConfig {
  WallFilter wall_filter = WallFilter::PolynomialRegression;
  int polynomial_order = 1;
  bool loupas = true;
  int kernel_axial = 4;
  int kernel_lateral = 1;
  real power_threshold_db = -35.0f;
  real coherence_threshold = 0.35f;
};

struct ColorFlowMap {
  ScanGrid grid;
  std::vector<real> velocity;
  std::vector<real> power;
  std::vector<real> variance;
  std::vector<std::uint8_t> valid;
  real nyquist_velocity = 0.0f;
};

std::vector<Frame> apply_wall_filter(const std::vector<Frame>& ensemble, WallFilter type,
                                     int polynomial_order);
ColorFlowMap color_flow(const std::vector<Frame>& ensemble, real prf, real speed_of_sound,
                        DopplerConfig config = {});
std::vector<real> power_doppler(const std::vector<Frame>& ensemble,
                                WallFilter type = WallFilter::PolynomialRegression,
                                int polynomial_order = 1);

struct DisplacementMap {
  ScanGrid grid;
  std::vector<real> axial;
  std::vector<real> correlation;
};

DisplacementMap estimate_axial_displacement(const Frame& before, const Frame& after,
                                            real speed_of_sound, int kernel_axial = 8,
                                            int kernel_lateral = 2, int max_lag = 8);
std::vector<real> axial_strain(const DisplacementMap& disp, int fit_length = 15);

}  // namespace usx
