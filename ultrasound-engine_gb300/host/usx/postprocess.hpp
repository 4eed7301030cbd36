// usx/postprocess.hpp — envelope, TGC, log compression, scan conversion
// (drop-in for the reference's core/include/usx/postprocess.hpp:18-61); runs
// on the GPU.
#pragma once

#include <vector>

#include "usx/types.hpp"

namespace usx {

std::vector<real> envelope(const Frame& frame);
std::vector<real> apply_tgc(const std::vector<real>& env, const ScanGrid& grid,
                            real attenuation_db_cm_mhz, real center_frequency_hz);
std::vector<real> log_compress(const std::vector<real>& env, real dynamic_range_db = 60.0f,
                               real gain_db = 0.0f, real reference = -1.0f);

struct ScanConverted {
  int width = 0;
  int height = 0;
  real x_min = 0, x_max = 0, z_min = 0, z_max = 0;
  std::vector<real> pixels;
};

ScanConverted scan_convert(const std::vector<real>& image, const ScanGrid& grid, int width,
                           int height, real fill_value = 0.0f);

}  // namespace usx
