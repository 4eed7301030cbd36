// usx/demodulate.hpp — RF to baseband IQ (drop-in for the reference's
// core/include/usx/demodulate.hpp:21-51); runs on the GPU (usx_cu_demodulate).
#pragma once

#include <vector>

#include "usx/types.hpp"

namespace usx {

struct DemodConfig {
  real demodulation_frequency = 0.0f;
  real cutoff_fraction = 0.5f;
  int filter_taps = 33;
  int decimation = 1;
};

ChannelData demodulate(const ChannelData& rf, DemodConfig config = {});
std::vector<real> design_lowpass(int n_taps, real normalized_cutoff);

}  // namespace usx
