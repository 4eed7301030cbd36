// demodulate.cpp — host front end of the GPU demodulator (behaviour of the
// reference's core/src/demodulate.cpp:13-121).
#include "usx/demodulate.hpp"

#include <algorithm>

#include "desc.hpp"
#include "usx/runtime.hpp"

namespace usx {

std::vector<real> design_lowpass(int n_taps, real normalized_cutoff) {
  int n = 0;
  rt::check(usx_cu_design_lowpass(n_taps, normalized_cutoff, nullptr, 0, &n), "design_lowpass");
  std::vector<real> h(static_cast<std::size_t>(n));
  rt::check(usx_cu_design_lowpass(n_taps, normalized_cutoff, h.data(), n, &n), "design_lowpass");
  return h;
}

ChannelData demodulate(const ChannelData& rf, DemodConfig config) {
  rf.validate();
  if (rf.is_iq) return rf;
  if (rf.rf.empty()) throw std::invalid_argument("demodulate: input has no RF samples");
  const int dec = std::max(1, config.decimation);
  ChannelData out;
  out.probe = rf.probe;
  out.medium = rf.medium;
  out.transmits = rf.transmits;
  out.acq = rf.acq;
  out.acq.sampling_frequency = rf.acq.sampling_frequency / dec;
  out.acq.n_samples = (rf.acq.n_samples + dec - 1) / dec;
  out.is_iq = true;
  out.demodulation_frequency = config.demodulation_frequency > 0.0f ? config.demodulation_frequency
                                                                     : rf.probe.center_frequency;
  out.allocate();

  desc::Channel ch(rf);
  const usx_demod_config dc = desc::demod(config);
  void* d_rf = rt::slot(0, rf.rf.size() * sizeof(float));
  void* d_iq = rt::slot(1, out.iq.size() * sizeof(cplx));
  rt::h2d(d_rf, rf.rf.data(), rf.rf.size() * sizeof(float));
  float fdem = 0.0f;
  rt::check(usx_cu_demodulate(rt::ctx(), &ch.cd, &dc, static_cast<const float*>(d_rf),
                              static_cast<float*>(d_iq), &fdem),
            "demodulate");
  rt::d2h(out.iq.data(), d_iq, out.iq.size() * sizeof(cplx));
  return out;
}

}  // namespace usx
