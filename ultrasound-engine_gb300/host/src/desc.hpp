// desc.hpp — conversions from the usx:: value types to the POD descriptors of
// the C-ABI (include/usx_types.h). Private to the host library.
#pragma once

#include <vector>

#include "usx/beamformer.hpp"
#include "usx/demodulate.hpp"
#include "usx/doppler.hpp"
#include "usx/simulator.hpp"
#include "usx/types.hpp"
#include "usx_cu.h"

namespace usx {
namespace desc {

inline usx_probe probe(const Probe& p) {
  return usx_probe{p.n_elements, p.pitch, p.element_width, p.elevation_height,
                   p.center_frequency, p.bandwidth};
}
inline usx_medium medium(const Medium& m) { return usx_medium{m.speed_of_sound, m.attenuation, m.density}; }
inline usx_acquisition acq(const Acquisition& a) {
  return usx_acquisition{a.sampling_frequency, a.n_samples, a.t0, a.prf};
}

// Channel metadata plus the transmit array it points into (kept alive here).
struct Channel {
  usx_channel_desc cd{};
  std::vector<usx_transmit> txs;
  Channel(const Probe& p, const Medium& m, const Acquisition& a, const std::vector<Transmit>& t,
          bool is_iq, real fdem) {
    txs.resize(t.size());
    for (std::size_t e = 0; e < t.size(); ++e) {
      usx_transmit& x = txs[e];
      x.type = static_cast<int32_t>(t[e].type);
      x.angle = t[e].angle;
      x.focus[0] = t[e].focus.x; x.focus[1] = t[e].focus.y; x.focus[2] = t[e].focus.z;
      x.origin[0] = t[e].origin.x; x.origin[1] = t[e].origin.y; x.origin[2] = t[e].origin.z;
      x.delays = t[e].delays.empty() ? nullptr : t[e].delays.data();
      x.apodization = t[e].apodization.empty() ? nullptr : t[e].apodization.data();
    }
    cd.probe = probe(p);
    cd.medium = medium(m);
    cd.acq = acq(a);
    cd.n_events = static_cast<int32_t>(t.size());
    cd.transmits = txs.empty() ? nullptr : txs.data();
    cd.is_iq = is_iq ? 1 : 0;
    cd.demodulation_frequency = fdem;
  }
  explicit Channel(const ChannelData& d)
      : Channel(d.probe, d.medium, d.acq, d.transmits, d.is_iq, d.demodulation_frequency) {}
  Channel(const Channel&) = delete;
  Channel& operator=(const Channel&) = delete;
};

inline usx_beamformer_config bf(const BeamformerConfig& c) {
  usx_beamformer_config b;
  b.f_number = c.f_number;
  b.rx_window = static_cast<int32_t>(c.rx_window);
  b.tukey_alpha = c.tukey_alpha;
  b.combiner = static_cast<int32_t>(c.combiner);
  b.compounding = static_cast<int32_t>(c.compounding);
  b.transmit_weighting = c.transmit_weighting ? 1 : 0;
  b.coherence_factor = c.coherence_factor ? 1 : 0;
  b.mv_subarray = c.mv_subarray;
  b.mv_diagonal_loading = c.mv_diagonal_loading;
  b.mv_range_average = c.mv_range_average;
  return b;
}

inline usx_demod_config demod(const DemodConfig& c) {
  return usx_demod_config{c.demodulation_frequency, c.cutoff_fraction, c.filter_taps, c.decimation};
}

inline usx_simulator_config sim(const SimulatorConfig& c) {
  usx_simulator_config s;
  s.pulse_cycles = c.pulse_cycles;
  s.tx_window = static_cast<int32_t>(c.tx_window);
  s.tx_f_number = c.tx_f_number;
  s.oversampling = c.oversampling;
  s.full_transmit_diffraction = c.full_transmit_diffraction ? 1 : 0;
  s.incident_trim_db = c.incident_trim_db;
  s.max_incident_window_us = c.max_incident_window_us;
  s.apply_attenuation = c.apply_attenuation ? 1 : 0;
  s.apply_directivity = c.apply_directivity ? 1 : 0;
  s.apply_spreading = c.apply_spreading ? 1 : 0;
  s.noise_db = c.noise_db;
  s.noise_seed = c.noise_seed;
  s.enable_motion = c.enable_motion ? 1 : 0;
  return s;
}

inline usx_doppler_config doppler(const DopplerConfig& c) {
  usx_doppler_config d;
  d.wall_filter = static_cast<int32_t>(c.wall_filter);
  d.polynomial_order = c.polynomial_order;
  d.loupas = c.loupas ? 1 : 0;
  d.kernel_axial = c.kernel_axial;
  d.kernel_lateral = c.kernel_lateral;
  d.power_threshold_db = c.power_threshold_db;
  d.coherence_threshold = c.coherence_threshold;
  return d;
}

inline usx_grid_desc grid(const ScanGrid& g) {
  usx_grid_desc d;
  d.type = static_cast<int32_t>(g.type);
  d.n_axis0 = g.n_axis0;
  d.n_axis1 = g.n_axis1;
  d.apex[0] = g.apex.x; d.apex[1] = g.apex.y; d.apex[2] = g.apex.z;
  d.axis0 = g.axis0.data();
  d.axis1 = g.axis1.data();
  return d;
}

// Grid points as a flat [n][3] float array (Vec3 is three packed floats).
inline const float* points(const ScanGrid& g) { return reinterpret_cast<const float*>(g.points.data()); }

static_assert(sizeof(Vec3) == 3 * sizeof(float), "Vec3 must be three packed floats");
static_assert(sizeof(cplx) == 2 * sizeof(float), "complex<float> must be two packed floats");

}  // namespace desc
}  // namespace usx
