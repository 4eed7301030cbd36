// usx/simulator.hpp — point-scatterer forward model (drop-in for the
// reference's core/include/usx/simulator.hpp:23-156). Phantom factories run
// on the host with the reference's seeded generators; Simulator::simulate
// runs on the GPU (usx_cu_simulate).
#pragma once

#include <cstdint>
#include <random>
#include <vector>

#include "usx/types.hpp"

namespace usx {

struct Scatterer {
  Vec3 position;
  real amplitude = 1.0f;
  Vec3 velocity{0, 0, 0};
};

struct Phantom {
  std::vector<Scatterer> scatterers;

  void add(const Scatterer& s) { scatterers.push_back(s); }
  std::size_t size() const { return scatterers.size(); }

  static Phantom point_targets(const std::vector<Vec3>& positions, real amplitude = 1.0f);
  static Phantom speckle_box(real x_min, real x_max, real z_min, real z_max, real y_half_thickness,
                             int n_scatterers, std::uint32_t seed = 1234,
                             real amplitude_sigma = 1.0f);
  static int recommended_scatterer_count(const Probe& probe, const Medium& medium, real x_span,
                                         real z_span, real y_span, real f_number = 2.0f,
                                         real per_cell = 10.0f);
  void scale_amplitude_in_circle(const Vec3& center, real radius, real scale);
  void add_flow_tube(const Vec3& center, real radius, real length, real axis_angle,
                     real peak_velocity, int n_scatterers, std::uint32_t seed = 99,
                     real amplitude = 0.05f);
};

struct SimulatorConfig {
  real pulse_cycles = 2.5f;
  Window tx_window = Window::Hann;
  real tx_f_number = 2.0f;
  int oversampling = 4;
  bool full_transmit_diffraction = true;
  real incident_trim_db = -40.0f;
  real max_incident_window_us = 30.0f;
  bool apply_attenuation = true;
  bool apply_directivity = true;
  bool apply_spreading = true;
  real noise_db = -60.0f;
  std::uint32_t noise_seed = 7;
  bool enable_motion = true;
};

class Simulator {
 public:
  Simulator(Probe probe, Medium medium, Acquisition acq, SimulatorConfig config = {});

  std::vector<Transmit> make_plane_waves(const std::vector<real>& angles) const;
  std::vector<Transmit> make_focused_scan(int n_lines, real x_min, real x_max, real focal_depth,
                                          real angle = 0.0f) const;
  std::vector<Transmit> make_diverging_waves(const std::vector<real>& angles,
                                             real virtual_source_depth) const;
  static std::vector<Transmit> repeat(const std::vector<Transmit>& txs, int n_ensemble);

  ChannelData simulate(const std::vector<Transmit>& transmits, const Phantom& phantom) const;

  const Probe& probe() const { return probe_; }
  const Medium& medium() const { return medium_; }
  const Acquisition& acquisition() const { return acq_; }
  const SimulatorConfig& config() const { return config_; }
  Acquisition& acquisition() { return acq_; }

  std::vector<real> pulse(real* half_duration = nullptr) const;

  // The standard normals the receive noise of event `ev` is built from
  // (std::normal_distribution<float> seeded noise_seed + ev), n per event.
  static void noise_normals(std::uint32_t seed, std::size_t n, float* out);

 private:
  Probe probe_;
  Medium medium_;
  Acquisition acq_;
  SimulatorConfig config_;
};

}  // namespace usx
