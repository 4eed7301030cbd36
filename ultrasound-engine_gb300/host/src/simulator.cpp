// simulator.cpp — phantom factories and the Simulator front end (behaviour of
// the reference's core/src/simulator.cpp:34-419). The seeded phantom factories
// run on the host with std::mt19937 and libstdc++'s distributions, drawing in
// the same sequence as the reference build, so a seed names the same phantom
// in both; simulate() runs on the GPU.
#include "usx/simulator.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "desc.hpp"
#include "usx/geometry.hpp"
#include "usx/runtime.hpp"

namespace usx {

Phantom Phantom::point_targets(const std::vector<Vec3>& positions, real amplitude) {
  Phantom p;
  p.scatterers.reserve(positions.size());
  for (const Vec3& v : positions) {
    Scatterer s;
    s.position = v;
    s.amplitude = amplitude;
    p.scatterers.push_back(s);
  }
  return p;
}

Phantom Phantom::speckle_box(real x_min, real x_max, real z_min, real z_max, real y_half_thickness,
                             int n_scatterers, std::uint32_t seed, real amplitude_sigma) {
  Phantom p;
  p.scatterers.reserve(static_cast<std::size_t>(std::max(0, n_scatterers)));
  std::mt19937 rng(seed);
  std::uniform_real_distribution<real> ux(x_min, x_max);
  std::uniform_real_distribution<real> uz(z_min, z_max);
  std::uniform_real_distribution<real> uy(-y_half_thickness, y_half_thickness);
  std::normal_distribution<real> amp(0.0f, amplitude_sigma);
  for (int i = 0; i < n_scatterers; ++i) {
    // The reference builds each position as Vec3(ux(), uy(), uz()); GCC
    // evaluates those arguments right to left, so z is drawn first. The order
    // is spelled out here so that every compiler and architecture agrees.
    const real z = uz(rng);
    const real y = uy(rng);
    const real x = ux(rng);
    Scatterer s;
    s.position = Vec3(x, y, z);
    s.amplitude = amp(rng);
    p.scatterers.push_back(s);
  }
  return p;
}

int Phantom::recommended_scatterer_count(const Probe& probe, const Medium& medium, real x_span,
                                         real z_span, real y_span, real f_number, real per_cell) {
  const real lambda = probe.wavelength(medium.speed_of_sound);
  const real dx = std::max(f_number * lambda, 1e-5f);
  const real dz = std::max(lambda / std::max(probe.bandwidth, 0.1f), 1e-5f);
  const real dy = std::max(probe.elevation_height, 1e-4f);
  const real cells = (x_span / dx) * (z_span / dz) * std::max(y_span / dy, 1.0f);
  const double n = static_cast<double>(cells) * per_cell;
  return static_cast<int>(std::min(n, 4.0e6));
}

void Phantom::scale_amplitude_in_circle(const Vec3& center, real radius, real scale) {
  const real r2 = radius * radius;
  for (Scatterer& s : scatterers) {
    const real dx = s.position.x - center.x;
    const real dz = s.position.z - center.z;
    if (dx * dx + dz * dz <= r2) s.amplitude *= scale;
  }
}

void Phantom::add_flow_tube(const Vec3& center, real radius, real length, real axis_angle,
                            real peak_velocity, int n_scatterers, std::uint32_t seed,
                            real amplitude) {
  std::mt19937 rng(seed);
  std::uniform_real_distribution<real> along(-0.5f * length, 0.5f * length);
  std::uniform_real_distribution<real> u01(0.0f, 1.0f);
  std::normal_distribution<real> amp(0.0f, amplitude);
  const real ax = std::cos(axis_angle), az = std::sin(axis_angle);
  const real nx = -std::sin(axis_angle), nz = std::cos(axis_angle);
  for (int i = 0; i < n_scatterers; ++i) {
    // Uniform over the vessel's circular cross-section (in-plane and
    // elevation offsets), uniform along its axis, Poiseuille speed profile.
    const real rr = radius * std::sqrt(u01(rng));
    const real phi = 2.0f * kPi * u01(rng);
    const real r_off = rr * std::cos(phi);
    const real y_off = rr * std::sin(phi);
    const real s_along = along(rng);
    Scatterer s;
    s.position = Vec3(center.x + ax * s_along + nx * r_off, y_off, center.z + az * s_along + nz * r_off);
    s.amplitude = amp(rng);
    const real v = peak_velocity * (1.0f - (rr / radius) * (rr / radius));
    s.velocity = Vec3(ax * v, 0.0f, az * v);
    scatterers.push_back(s);
  }
}

Simulator::Simulator(Probe probe, Medium medium, Acquisition acq, SimulatorConfig config)
    : probe_(probe), medium_(medium), acq_(acq), config_(config) {
  probe_.validate();
  medium_.validate();
  acq_.validate();
  if (config_.oversampling < 1) config_.oversampling = 1;
}

std::vector<real> Simulator::pulse(real* half_duration) const {
  const usx_probe p = desc::probe(probe_);
  const usx_acquisition a = desc::acq(acq_);
  const usx_simulator_config c = desc::sim(config_);
  int n = 0;
  rt::check(usx_cu_pulse(&p, &a, &c, nullptr, 0, &n, half_duration), "pulse");
  std::vector<real> out(static_cast<std::size_t>(n));
  rt::check(usx_cu_pulse(&p, &a, &c, out.data(), n, &n, half_duration), "pulse");
  return out;
}

std::vector<Transmit> Simulator::make_plane_waves(const std::vector<real>& angles) const {
  std::vector<Transmit> txs;
  for (real a : angles) {
    Transmit tx;
    tx.type = TransmitType::PlaneWave;
    tx.angle = a;
    compute_transmit_delays(probe_, medium_, tx, config_.tx_window, config_.tx_f_number, nullptr);
    txs.push_back(std::move(tx));
  }
  return txs;
}

std::vector<Transmit> Simulator::make_focused_scan(int n_lines, real x_min, real x_max,
                                                   real focal_depth, real angle) const {
  std::vector<Transmit> txs;
  for (int i = 0; i < n_lines; ++i) {
    const real x = (n_lines == 1) ? x_min : x_min + (x_max - x_min) * i / (n_lines - 1);
    Transmit tx;
    tx.type = TransmitType::Focused;
    tx.angle = angle;
    tx.origin = Vec3(x, 0, 0);
    tx.focus = Vec3(x + focal_depth * std::tan(angle), 0, focal_depth);
    compute_transmit_delays(probe_, medium_, tx, config_.tx_window, config_.tx_f_number, nullptr);
    txs.push_back(std::move(tx));
  }
  return txs;
}

std::vector<Transmit> Simulator::make_diverging_waves(const std::vector<real>& angles,
                                                      real virtual_source_depth) const {
  std::vector<Transmit> txs;
  for (real a : angles) {
    Transmit tx;
    tx.type = TransmitType::Diverging;
    tx.angle = a;
    tx.focus = Vec3(-virtual_source_depth * std::tan(a), 0, -virtual_source_depth);
    compute_transmit_delays(probe_, medium_, tx, config_.tx_window, config_.tx_f_number, nullptr);
    txs.push_back(std::move(tx));
  }
  return txs;
}

std::vector<Transmit> Simulator::repeat(const std::vector<Transmit>& txs, int n_ensemble) {
  std::vector<Transmit> out;
  for (int e = 0; e < n_ensemble; ++e) out.insert(out.end(), txs.begin(), txs.end());
  return out;
}

void Simulator::noise_normals(std::uint32_t seed, std::size_t n, float* out) {
  // std::normal_distribution<float>(0, sigma) returns z * sigma + 0 for a
  // draw z that does not depend on sigma; these are those z.
  std::mt19937 rng(seed);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  for (std::size_t k = 0; k < n; ++k) out[k] = nd(rng);
}

ChannelData Simulator::simulate(const std::vector<Transmit>& transmits, const Phantom& phantom) const {
  ChannelData cd;
  cd.probe = probe_;
  cd.medium = medium_;
  cd.acq = acq_;
  cd.transmits = transmits;
  cd.is_iq = false;
  cd.allocate();

  const std::size_t n_scat = phantom.scatterers.size();
  std::vector<usx_scatterer> sc(n_scat);
  for (std::size_t i = 0; i < n_scat; ++i) {
    const Scatterer& s = phantom.scatterers[i];
    sc[i] = usx_scatterer{s.position.x, s.position.y, s.position.z, s.amplitude,
                          s.velocity.x, s.velocity.y, s.velocity.z, 0.0f};
  }
  const std::size_t ev_size = static_cast<std::size_t>(cd.n_channels()) * cd.n_samples();
  const std::size_t total = ev_size * cd.n_events();
  usx_ctx* ctx = rt::ctx();
  void* d_scat = rt::slot(0, std::max<std::size_t>(1, n_scat) * sizeof(usx_scatterer));
  void* d_rf = rt::slot(1, total * sizeof(float));
  if (n_scat) rt::h2d(d_scat, sc.data(), n_scat * sizeof(usx_scatterer));
  const float* d_noise = nullptr;
  std::vector<float> z;
  if (config_.noise_db > -200.0f) {
    z.resize(total);
    for (int ev = 0; ev < cd.n_events(); ++ev)
      noise_normals(config_.noise_seed + static_cast<std::uint32_t>(ev), ev_size, z.data() + ev * ev_size);
    void* d_z = rt::slot(2, total * sizeof(float));
    rt::h2d(d_z, z.data(), total * sizeof(float));
    d_noise = static_cast<const float*>(d_z);
  }
  desc::Channel ch(cd);
  const usx_simulator_config scfg = desc::sim(config_);
  rt::check(usx_cu_simulate(ctx, &ch.cd, &scfg, static_cast<const usx_scatterer*>(d_scat),
                            static_cast<int64_t>(n_scat), d_noise, static_cast<float*>(d_rf), nullptr),
            "simulate");
  rt::d2h(cd.rf.data(), d_rf, total * sizeof(float));
  return cd;
}

}  // namespace usx
