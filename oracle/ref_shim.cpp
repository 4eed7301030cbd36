// ref_shim.cpp — C entry points over the reference engine's own C++ API.
//
// TEST INFRASTRUCTURE ONLY. Compiled by oracle/build_ref.sh together with the
// reference's unmodified core/src/*.cpp (read in place, never copied) into
// oracle/_ref/libusx_ref.so, so that the CPU oracle and the golden fixtures can
// be checked against the reference itself. Every function converts the plain
// descriptors of include/usx_types.h into the reference's types, calls the
// reference function named in its comment, and copies the result out.
#include <cstring>
#include <vector>

#include "usx/beamformer.hpp"
#include "usx/demodulate.hpp"
#include "usx/doppler.hpp"
#include "usx/geometry.hpp"
#include "usx/postprocess.hpp"
#include "usx/simulator.hpp"

#include "../include/usx_types.h"

using namespace usx;

namespace {

Probe to_probe(const usx_probe& p) {
  Probe q;
  q.n_elements = p.n_elements;
  q.pitch = p.pitch;
  q.element_width = p.element_width;
  q.elevation_height = p.elevation_height;
  q.center_frequency = p.center_frequency;
  q.bandwidth = p.bandwidth;
  return q;
}

Transmit to_tx(const usx_transmit& t, int n) {
  Transmit x;
  x.type = static_cast<TransmitType>(t.type);
  x.angle = t.angle;
  x.focus = Vec3(t.focus[0], t.focus[1], t.focus[2]);
  x.origin = Vec3(t.origin[0], t.origin[1], t.origin[2]);
  if (t.delays) x.delays.assign(t.delays, t.delays + n);
  if (t.apodization) x.apodization.assign(t.apodization, t.apodization + n);
  return x;
}

ChannelData to_cd(const usx_channel_desc& d) {
  ChannelData cd;
  cd.probe = to_probe(d.probe);
  cd.medium.speed_of_sound = d.medium.speed_of_sound;
  cd.medium.attenuation = d.medium.attenuation;
  cd.medium.density = d.medium.density;
  cd.acq.sampling_frequency = d.acq.sampling_frequency;
  cd.acq.n_samples = d.acq.n_samples;
  cd.acq.t0 = d.acq.t0;
  cd.acq.prf = d.acq.prf;
  for (int e = 0; e < d.n_events; ++e) cd.transmits.push_back(to_tx(d.transmits[e], d.probe.n_elements));
  cd.is_iq = d.is_iq != 0;
  cd.demodulation_frequency = d.demodulation_frequency;
  return cd;
}

SimulatorConfig to_simcfg(const usx_simulator_config& c) {
  SimulatorConfig s;
  s.pulse_cycles = c.pulse_cycles;
  s.tx_window = static_cast<Window>(c.tx_window);
  s.tx_f_number = c.tx_f_number;
  s.oversampling = c.oversampling;
  s.full_transmit_diffraction = c.full_transmit_diffraction != 0;
  s.incident_trim_db = c.incident_trim_db;
  s.max_incident_window_us = c.max_incident_window_us;
  s.apply_attenuation = c.apply_attenuation != 0;
  s.apply_directivity = c.apply_directivity != 0;
  s.apply_spreading = c.apply_spreading != 0;
  s.noise_db = c.noise_db;
  s.noise_seed = c.noise_seed;
  s.enable_motion = c.enable_motion != 0;
  return s;
}

ScanGrid to_grid(int type, int n0, int n1, const float* axis0, const float* axis1,
                 const float* apex, const float* points) {
  ScanGrid g;
  g.type = static_cast<GridType>(type);
  g.n_axis0 = n0;
  g.n_axis1 = n1;
  g.axis0.assign(axis0, axis0 + n0);
  g.axis1.assign(axis1, axis1 + n1);
  if (apex) g.apex = Vec3(apex[0], apex[1], apex[2]);
  g.points.resize(static_cast<std::size_t>(n0) * n1);
  for (std::size_t k = 0; k < g.points.size(); ++k)
    g.points[k] = Vec3(points[3 * k], points[3 * k + 1], points[3 * k + 2]);
  return g;
}

Frame to_frame(const ScanGrid& g, const float* data, float fdem) {
  Frame f;
  f.grid = g;
  f.demodulation_frequency = fdem;
  f.data.resize(static_cast<std::size_t>(g.n_pixels()));
  std::memcpy(f.data.data(), data, f.data.size() * sizeof(cplx));
  return f;
}

void put_phantom(const Phantom& p, float* out) {
  for (std::size_t i = 0; i < p.scatterers.size(); ++i) {
    const Scatterer& s = p.scatterers[i];
    float* o = out + 8 * i;
    o[0] = s.position.x; o[1] = s.position.y; o[2] = s.position.z; o[3] = s.amplitude;
    o[4] = s.velocity.x; o[5] = s.velocity.y; o[6] = s.velocity.z; o[7] = 0.0f;
  }
}

Phantom get_phantom(const float* in, long n) {
  Phantom p;
  p.scatterers.resize(static_cast<std::size_t>(n));
  for (long i = 0; i < n; ++i) {
    const float* o = in + 8 * i;
    p.scatterers[static_cast<std::size_t>(i)].position = Vec3(o[0], o[1], o[2]);
    p.scatterers[static_cast<std::size_t>(i)].amplitude = o[3];
    p.scatterers[static_cast<std::size_t>(i)].velocity = Vec3(o[4], o[5], o[6]);
  }
  return p;
}

}  // namespace

extern "C" {

// Phantom::speckle_box (simulator.cpp:46-65); out holds n * 8 floats.
void ref_speckle_box(float x_min, float x_max, float z_min, float z_max, float y_half, int n,
                     unsigned seed, float sigma, float* out) {
  put_phantom(Phantom::speckle_box(x_min, x_max, z_min, z_max, y_half, n, seed, sigma), out);
}

// Phantom::scale_amplitude_in_circle (simulator.cpp:82-89), in place.
void ref_scale_in_circle(float* scat, long n, float cx, float cz, float radius, float scale) {
  Phantom p = get_phantom(scat, n);
  p.scale_amplitude_in_circle(Vec3(cx, 0, cz), radius, scale);
  put_phantom(p, scat);
}

// Phantom::add_flow_tube (simulator.cpp:91-126); out holds n * 8 floats.
void ref_flow_tube(float cx, float cz, float radius, float length, float axis_angle,
                   float peak_velocity, int n, unsigned seed, float amplitude, float* out) {
  Phantom p;
  p.add_flow_tube(Vec3(cx, 0, cz), radius, length, axis_angle, peak_velocity, n, seed, amplitude);
  put_phantom(p, out);
}

// compute_transmit_delays (geometry.cpp:17-80); delays/apod hold n_elements.
float ref_transmit_delays(const usx_probe* probe, const usx_medium* med, usx_transmit* tx,
                          int window, float f_number, float* delays, float* apod) {
  Medium m;
  m.speed_of_sound = med->speed_of_sound;
  Transmit t = to_tx(*tx, probe->n_elements);
  float t0 = 0;
  compute_transmit_delays(to_probe(*probe), m, t, static_cast<Window>(window), f_number, &t0);
  std::memcpy(delays, t.delays.data(), t.delays.size() * sizeof(float));
  std::memcpy(apod, t.apodization.data(), t.apodization.size() * sizeof(float));
  return t0;
}

// ScanGrid::cartesian / ScanGrid::sector (types.cpp:36-75); points n0*n1*3.
void ref_grid(int type, float a0_min, float a0_max, int n0, float a1_min, float a1_max, int n1,
              const float* apex, float* axis0, float* axis1, float* points) {
  ScanGrid g = type == 0 ? ScanGrid::cartesian(a0_min, a0_max, n0, a1_min, a1_max, n1)
                         : ScanGrid::sector(a0_min, a0_max, n0, a1_min, a1_max, n1,
                                            Vec3(apex[0], apex[1], apex[2]));
  std::memcpy(axis0, g.axis0.data(), sizeof(float) * n0);
  std::memcpy(axis1, g.axis1.data(), sizeof(float) * n1);
  for (std::size_t k = 0; k < g.points.size(); ++k) {
    points[3 * k] = g.points[k].x;
    points[3 * k + 1] = g.points[k].y;
    points[3 * k + 2] = g.points[k].z;
  }
}

// Simulator::pulse (simulator.cpp:140-154); returns the tap count.
int ref_pulse(const usx_channel_desc* cd, const usx_simulator_config* cfg, float* out,
              float* half) {
  ChannelData c = to_cd(*cd);
  Simulator sim(c.probe, c.medium, c.acq, to_simcfg(*cfg));
  std::vector<real> p = sim.pulse(half);
  if (out) std::memcpy(out, p.data(), p.size() * sizeof(float));
  return static_cast<int>(p.size());
}

// Simulator::simulate (simulator.cpp:213-419).
void ref_simulate(const usx_channel_desc* cd, const usx_simulator_config* cfg,
                  const float* scat, long n_scat, float* rf) {
  ChannelData c = to_cd(*cd);
  Simulator sim(c.probe, c.medium, c.acq, to_simcfg(*cfg));
  ChannelData out = sim.simulate(c.transmits, get_phantom(scat, n_scat));
  std::memcpy(rf, out.rf.data(), out.rf.size() * sizeof(float));
}

// The standard normals std::normal_distribution<float> draws from an engine
// seeded `seed` (the receive-noise stream of simulator.cpp:406-415 is these
// draws scaled by sigma).
void ref_normals(unsigned seed, long n, float* out) {
  std::mt19937 rng(seed);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  for (long k = 0; k < n; ++k) out[k] = nd(rng);
}

// demodulate (demodulate.cpp:36-121).
void ref_demodulate(const usx_channel_desc* cd, const usx_demod_config* cfg, const float* rf,
                    float* iq) {
  ChannelData c = to_cd(*cd);
  c.is_iq = false;
  c.rf.assign(rf, rf + c.size());
  DemodConfig d;
  d.demodulation_frequency = cfg->demodulation_frequency;
  d.cutoff_fraction = cfg->cutoff_fraction;
  d.filter_taps = cfg->filter_taps;
  d.decimation = cfg->decimation;
  ChannelData out = demodulate(c, d);
  std::memcpy(iq, out.iq.data(), out.iq.size() * sizeof(cplx));
}

// design_lowpass (demodulate.cpp:13-34); returns the tap count.
int ref_design_lowpass(int n, float fc, float* h) {
  std::vector<real> v = design_lowpass(n, fc);
  if (h) std::memcpy(h, v.data(), v.size() * sizeof(float));
  return static_cast<int>(v.size());
}

// Beamformer::beamform (beamformer.cpp:297-549).
void ref_beamform(const usx_channel_desc* cd, const float* data, int grid_type, int n0, int n1,
                  const float* axis0, const float* axis1, const float* apex, const float* points,
                  const usx_beamformer_config* cfg, int ev_begin, int ev_end, float* frame) {
  ChannelData c = to_cd(*cd);
  if (c.is_iq) {
    c.iq.resize(c.size());
    std::memcpy(c.iq.data(), data, c.size() * sizeof(cplx));
  } else {
    c.rf.assign(data, data + c.size());
  }
  BeamformerConfig b;
  b.f_number = cfg->f_number;
  b.rx_window = static_cast<Window>(cfg->rx_window);
  b.tukey_alpha = cfg->tukey_alpha;
  b.combiner = static_cast<Combiner>(cfg->combiner);
  b.compounding = static_cast<Compounding>(cfg->compounding);
  b.transmit_weighting = cfg->transmit_weighting != 0;
  b.coherence_factor = cfg->coherence_factor != 0;
  b.mv_subarray = cfg->mv_subarray;
  b.mv_diagonal_loading = cfg->mv_diagonal_loading;
  b.mv_range_average = cfg->mv_range_average;
  Beamformer bf(b);
  Frame f = bf.beamform(c, to_grid(grid_type, n0, n1, axis0, axis1, apex, points), ev_begin, ev_end);
  std::memcpy(frame, f.data.data(), f.data.size() * sizeof(cplx));
}

// transmit_sensitivity (beamformer.cpp:292-295) and transmit_arrival_time
// (geometry.cpp:82-109) at one point.
float ref_transmit_sensitivity(const usx_probe* probe, const usx_transmit* tx, const float* p,
                               float wavelength) {
  return transmit_sensitivity(to_probe(*probe), to_tx(*tx, probe->n_elements),
                              Vec3(p[0], p[1], p[2]), wavelength);
}
float ref_transmit_arrival_time(const usx_transmit* tx, int n_el, const float* p, float c) {
  return transmit_arrival_time(to_tx(*tx, n_el), Vec3(p[0], p[1], p[2]), c);
}
float ref_window_value(int w, float u, float alpha) {
  return window_value(static_cast<Window>(w), u, alpha);
}
float ref_element_directivity(float w, float lambda, float st) {
  return element_directivity(w, lambda, st);
}

namespace {
std::vector<Frame> to_ensemble(const float* ens, int n_frames, const ScanGrid& g, float fdem) {
  std::vector<Frame> v;
  const std::size_t n_pix = static_cast<std::size_t>(g.n_pixels());
  for (int e = 0; e < n_frames; ++e) v.push_back(to_frame(g, ens + 2 * n_pix * e, fdem));
  return v;
}
ScanGrid simple_grid(int n0, int n1, const float* axis1) {
  ScanGrid g;
  g.n_axis0 = n0;
  g.n_axis1 = n1;
  g.axis0.assign(static_cast<std::size_t>(n0), 0.0f);
  g.axis1.assign(axis1, axis1 + n1);
  g.points.resize(static_cast<std::size_t>(n0) * n1);
  return g;
}
}  // namespace

// apply_wall_filter (doppler.cpp:51-75).
void ref_wall_filter(const float* ens, int n_frames, int n0, int n1, const float* axis1, int type,
                     int order, float* out) {
  ScanGrid g = simple_grid(n0, n1, axis1);
  std::vector<Frame> f = apply_wall_filter(to_ensemble(ens, n_frames, g, 5e6f),
                                           static_cast<WallFilter>(type), order);
  const std::size_t n_pix = static_cast<std::size_t>(g.n_pixels());
  for (int e = 0; e < n_frames; ++e)
    std::memcpy(out + 2 * n_pix * e, f[static_cast<std::size_t>(e)].data.data(), n_pix * sizeof(cplx));
}

// color_flow (doppler.cpp:77-176).
float ref_color_flow(const float* ens, int n_frames, int n0, int n1, const float* axis1, float fdem,
                     float prf, float c, const usx_doppler_config* cfg, float* vel, float* pw,
                     float* var, unsigned char* valid) {
  ScanGrid g = simple_grid(n0, n1, axis1);
  DopplerConfig d;
  d.wall_filter = static_cast<WallFilter>(cfg->wall_filter);
  d.polynomial_order = cfg->polynomial_order;
  d.loupas = cfg->loupas != 0;
  d.kernel_axial = cfg->kernel_axial;
  d.kernel_lateral = cfg->kernel_lateral;
  d.power_threshold_db = cfg->power_threshold_db;
  d.coherence_threshold = cfg->coherence_threshold;
  ColorFlowMap m = color_flow(to_ensemble(ens, n_frames, g, fdem), prf, c, d);
  const std::size_t n = m.velocity.size();
  std::memcpy(vel, m.velocity.data(), n * sizeof(float));
  std::memcpy(pw, m.power.data(), n * sizeof(float));
  std::memcpy(var, m.variance.data(), n * sizeof(float));
  std::memcpy(valid, m.valid.data(), n);
  return m.nyquist_velocity;
}

// power_doppler (doppler.cpp:178-186).
void ref_power_doppler(const float* ens, int n_frames, int n0, int n1, const float* axis1, int type,
                       int order, float* out) {
  ScanGrid g = simple_grid(n0, n1, axis1);
  std::vector<real> p = power_doppler(to_ensemble(ens, n_frames, g, 5e6f),
                                      static_cast<WallFilter>(type), order);
  std::memcpy(out, p.data(), p.size() * sizeof(float));
}

// estimate_axial_displacement (doppler.cpp:188-273) and axial_strain (:275-305).
void ref_displacement(const float* a, const float* b, int n0, int n1, const float* axis1, float fdem,
                      float c, int ka, int kl, int max_lag, float* axial, float* corr) {
  ScanGrid g = simple_grid(n0, n1, axis1);
  DisplacementMap d = estimate_axial_displacement(to_frame(g, a, fdem), to_frame(g, b, fdem), c, ka,
                                                  kl, max_lag);
  std::memcpy(axial, d.axial.data(), d.axial.size() * sizeof(float));
  std::memcpy(corr, d.correlation.data(), d.correlation.size() * sizeof(float));
}
void ref_strain(const float* axial, int n0, int n1, const float* axis1, int fit, float* out) {
  DisplacementMap d;
  d.grid = simple_grid(n0, n1, axis1);
  d.axial.assign(axial, axial + static_cast<std::size_t>(n0) * n1);
  d.correlation.assign(static_cast<std::size_t>(n0) * n1, 0.0f);
  std::vector<real> s = axial_strain(d, fit);
  std::memcpy(out, s.data(), s.size() * sizeof(float));
}

// envelope (postprocess.cpp:67-82), apply_tgc (:84-98), log_compress (:100-117),
// scan_convert (:119-178).
void ref_envelope(const float* frame, int grid_type, int n0, int n1, const float* axis0,
                  const float* axis1, const float* apex, const float* points, float fdem,
                  float* env) {
  Frame f = to_frame(to_grid(grid_type, n0, n1, axis0, axis1, apex, points), frame, fdem);
  std::vector<real> e = envelope(f);
  std::memcpy(env, e.data(), e.size() * sizeof(float));
}
void ref_apply_tgc(const float* env, int grid_type, int n0, int n1, const float* axis0,
                   const float* axis1, const float* apex, const float* points, float atten,
                   float f0, float* out) {
  ScanGrid g = to_grid(grid_type, n0, n1, axis0, axis1, apex, points);
  std::vector<real> v(env, env + static_cast<std::size_t>(n0) * n1);
  std::vector<real> o = apply_tgc(v, g, atten, f0);
  std::memcpy(out, o.data(), o.size() * sizeof(float));
}
void ref_log_compress(const float* env, long n, float dr, float gain, float ref, float* out) {
  std::vector<real> v(env, env + n);
  std::vector<real> o = log_compress(v, dr, gain, ref);
  std::memcpy(out, o.data(), o.size() * sizeof(float));
}
void ref_scan_convert(const float* img, int grid_type, int n0, int n1, const float* axis0,
                      const float* axis1, const float* apex, const float* points, int width,
                      int height, float fill, float* pixels, float* extent) {
  ScanGrid g = to_grid(grid_type, n0, n1, axis0, axis1, apex, points);
  std::vector<real> v(img, img + static_cast<std::size_t>(n0) * n1);
  ScanConverted sc = scan_convert(v, g, width, height, fill);
  std::memcpy(pixels, sc.pixels.data(), sc.pixels.size() * sizeof(float));
  extent[0] = sc.x_min; extent[1] = sc.x_max; extent[2] = sc.z_min; extent[3] = sc.z_max;
}

}  // extern "C"
