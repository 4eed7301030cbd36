// doppler.cpp — host front ends of the GPU Doppler and elastography kernels
// (behaviour of the reference's core/src/doppler.cpp:51-305).
#include "usx/doppler.hpp"

#include <algorithm>

#include "desc.hpp"
#include "usx/runtime.hpp"

namespace usx {

namespace {
// Stage an ensemble [frame][pixel] on the device; frames must share a size.
void* upload_ensemble(const std::vector<Frame>& ens, std::size_t* n_pix, const char* who) {
  *n_pix = ens.front().data.size();
  for (const Frame& f : ens)
    if (f.data.size() != *n_pix) throw std::invalid_argument(std::string(who) + ": frames have different sizes");
  void* d = rt::slot(8, *n_pix * ens.size() * sizeof(cplx));
  for (std::size_t e = 0; e < ens.size(); ++e)
    rt::h2d(static_cast<char*>(d) + e * *n_pix * sizeof(cplx), ens[e].data.data(), *n_pix * sizeof(cplx));
  return d;
}
}  // namespace

std::vector<Frame> apply_wall_filter(const std::vector<Frame>& ensemble, WallFilter type,
                                     int polynomial_order) {
  if (ensemble.empty()) return {};
  if (type == WallFilter::None) return ensemble;
  std::size_t n_pix = 0;
  void* d_in = upload_ensemble(ensemble, &n_pix, "apply_wall_filter");
  void* d_out = rt::slot(9, n_pix * ensemble.size() * sizeof(cplx));
  rt::check(usx_cu_wall_filter(rt::ctx(), static_cast<const float*>(d_in), static_cast<int>(ensemble.size()),
                               static_cast<int64_t>(n_pix), static_cast<int>(type), polynomial_order,
                               static_cast<float*>(d_out)),
            "apply_wall_filter");
  std::vector<Frame> out = ensemble;
  for (std::size_t e = 0; e < out.size(); ++e)
    rt::d2h(out[e].data.data(), static_cast<char*>(d_out) + e * n_pix * sizeof(cplx), n_pix * sizeof(cplx));
  return out;
}

ColorFlowMap color_flow(const std::vector<Frame>& ensemble, real prf, real speed_of_sound,
                        DopplerConfig config) {
  if (ensemble.size() < 2) throw std::invalid_argument("color_flow: need at least 2 frames in the ensemble");
  const ScanGrid& grid = ensemble.front().grid;
  std::size_t n_pix = 0;
  void* d_in = upload_ensemble(ensemble, &n_pix, "color_flow");
  if (n_pix != static_cast<std::size_t>(grid.n_pixels()))
    throw std::invalid_argument("color_flow: frame data does not match its grid");
  ColorFlowMap out;
  out.grid = grid;
  out.velocity.assign(n_pix, 0.0f);
  out.power.assign(n_pix, 0.0f);
  out.variance.assign(n_pix, 0.0f);
  out.valid.assign(n_pix, 0);
  char* d_out = static_cast<char*>(rt::slot(9, n_pix * (3 * sizeof(float) + 1) + 64));
  float* d_vel = reinterpret_cast<float*>(d_out);
  float* d_pow = d_vel + n_pix;
  float* d_var = d_pow + n_pix;
  uint8_t* d_valid = reinterpret_cast<uint8_t*>(d_var + n_pix);
  const usx_doppler_config dc = desc::doppler(config);
  float nyq = 0.0f;
  rt::check(usx_cu_color_flow(rt::ctx(), static_cast<const float*>(d_in), static_cast<int>(ensemble.size()),
                              grid.n_axis0, grid.n_axis1, grid.axis1.data(),
                              ensemble.front().demodulation_frequency, prf, speed_of_sound, &dc, d_vel,
                              d_pow, d_var, d_valid, &nyq),
            "color_flow");
  rt::d2h(out.velocity.data(), d_vel, n_pix * sizeof(float));
  rt::d2h(out.power.data(), d_pow, n_pix * sizeof(float));
  rt::d2h(out.variance.data(), d_var, n_pix * sizeof(float));
  rt::d2h(out.valid.data(), d_valid, n_pix);
  out.nyquist_velocity = nyq;
  return out;
}

std::vector<real> power_doppler(const std::vector<Frame>& ensemble, WallFilter type, int polynomial_order) {
  if (ensemble.empty()) return {};
  std::size_t n_pix = 0;
  void* d_in = upload_ensemble(ensemble, &n_pix, "power_doppler");
  void* d_out = rt::slot(9, n_pix * sizeof(float));
  rt::check(usx_cu_power_doppler(rt::ctx(), static_cast<const float*>(d_in), static_cast<int>(ensemble.size()),
                                 static_cast<int64_t>(n_pix), static_cast<int>(type), polynomial_order,
                                 static_cast<float*>(d_out)),
            "power_doppler");
  std::vector<real> p(n_pix);
  rt::d2h(p.data(), d_out, n_pix * sizeof(float));
  return p;
}

DisplacementMap estimate_axial_displacement(const Frame& before, const Frame& after, real speed_of_sound,
                                            int kernel_axial, int kernel_lateral, int max_lag) {
  if (before.data.size() != after.data.size())
    throw std::invalid_argument("estimate_axial_displacement: frame size mismatch");
  const ScanGrid& grid = before.grid;
  const std::size_t n = before.data.size();
  DisplacementMap out;
  out.grid = grid;
  out.axial.assign(n, 0.0f);
  out.correlation.assign(n, 0.0f);
  if (n == 0) return out;
  if (n != static_cast<std::size_t>(grid.n_pixels()))
    throw std::invalid_argument("estimate_axial_displacement: frame data does not match its grid");
  char* d_in = static_cast<char*>(rt::slot(8, 2 * n * sizeof(cplx)));
  rt::h2d(d_in, before.data.data(), n * sizeof(cplx));
  rt::h2d(d_in + n * sizeof(cplx), after.data.data(), n * sizeof(cplx));
  float* d_out = static_cast<float*>(rt::slot(9, 2 * n * sizeof(float)));
  rt::check(usx_cu_axial_displacement(rt::ctx(), reinterpret_cast<const float*>(d_in),
                                      reinterpret_cast<const float*>(d_in + n * sizeof(cplx)), grid.n_axis0,
                                      grid.n_axis1, grid.axis1.data(), before.demodulation_frequency,
                                      speed_of_sound, kernel_axial, kernel_lateral, max_lag, d_out, d_out + n),
            "estimate_axial_displacement");
  rt::d2h(out.axial.data(), d_out, n * sizeof(float));
  rt::d2h(out.correlation.data(), d_out + n, n * sizeof(float));
  return out;
}

std::vector<real> axial_strain(const DisplacementMap& disp, int fit_length) {
  const int n0 = disp.grid.n_axis0, n1 = disp.grid.n_axis1;
  const std::size_t n = static_cast<std::size_t>(n0) * n1;
  std::vector<real> strain(n, 0.0f);
  if (n == 0) return strain;
  if (disp.axial.size() != n) throw std::invalid_argument("axial_strain: displacement does not match its grid");
  float* d = static_cast<float*>(rt::slot(8, 2 * n * sizeof(float)));
  rt::h2d(d, disp.axial.data(), n * sizeof(float));
  rt::check(usx_cu_axial_strain(rt::ctx(), d, n0, n1, disp.grid.axis1.data(), fit_length, d + n), "axial_strain");
  rt::d2h(strain.data(), d + n, n * sizeof(float));
  return strain;
}

}  // namespace usx
