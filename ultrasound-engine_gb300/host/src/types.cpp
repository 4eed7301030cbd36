// types.cpp — validation, grid construction and apodization windows
// (behaviour of the reference's core/src/types.cpp:8-157).
#include "usx/types.hpp"

#include <algorithm>
#include <cmath>

namespace usx {

void Probe::validate() const {
  if (n_elements <= 0) throw std::invalid_argument("Probe.n_elements must be > 0");
  if (pitch <= 0) throw std::invalid_argument("Probe.pitch must be > 0");
  if (element_width <= 0) throw std::invalid_argument("Probe.element_width must be > 0");
  if (element_width > pitch * 1.001f)
    throw std::invalid_argument("Probe.element_width exceeds pitch (elements would overlap)");
  if (center_frequency <= 0) throw std::invalid_argument("Probe.center_frequency must be > 0");
  if (bandwidth <= 0) throw std::invalid_argument("Probe.bandwidth must be > 0");
}

void Medium::validate() const {
  if (speed_of_sound <= 0) throw std::invalid_argument("Medium.speed_of_sound must be > 0");
  if (attenuation < 0) throw std::invalid_argument("Medium.attenuation must be >= 0");
}

void Acquisition::validate() const {
  if (sampling_frequency <= 0) throw std::invalid_argument("Acquisition.sampling_frequency must be > 0");
  if (n_samples <= 0) throw std::invalid_argument("Acquisition.n_samples must be > 0");
  if (prf <= 0) throw std::invalid_argument("Acquisition.prf must be > 0");
}

int Transmit::n_active() const {
  return static_cast<int>(std::count_if(apodization.begin(), apodization.end(),
                                        [](real w) { return w != 0.0f; }));
}

void ChannelData::allocate() {
  validate();
  if (is_iq) {
    iq.assign(size(), cplx(0, 0));
    rf.clear();
  } else {
    rf.assign(size(), 0.0f);
    iq.clear();
  }
}

void ChannelData::validate() const {
  probe.validate();
  medium.validate();
  acq.validate();
  if (transmits.empty()) throw std::invalid_argument("ChannelData has no transmit events");
  for (const Transmit& tx : transmits) {
    if (!tx.delays.empty() && static_cast<int>(tx.delays.size()) != probe.n_elements)
      throw std::invalid_argument("Transmit.delays length != probe.n_elements");
    if (!tx.apodization.empty() && static_cast<int>(tx.apodization.size()) != probe.n_elements)
      throw std::invalid_argument("Transmit.apodization length != probe.n_elements");
  }
  const std::size_t have = is_iq ? iq.size() : rf.size();
  if (have != 0 && have != size())
    throw std::invalid_argument("ChannelData buffer size does not match n_events*n_channels*n_samples");
  if (is_iq && demodulation_frequency <= 0)
    throw std::invalid_argument("IQ ChannelData needs a positive demodulation_frequency");
}

namespace {
// Evenly spaced samples in [lo, hi] with the reference's float expression.
std::vector<real> linspace(real lo, real hi, int n) {
  std::vector<real> v(static_cast<std::size_t>(std::max(n, 0)));
  for (int i = 0; i < n; ++i) v[static_cast<std::size_t>(i)] = n == 1 ? lo : lo + (hi - lo) * i / (n - 1);
  return v;
}
}  // namespace

ScanGrid ScanGrid::cartesian(real x_min, real x_max, int nx, real z_min, real z_max, int nz) {
  ScanGrid g;
  g.type = GridType::Cartesian;
  g.n_axis0 = nx;
  g.n_axis1 = nz;
  g.axis0 = linspace(x_min, x_max, nx);
  g.axis1 = linspace(z_min, z_max, nz);
  g.build_points();
  g.validate();
  return g;
}

ScanGrid ScanGrid::sector(real theta_min, real theta_max, int n_theta, real r_min, real r_max,
                          int n_r, Vec3 apex) {
  ScanGrid g;
  g.type = GridType::Sector;
  g.n_axis0 = n_theta;
  g.n_axis1 = n_r;
  g.apex = apex;
  g.axis0 = linspace(theta_min, theta_max, n_theta);
  g.axis1 = linspace(r_min, r_max, n_r);
  g.build_points();
  g.validate();
  return g;
}

void ScanGrid::build_points() {
  points.resize(static_cast<std::size_t>(std::max(n_axis0, 0)) * std::max(n_axis1, 0));
  for (int i = 0; i < n_axis0; ++i)
    for (int j = 0; j < n_axis1; ++j) {
      Vec3& p = points[static_cast<std::size_t>(i) * n_axis1 + j];
      if (type == GridType::Cartesian) {
        p = Vec3(axis0[static_cast<std::size_t>(i)], 0.0f, axis1[static_cast<std::size_t>(j)]);
      } else {
        const real th = axis0[static_cast<std::size_t>(i)], r = axis1[static_cast<std::size_t>(j)];
        p = Vec3(apex.x + r * std::sin(th), 0.0f, apex.z + r * std::cos(th));
      }
    }
}

void ScanGrid::validate() const {
  if (n_axis0 <= 0 || n_axis1 <= 0) throw std::invalid_argument("ScanGrid dimensions must be > 0");
  if (static_cast<int>(axis0.size()) != n_axis0 || static_cast<int>(axis1.size()) != n_axis1)
    throw std::invalid_argument("ScanGrid axis length mismatch");
  if (points.size() != static_cast<std::size_t>(n_axis0) * n_axis1)
    throw std::invalid_argument("ScanGrid points not built (call build_points)");
}

real window_value(Window w, real u, real tukey_alpha) {
  if (u < -1.0f || u > 1.0f) return 0.0f;
  const real t = 0.5f * (u + 1.0f);
  const real two_pi = 2.0f * kPi;
  switch (w) {
    case Window::Rect: return 1.0f;
    case Window::Hann: return 0.5f * (1.0f - std::cos(two_pi * t));
    case Window::Hamming: return 0.54f - 0.46f * std::cos(two_pi * t);
    case Window::Blackman:
      return 0.42f - 0.5f * std::cos(two_pi * t) + 0.08f * std::cos(4.0f * kPi * t);
    case Window::Tukey: {
      const real a = std::clamp(tukey_alpha, 0.0f, 1.0f);
      if (a <= 0.0f) return 1.0f;
      if (t < a * 0.5f) return 0.5f * (1.0f + std::cos(two_pi / a * (t - a * 0.5f)));
      if (t > 1.0f - a * 0.5f) return 0.5f * (1.0f + std::cos(two_pi / a * (t - 1.0f + a * 0.5f)));
      return 1.0f;
    }
  }
  return 1.0f;
}

Window window_from_string(const std::string& name) {
  if (name == "rect" || name == "boxcar" || name == "none") return Window::Rect;
  if (name == "hann" || name == "hanning") return Window::Hann;
  if (name == "hamming") return Window::Hamming;
  if (name == "tukey") return Window::Tukey;
  if (name == "blackman") return Window::Blackman;
  throw std::invalid_argument("unknown window: " + name);
}

}  // namespace usx
