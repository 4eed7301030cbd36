// usx/types.hpp — the engine's value types (drop-in for the reference's
// core/include/usx/types.hpp:30-296): same names, fields, defaults, units (SI)
// and memory layouts, so code written against the reference compiles against
// this header unchanged.
//
// The difference is where work happens: the methods here are bookkeeping on
// the host; every per-sample or per-pixel computation is a CUDA kernel behind
// the C-ABI in include/usx_cu.h.
#pragma once

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace usx {

using real = float;
using cplx = std::complex<real>;

constexpr real kPi = static_cast<real>(3.14159265358979323846);

struct Vec3 {
  real x = 0, y = 0, z = 0;
  Vec3() = default;
  Vec3(real x_, real y_, real z_) : x(x_), y(y_), z(z_) {}
  Vec3 operator-(const Vec3& o) const { return {x - o.x, y - o.y, z - o.z}; }
  Vec3 operator+(const Vec3& o) const { return {x + o.x, y + o.y, z + o.z}; }
  Vec3 operator*(real s) const { return {x * s, y * s, z * s}; }
  real norm() const { return std::sqrt(x * x + y * y + z * z); }
  real norm_sq() const { return x * x + y * y + z * z; }
};

inline real distance(const Vec3& a, const Vec3& b) { return (a - b).norm(); }

// Linear/phased array of elements along x, centred on x = 0.
struct Probe {
  int n_elements = 128;
  real pitch = 300e-6f;
  real element_width = 270e-6f;
  real elevation_height = 5e-3f;
  real center_frequency = 5.0e6f;
  real bandwidth = 0.6f;

  Vec3 element_position(int i) const {
    return {(static_cast<real>(i) - 0.5f * static_cast<real>(n_elements - 1)) * pitch, 0.0f, 0.0f};
  }
  real aperture_width() const { return static_cast<real>(n_elements - 1) * pitch + element_width; }
  real wavelength(real speed_of_sound) const { return speed_of_sound / center_frequency; }
  void validate() const;
};

struct Medium {
  real speed_of_sound = 1540.0f;
  real attenuation = 0.5f;   // dB / (cm MHz), one way
  real density = 1000.0f;
  void validate() const;
};

struct Acquisition {
  real sampling_frequency = 40.0e6f;
  int n_samples = 2048;
  real t0 = 0.0f;
  real prf = 5000.0f;

  real sample_time(int n) const { return t0 + static_cast<real>(n) / sampling_frequency; }
  real time_to_sample(real t) const { return (t - t0) * sampling_frequency; }
  real max_depth(real c) const { return 0.5f * c / prf; }
  void validate() const;
};

enum class TransmitType : std::uint8_t { Focused = 0, PlaneWave = 1, Diverging = 2 };

struct Transmit {
  TransmitType type = TransmitType::PlaneWave;
  real angle = 0.0f;
  Vec3 focus{0, 0, 0.03f};
  Vec3 origin{0, 0, 0};
  std::vector<real> delays;
  std::vector<real> apodization;
  int n_active() const;
};

// Raw channel data [event][channel][sample], RF or complex IQ.
struct ChannelData {
  Probe probe;
  Medium medium;
  Acquisition acq;
  std::vector<Transmit> transmits;

  bool is_iq = false;
  std::vector<real> rf;
  std::vector<cplx> iq;
  real demodulation_frequency = 0.0f;

  int n_events() const { return static_cast<int>(transmits.size()); }
  int n_channels() const { return probe.n_elements; }
  int n_samples() const { return acq.n_samples; }
  std::size_t index(int event, int channel, int sample) const {
    return (static_cast<std::size_t>(event) * n_channels() + channel) *
               static_cast<std::size_t>(n_samples()) + sample;
  }
  std::size_t size() const {
    return static_cast<std::size_t>(n_events()) * n_channels() * n_samples();
  }
  void allocate();
  void validate() const;
};

enum class GridType : std::uint8_t { Cartesian = 0, Sector = 1 };

// Pixel positions, stored explicitly [axis0][axis1] with axis1 fastest.
struct ScanGrid {
  GridType type = GridType::Cartesian;
  int n_axis0 = 0;
  int n_axis1 = 0;
  std::vector<real> axis0;
  std::vector<real> axis1;
  Vec3 apex{0, 0, 0};
  std::vector<Vec3> points;

  int n_pixels() const { return n_axis0 * n_axis1; }
  static ScanGrid cartesian(real x_min, real x_max, int nx, real z_min, real z_max, int nz);
  static ScanGrid sector(real theta_min, real theta_max, int n_theta, real r_min, real r_max,
                         int n_r, Vec3 apex);
  void build_points();
  void validate() const;
};

// A beamformed complex image.
struct Frame {
  ScanGrid grid;
  std::vector<cplx> data;
  real demodulation_frequency = 0.0f;
  double timestamp = 0.0;
  std::int64_t sequence = 0;

  void allocate() { data.assign(static_cast<std::size_t>(grid.n_pixels()), cplx(0, 0)); }
  const cplx& at(int i0, int i1) const { return data[static_cast<std::size_t>(i0) * grid.n_axis1 + i1]; }
  cplx& at(int i0, int i1) { return data[static_cast<std::size_t>(i0) * grid.n_axis1 + i1]; }
};

enum class Window : std::uint8_t { Rect = 0, Hann = 1, Hamming = 2, Tukey = 3, Blackman = 4 };

real window_value(Window w, real u, real tukey_alpha = 0.5f);
Window window_from_string(const std::string& name);

}  // namespace usx
