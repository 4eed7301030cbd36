// postprocess.cpp — host front ends of the GPU post-processing kernels
// (behaviour of the reference's core/src/postprocess.cpp:67-178).
#include "usx/postprocess.hpp"

#include "desc.hpp"
#include "usx/runtime.hpp"

namespace usx {

std::vector<real> envelope(const Frame& frame) {
  const int n0 = frame.grid.n_axis0, n1 = frame.grid.n_axis1;
  const std::size_t n = static_cast<std::size_t>(n0) * n1;
  std::vector<real> env(n);
  if (n == 0) return env;
  if (frame.data.size() != n) throw std::invalid_argument("envelope: frame data does not match its grid");
  void* d_in = rt::slot(5, n * sizeof(cplx));
  void* d_out = rt::slot(6, n * sizeof(float));
  rt::h2d(d_in, frame.data.data(), n * sizeof(cplx));
  rt::check(usx_cu_envelope(rt::ctx(), static_cast<const float*>(d_in), n0, n1,
                            frame.demodulation_frequency, static_cast<float*>(d_out)),
            "envelope");
  rt::d2h(env.data(), d_out, n * sizeof(float));
  return env;
}

std::vector<real> apply_tgc(const std::vector<real>& env, const ScanGrid& grid,
                            real attenuation_db_cm_mhz, real center_frequency_hz) {
  const std::size_t n = static_cast<std::size_t>(grid.n_pixels());
  if (env.size() < n) throw std::invalid_argument("apply_tgc: envelope smaller than the grid");
  std::vector<real> out(env.size());
  if (n == 0) return out;
  void* d_env = rt::slot(5, n * sizeof(float));
  void* d_pts = rt::slot(6, n * 3 * sizeof(float));
  void* d_out = rt::slot(7, n * sizeof(float));
  rt::h2d(d_env, env.data(), n * sizeof(float));
  rt::h2d(d_pts, desc::points(grid), n * 3 * sizeof(float));
  rt::check(usx_cu_apply_tgc(rt::ctx(), static_cast<const float*>(d_env), grid.n_axis0, grid.n_axis1,
                             static_cast<const float*>(d_pts), attenuation_db_cm_mhz,
                             center_frequency_hz, static_cast<float*>(d_out)),
            "apply_tgc");
  rt::d2h(out.data(), d_out, n * sizeof(float));
  return out;
}

std::vector<real> log_compress(const std::vector<real>& env, real dynamic_range_db, real gain_db,
                               real reference) {
  std::vector<real> out(env.size());
  if (env.empty()) return out;
  void* d_env = rt::slot(5, env.size() * sizeof(float));
  void* d_out = rt::slot(7, env.size() * sizeof(float));
  rt::h2d(d_env, env.data(), env.size() * sizeof(float));
  rt::check(usx_cu_log_compress(rt::ctx(), static_cast<const float*>(d_env),
                                static_cast<int64_t>(env.size()), dynamic_range_db, gain_db, reference,
                                static_cast<float*>(d_out)),
            "log_compress");
  rt::d2h(out.data(), d_out, env.size() * sizeof(float));
  return out;
}

ScanConverted scan_convert(const std::vector<real>& image, const ScanGrid& grid, int width, int height,
                           real fill_value) {
  grid.validate();
  const std::size_t n = static_cast<std::size_t>(grid.n_pixels());
  if (image.size() < n) throw std::invalid_argument("scan_convert: image smaller than the grid");
  ScanConverted sc;
  sc.width = width;
  sc.height = height;
  sc.pixels.assign(static_cast<std::size_t>(std::max(width, 0)) * std::max(height, 0), fill_value);
  if (width <= 0 || height <= 0) return sc;
  void* d_img = rt::slot(5, n * sizeof(float));
  void* d_px = rt::slot(7, sc.pixels.size() * sizeof(float));
  rt::h2d(d_img, image.data(), n * sizeof(float));
  const usx_grid_desc g = desc::grid(grid);
  float ext[4] = {0, 0, 0, 0};
  rt::check(usx_cu_scan_convert(rt::ctx(), static_cast<const float*>(d_img), &g, desc::points(grid),
                                width, height, fill_value, static_cast<float*>(d_px), ext),
            "scan_convert");
  rt::d2h(sc.pixels.data(), d_px, sc.pixels.size() * sizeof(float));
  sc.x_min = ext[0];
  sc.x_max = ext[1];
  sc.z_min = ext[2];
  sc.z_max = ext[3];
  return sc;
}

}  // namespace usx
