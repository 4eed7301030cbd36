// pipeline.cpp — the streaming front end (behaviour of the reference's
// core/src/pipeline.cpp:14-79). Demodulation, beamforming and the display
// chain run back to back on the device; the raw acquisition goes up once and
// only the frame (or display image) comes back.
#include "usx/pipeline.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>

#include "desc.hpp"
#include "usx/runtime.hpp"

namespace usx {

ImagingPipeline::ImagingPipeline(ScanGrid grid, PipelineConfig config)
    : grid_(std::move(grid)), config_(config), beamformer_(config.beamformer) {
  grid_.validate();
}

void ImagingPipeline::reset() {
  reference_ = 0.0f;
  frame_count_ = 0;
  stats_ = PipelineStats{};
}

const void* ImagingPipeline::to_device_iq(const ChannelData& data, ChannelData& meta) {
  data.validate();
  meta.probe = data.probe;
  meta.medium = data.medium;
  meta.transmits = data.transmits;
  meta.acq = data.acq;
  meta.is_iq = true;
  meta.demodulation_frequency = data.demodulation_frequency;
  if (data.is_iq) {
    if (data.iq.size() != data.size()) throw std::invalid_argument("ChannelData has no IQ samples");
    void* d_iq = rt::slot(11, data.iq.size() * sizeof(cplx));
    rt::h2d(d_iq, data.iq.data(), data.iq.size() * sizeof(cplx));
    return d_iq;
  }
  // RF goes up once; the IQ stays on the device for the beamformer.
  if (data.rf.size() != data.size()) throw std::invalid_argument("demodulate: input has no RF samples");
  const double t = rt::now_ms();
  const int dec = std::max(1, config_.demod.decimation);
  meta.acq.sampling_frequency = data.acq.sampling_frequency / dec;
  meta.acq.n_samples = (data.acq.n_samples + dec - 1) / dec;
  const std::size_t n_iq = meta.size();
  void* d_rf = rt::slot(10, data.rf.size() * sizeof(float));
  void* d_iq = rt::slot(11, n_iq * sizeof(cplx));
  rt::h2d(d_rf, data.rf.data(), data.rf.size() * sizeof(float));
  desc::Channel ch(data);
  const usx_demod_config dc = desc::demod(config_.demod);
  float fdem = 0.0f;
  rt::check(usx_cu_demodulate(rt::ctx(), &ch.cd, &dc, static_cast<const float*>(d_rf), static_cast<float*>(d_iq),
                              &fdem),
            "demodulate");
  meta.demodulation_frequency = fdem;
  stats_.demodulate_ms = rt::now_ms() - t;
  return d_iq;
}

Frame ImagingPipeline::process_frame(const ChannelData& data) {
  const double t_start = rt::now_ms();
  stats_ = PipelineStats{};
  Frame frame;
  if (!data.is_iq) {
    ChannelData meta;
    const void* d_iq = to_device_iq(data, meta);
    const double t_bf = rt::now_ms();
    beamformer_.config() = config_.beamformer;
    frame = beamformer_.beamform_device(meta, d_iq, grid_);
    stats_.beamform_ms = rt::now_ms() - t_bf;
  } else {
    const double t_bf = rt::now_ms();
    beamformer_.config() = config_.beamformer;
    frame = beamformer_.beamform(data, grid_);
    stats_.beamform_ms = rt::now_ms() - t_bf;
  }
  frame.sequence = frame_count_++;
  stats_.total_ms = rt::now_ms() - t_start;
  return frame;
}

std::vector<real> ImagingPipeline::display_device(const void* d_frame, const ScanGrid& grid, real fdem,
                                                  const Medium& medium) {
  const int n0 = grid.n_axis0, n1 = grid.n_axis1;
  const std::size_t n = static_cast<std::size_t>(grid.n_pixels());
  std::vector<real> img(n);
  if (n == 0) return img;
  float* d_env = static_cast<float*>(rt::slot(12, n * sizeof(float)));
  float* d_tgc = static_cast<float*>(rt::slot(13, n * sizeof(float)));
  float* d_img = static_cast<float*>(rt::slot(14, n * sizeof(float)));
  rt::check(usx_cu_envelope(rt::ctx(), static_cast<const float*>(d_frame), n0, n1, fdem, d_env), "envelope");
  const float* env = d_env;
  if (config_.apply_tgc) {
    // Gain on the envelope, as the reference's pipeline applies it (cosmetic:
    // the beamformer already saw the full dynamic range).
    real f0 = fdem;
    if (f0 <= 0.0f) f0 = 5.0e6f;
    const void* d_pts = nullptr;
    const std::size_t pts_bytes = n * 3 * sizeof(float);
    if (&grid == &grid_ || (grid.points.size() == grid_.points.size() &&
                            std::memcmp(grid.points.data(), grid_.points.data(), pts_bytes) == 0)) {
      if (!grid_points_) {
        auto buf = std::make_shared<rt::DeviceBuffer>();
        rt::h2d(buf->ensure(pts_bytes), desc::points(grid_), pts_bytes);
        grid_points_ = buf;
      }
      d_pts = grid_points_->get();
    } else {
      void* d = rt::slot(15, pts_bytes);
      rt::h2d(d, desc::points(grid), pts_bytes);
      d_pts = d;
    }
    rt::check(usx_cu_apply_tgc(rt::ctx(), d_env, n0, n1, static_cast<const float*>(d_pts), medium.attenuation, f0,
                               d_tgc),
              "apply_tgc");
    env = d_tgc;
  }
  real peak = 0.0f;
  rt::check(usx_cu_max(rt::ctx(), env, static_cast<int64_t>(n), &peak), "max");
  peak = std::max(peak, 0.0f);
  if (peak > 0.0f) {
    const real a = std::clamp(config_.reference_smoothing, 0.0f, 0.999f);
    reference_ = (reference_ > 0.0f) ? (a * reference_ + (1.0f - a) * peak) : peak;
  }
  rt::check(usx_cu_log_compress(rt::ctx(), env, static_cast<int64_t>(n), config_.dynamic_range_db, config_.gain_db,
                                reference_ > 0.0f ? reference_ : -1.0f, d_img),
            "log_compress");
  rt::d2h(img.data(), d_img, n * sizeof(float));
  return img;
}

std::vector<real> ImagingPipeline::to_display(const Frame& frame, const Medium& medium) {
  const double t = rt::now_ms();
  const std::size_t n = static_cast<std::size_t>(frame.grid.n_pixels());
  if (frame.data.size() != n) throw std::invalid_argument("envelope: frame data does not match its grid");
  std::vector<real> img;
  if (n == 0) {
    img.resize(0);
  } else {
    void* d_frame = rt::slot(9, n * sizeof(cplx));
    rt::h2d(d_frame, frame.data.data(), n * sizeof(cplx));
    img = display_device(d_frame, frame.grid, frame.demodulation_frequency, medium);
  }
  stats_.postprocess_ms += rt::now_ms() - t;
  stats_.total_ms += stats_.postprocess_ms;
  return img;
}

std::vector<real> ImagingPipeline::process_display(const ChannelData& data) {
  // process_frame followed by to_display, with the frame kept on the device.
  const double t_start = rt::now_ms();
  stats_ = PipelineStats{};
  ChannelData meta;
  const void* d_iq = to_device_iq(data, meta);
  const double t_bf = rt::now_ms();
  beamformer_.config() = config_.beamformer;
  void* d_frame = rt::slot(9, static_cast<std::size_t>(grid_.n_pixels()) * sizeof(cplx));
  beamformer_.beamform_into(meta, d_iq, grid_, d_frame);
  stats_.beamform_ms = rt::now_ms() - t_bf;
  ++frame_count_;
  stats_.total_ms = rt::now_ms() - t_start;
  const double t = rt::now_ms();
  std::vector<real> img = display_device(d_frame, grid_, meta.demodulation_frequency, data.medium);
  stats_.postprocess_ms += rt::now_ms() - t;
  stats_.total_ms += stats_.postprocess_ms;
  return img;
}

}  // namespace usx
