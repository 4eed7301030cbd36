// pipeline.cpp — the streaming front end (behaviour of the reference's
// core/src/pipeline.cpp:14-79). Demodulation, beamforming and the display
// chain run back to back on the device; the raw acquisition goes up once and
// only the frame (or display image) comes back.
#include "usx/pipeline.hpp"

#include <algorithm>
#include <cmath>

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

Frame ImagingPipeline::process_frame(const ChannelData& data) {
  const double t_start = rt::now_ms();
  stats_ = PipelineStats{};
  Frame frame;
  if (!data.is_iq) {
    // RF goes up once; the IQ stays on the device for the beamformer.
    data.validate();
    if (data.rf.size() != data.size()) throw std::invalid_argument("demodulate: input has no RF samples");
    const double t = rt::now_ms();
    const int dec = std::max(1, config_.demod.decimation);
    ChannelData meta;
    meta.probe = data.probe;
    meta.medium = data.medium;
    meta.transmits = data.transmits;
    meta.acq = data.acq;
    meta.acq.sampling_frequency = data.acq.sampling_frequency / dec;
    meta.acq.n_samples = (data.acq.n_samples + dec - 1) / dec;
    meta.is_iq = true;
    const std::size_t n_iq = meta.size();
    void* d_rf = rt::slot(10, data.rf.size() * sizeof(float));
    void* d_iq = rt::slot(11, n_iq * sizeof(cplx));
    rt::h2d(d_rf, data.rf.data(), data.rf.size() * sizeof(float));
    desc::Channel ch(data);
    const usx_demod_config dc = desc::demod(config_.demod);
    float fdem = 0.0f;
    rt::check(usx_cu_demodulate(rt::ctx(), &ch.cd, &dc, static_cast<const float*>(d_rf),
                                static_cast<float*>(d_iq), &fdem),
              "demodulate");
    meta.demodulation_frequency = fdem;
    stats_.demodulate_ms = rt::now_ms() - t;
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

std::vector<real> ImagingPipeline::to_display(const Frame& frame, const Medium& medium) {
  const double t = rt::now_ms();
  std::vector<real> env = envelope(frame);
  if (config_.apply_tgc) {
    real f0 = frame.demodulation_frequency;
    if (f0 <= 0.0f) f0 = 5.0e6f;
    env = apply_tgc(env, frame.grid, medium.attenuation, f0);
  }
  real peak = 0.0f;
  for (real v : env) peak = std::max(peak, v);
  if (peak > 0.0f) {
    const real a = std::clamp(config_.reference_smoothing, 0.0f, 0.999f);
    reference_ = (reference_ > 0.0f) ? (a * reference_ + (1.0f - a) * peak) : peak;
  }
  std::vector<real> img = log_compress(env, config_.dynamic_range_db, config_.gain_db,
                                       reference_ > 0.0f ? reference_ : -1.0f);
  stats_.postprocess_ms += rt::now_ms() - t;
  stats_.total_ms += stats_.postprocess_ms;
  return img;
}

std::vector<real> ImagingPipeline::process_display(const ChannelData& data) {
  const Frame frame = process_frame(data);
  return to_display(frame, data.medium);
}

}  // namespace usx
