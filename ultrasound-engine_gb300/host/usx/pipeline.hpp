// usx/pipeline.hpp — the streaming front end (drop-in for the reference's
// core/include/usx/pipeline.hpp:23-77). Keeps the raw acquisition, IQ, frame
// and display buffers resident on the GPU between stages; only the final
// frame (or display image) is copied back to the host.
#pragma once

#include <memory>
#include <vector>

#include "usx/beamformer.hpp"
#include "usx/demodulate.hpp"
#include "usx/doppler.hpp"
#include "usx/postprocess.hpp"
#include "usx/runtime.hpp"
#include "usx/types.hpp"

namespace usx {

struct PipelineConfig {
  DemodConfig demod;
  BeamformerConfig beamformer;
  real dynamic_range_db = 60.0f;
  real gain_db = 0.0f;
  bool apply_tgc = true;
  real reference_smoothing = 0.85f;
};

struct PipelineStats {
  double demodulate_ms = 0;
  double beamform_ms = 0;
  double postprocess_ms = 0;
  double total_ms = 0;
  double frames_per_second() const { return total_ms > 0 ? 1000.0 / total_ms : 0.0; }
};

class ImagingPipeline {
 public:
  ImagingPipeline(ScanGrid grid, PipelineConfig config = {});

  Frame process_frame(const ChannelData& data);
  std::vector<real> process_display(const ChannelData& data);
  std::vector<real> to_display(const Frame& frame, const Medium& medium);

  const ScanGrid& grid() const { return grid_; }
  const PipelineStats& stats() const { return stats_; }
  PipelineConfig& config() { return config_; }
  const PipelineConfig& config() const { return config_; }
  std::int64_t frame_count() const { return frame_count_; }
  void reset();

 private:
  // The acquisition on the device, demodulated if it was RF; `meta` describes it.
  const void* to_device_iq(const ChannelData& data, ChannelData& meta);
  // Envelope, TGC, peak and log compression of a device frame on `grid`; only
  // the peak (4 bytes) and the display image come back to the host.
  std::vector<real> display_device(const void* d_frame, const ScanGrid& grid, real fdem, const Medium& medium);

  ScanGrid grid_;
  PipelineConfig config_;
  Beamformer beamformer_;
  PipelineStats stats_;
  real reference_ = 0.0f;
  std::int64_t frame_count_ = 0;
  std::shared_ptr<rt::DeviceBuffer> grid_points_;  // grid_'s points on the device, uploaded once
};

}  // namespace usx
