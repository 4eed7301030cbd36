// usx/beamformer.hpp — delay, apodize, combine (drop-in for the reference's
// core/include/usx/beamformer.hpp:40-138); runs on the GPU through cached
// beamforming plans (usx_cu_bf_plan_*).
#pragma once

#include <cstdint>
#include <memory>
#include <vector>

#include "usx/types.hpp"

namespace usx {

// LearnedMV has no reference counterpart: the learned minimum-variance
// surrogate (usx/learned.hpp) with plain MV as per-pixel fallback.
enum class Combiner : std::uint8_t { DAS = 0, DMAS = 1, MV = 2, LearnedMV = 3 };
enum class Compounding : std::uint8_t { Coherent = 0, Incoherent = 1, Select = 2 };

// How minimum variance is solved (no counterpart in the reference, whose
// solver is its FP32 Cholesky): Tensor = BF16 covariance on the tensor cores
// with FP32 accumulation, one refinement step against the FP32 covariance and
// an FP64 re-solve where it fails (within 1e-3 of the reference); Exact = the
// reference's FP32 operation order (within 1e-4, several times slower); FP32 =
// FP32 covariance by the lag recurrence and one FP32 solve (the reference's
// precision in another summation order). For LearnedMV the solver of the
// gated pixels: FP32, else the tensor-core one.
enum class MvSolver { Tensor = 0, Exact = 1, FP32 = 2 };

struct BeamformerConfig {
  real f_number = 1.75f;
  Window rx_window = Window::Hann;
  real tukey_alpha = 0.5f;
  Combiner combiner = Combiner::DAS;
  Compounding compounding = Compounding::Coherent;
  bool transmit_weighting = true;
  bool coherence_factor = false;
  int mv_subarray = 16;
  real mv_diagonal_loading = 1e-2f;
  int mv_range_average = 2;
  // Fields below have no counterpart in the reference.
  MvSolver mv_solver = MvSolver::FP32;
  // Learned minimum variance: the gate on the network's distortionless
  // residual, the DFT beams of the subspace refinement (< 0: none), the gate
  // on the network direction's share of the power reduction and the gate on
  // tr(R) over its depth's level. Negative gates and a refinement of -2 mean
  // "as recorded with the weights" (their ".gate" file).
  real learned_gate = -1.0f;
  int learned_refine = -2;
  real learned_share_gate = -1.0f;
  real learned_level_gate = -1.0f;
  void validate() const;
};

class PlanCache;

class Beamformer {
 public:
  explicit Beamformer(BeamformerConfig config = {});
  ~Beamformer();
  Beamformer(const Beamformer& o);
  Beamformer& operator=(const Beamformer& o);

  Frame beamform(const ChannelData& data, const ScanGrid& grid, int event_begin = 0,
                 int event_end = -1) const;
  std::vector<Frame> beamform_sequence(const ChannelData& data, const ScanGrid& grid,
                                       int events_per_frame) const;

  // Device-resident entry (no reference counterpart): `meta` carries the
  // channel metadata only (its sample vectors may be empty) and `device_data`
  // points at the matching samples already in GPU memory.
  Frame beamform_device(const ChannelData& meta, const void* device_data, const ScanGrid& grid,
                        int event_begin = 0, int event_end = -1) const;
  // As beamform_device, but the frame stays on the device: written to
  // `device_frame` ([n_axis0][n_axis1] complex), nothing is copied back.
  void beamform_into(const ChannelData& meta, const void* device_data, const ScanGrid& grid,
                     void* device_frame, int event_begin = 0, int event_end = -1) const;

  const BeamformerConfig& config() const { return config_; }
  BeamformerConfig& config() { return config_; }

 private:
  BeamformerConfig config_;
  std::shared_ptr<PlanCache> plans_;
};

real transmit_sensitivity(const Probe& probe, const Transmit& tx, const Vec3& point,
                          real wavelength);

}  // namespace usx
