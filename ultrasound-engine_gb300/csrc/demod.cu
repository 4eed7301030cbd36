// demod.cu — quadrature demodulation + decimating FIR (reference
// demodulate.cpp:36-121), HBM-bound.
//
// Layout: RF [trace][n_in] float -> IQ [trace][n_out] complex, trace =
// event*n_channels + channel.
//
// demod_slide_kernel<NT> (no decimation, NT taps; the default 33-tap filter):
// a block of 8 warps owns 8 traces x 256 output samples. It stages the 288
// input samples those outputs need for each trace in shared memory, already
// mixed to baseband (the rotator once per block for all 8 traces), with one
// pad word every 8 samples so that lanes reading 8-sample strides hit distinct
// banks. Each warp then filters one trace: lane l produces outputs 8l..8l+7
// from one descending pass over its 8+NT-1 window samples, each sample read
// from shared memory once and multiplied into every output it reaches (the
// taps are compile-time constant-bank operands). Every output still sums its
// taps in ascending order, as the reference does. The outputs go back through
// the warp's own shared-memory row so the IQ stores are coalesced. Samples
// outside the trace are staged as zeros: an output whose tap range the
// reference clips (j_lo > 0 or j_hi < NT-1) then adds exact zeros outside
// that range, which leaves its sum unchanged.
//
// demod_kernel (any decimation or tap count): a block owns 8 traces x 128
// outputs, one output per thread per trace, taps read from the parameter
// block in a runtime loop.
//
// Arithmetic follows the reference term by term (mix, then tap product and
// accumulation in ascending tap order, then x2); the tap product and the
// accumulation are one FMA (~1e-7 relative from the reference's separate
// multiply and add); the mixing phase -2*pi*f*t(n) is evaluated on the device
// with sincosf.
#include <algorithm>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kMaxTaps = 255;
constexpr int kTraces = 8;
constexpr int kOut = 128;

struct DemodParams {
  const float* rf;
  float2* iq;
  long n_traces;
  int n_in, n_out, dec, n_taps, gd;
  float neg_two_pi_f;   // -2*pi*fdem, float-rounded as the reference folds it
  float t0, fs;
  float h[kMaxTaps];
};

__global__ void __launch_bounds__(kOut) demod_kernel(const DemodParams p) {
  extern __shared__ float4 smem_raw[];
  const int span = kOut * p.dec + p.n_taps - 1;
  float2* rot = reinterpret_cast<float2*>(smem_raw);          // [span]
  float2* mixed = rot + span;                                 // [kTraces][span]

  const int k0 = blockIdx.y * kOut;
  const long tr0 = static_cast<long>(blockIdx.x) * kTraces;
  // Input index of mixed[0]: centre(k0) - (n_taps - 1).
  const int n_base = k0 * p.dec + p.gd - (p.n_taps - 1);

  for (int s = threadIdx.x; s < span; s += blockDim.x) {
    const int n = n_base + s;
    float2 r = make_float2(0.f, 0.f);
    if (n >= 0 && n < p.n_in) {
      const float t = p.t0 + static_cast<float>(n) / p.fs;
      const float ph = p.neg_two_pi_f * t;
      float sv, cv;
      sincosf(ph, &sv, &cv);
      r = make_float2(cv, sv);
    }
    rot[s] = r;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < kTraces * span; q += blockDim.x) {
    const int t = q / span, s = q - t * span;
    const long tr = tr0 + t;
    const int n = n_base + s;
    float x = 0.f;
    if (tr < p.n_traces && n >= 0 && n < p.n_in) x = __ldg(p.rf + tr * p.n_in + n);
    const float2 r = rot[s];
    mixed[q] = make_float2(r.x * x, r.y * x);
  }
  __syncthreads();

  const int k = k0 + threadIdx.x;
  if (k >= p.n_out) return;
  const int centre = k * p.dec + p.gd;
  const int j_lo = max(0, centre - p.n_in + 1);
  const int j_hi = min(p.n_taps - 1, centre);
  // mixed index of input sample (centre - j) is centre - j - n_base.
  const int off = centre - n_base;
#pragma unroll
  for (int t = 0; t < kTraces; ++t) {
    const long tr = tr0 + t;
    if (tr >= p.n_traces) break;
    const float2* m = mixed + t * span;
    float ar = 0.f, ai = 0.f;
    for (int j = j_lo; j <= j_hi; ++j) {
      const float2 v = m[off - j];
      const float hj = p.h[j];
      ar = fmaf(v.x, hj, ar);
      ai = fmaf(v.y, hj, ai);
    }
    p.iq[tr * p.n_out + k] = make_float2(ar * 2.0f, ai * 2.0f);
  }
}

constexpr int kSlideR = 8;                       // outputs per lane
constexpr int kSlideWarps = 8;                   // traces per block
constexpr int kSlideOut = 32 * kSlideR;          // outputs per trace segment

// Shared-memory slot of window sample s: one pad word after every 8 samples.
__device__ __forceinline__ int slide_pos(int s) { return s + (s >> 3); }

template <int NT>
__global__ void __launch_bounds__(32 * kSlideWarps) demod_slide_kernel(const DemodParams p) {
  constexpr int W = kSlideOut + NT - 1;          // window samples per trace
  constexpr int ROW = W + W / 8 + 1;             // padded row length (float2)
  __shared__ float2 rot[W];
  __shared__ float2 mixed[kSlideWarps][ROW];

  const int k0 = blockIdx.y * kSlideOut;
  const long tr0 = static_cast<long>(blockIdx.x) * kSlideWarps;
  const int n_base = k0 + p.gd - (NT - 1);       // input index of window sample 0

  for (int s = threadIdx.x; s < W; s += blockDim.x) {
    const int n = n_base + s;
    float2 r = make_float2(0.f, 0.f);
    if (n >= 0 && n < p.n_in) {
      const float t = p.t0 + static_cast<float>(n) / p.fs;
      const float ph = p.neg_two_pi_f * t;
      float sv, cv;
      sincosf(ph, &sv, &cv);
      r = make_float2(cv, sv);
    }
    rot[s] = r;
  }
  // Raw samples first (independent loads in flight), then mix once the rotator is in.
  constexpr int kPer = (kSlideWarps * W + 32 * kSlideWarps - 1) / (32 * kSlideWarps);
  float x[kPer];
#pragma unroll
  for (int m = 0; m < kPer; ++m) {
    const int q = threadIdx.x + m * 32 * kSlideWarps;
    const int t = q / W, s = q - t * W;
    const long tr = tr0 + t;
    const int n = n_base + s;
    x[m] = (q < kSlideWarps * W && tr < p.n_traces && n >= 0 && n < p.n_in) ? __ldg(p.rf + tr * p.n_in + n) : 0.f;
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < kPer; ++m) {
    const int q = threadIdx.x + m * 32 * kSlideWarps;
    if (q < kSlideWarps * W) {
      const int t = q / W, s = q - t * W;
      const float2 r = rot[s];
      mixed[t][slide_pos(s)] = make_float2(r.x * x[m], r.y * x[m]);
    }
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long tr = tr0 + warp;
  if (tr >= p.n_traces) return;
  float2* row = mixed[warp];
  // (re, im) of each output accumulate as one packed pair (two FP32 FMAs per
  // instruction, each rounded as fmaf).
  float2 acc[kSlideR];
#pragma unroll
  for (int r = 0; r < kSlideR; ++r) acc[r] = make_float2(0.f, 0.f);
  // Window sample i of this lane is s = 8*lane + i; output r uses tap
  // j = r + NT - 1 - i, so descending i visits each output's taps in ascending j.
#pragma unroll
  for (int i = kSlideR + NT - 2; i >= 0; --i) {
    const float2 v = row[slide_pos(kSlideR * lane + i)];
#pragma unroll
    for (int r = 0; r < kSlideR; ++r) {
      const int j = r + NT - 1 - i;
      if (j >= 0 && j < NT) acc[r] = __ffma2_rn(v, make_float2(p.h[j], p.h[j]), acc[r]);
    }
  }
  __syncwarp();
#pragma unroll
  for (int r = 0; r < kSlideR; ++r)
    row[slide_pos(kSlideR * lane + r)] = make_float2(acc[r].x * 2.0f, acc[r].y * 2.0f);
  __syncwarp();
  float2* dst = p.iq + tr * p.n_out + k0;
  const int n_here = min(kSlideOut, p.n_out - k0);
#pragma unroll
  for (int q = 0; q < kSlideR; ++q) {
    const int o = lane + 32 * q;
    if (o < n_here) dst[o] = row[slide_pos(o)];
  }
}

}  // namespace
}  // namespace usxcu

using namespace usxcu;

extern "C" int usx_cu_demodulate(usx_ctx* ctx, const usx_channel_desc* cd,
                                 const usx_demod_config* cfg, const float* rf, float* iq,
                                 float* out_fdem) {
  if (!ctx || !cd || !cfg || !rf || !iq) return fail(USX_ERR_INVALID, "usx_cu_demodulate: null argument");
  if (cd->is_iq) return fail(USX_ERR_INVALID, "usx_cu_demodulate: input already holds IQ");
  if (int rc = validate_channel(*cd)) return rc;
  const float fdem = cfg->demodulation_frequency > 0.0f ? cfg->demodulation_frequency
                                                        : cd->probe.center_frequency;
  const int dec = std::max(1, cfg->decimation);
  const float fs = cd->acq.sampling_frequency;
  DemodParams p;
  int n_taps = 0;
  usx_cu_design_lowpass(cfg->filter_taps, cfg->cutoff_fraction * fdem / fs, nullptr, 0, &n_taps);
  if (n_taps > kMaxTaps) return fail(USX_ERR_UNSUPPORTED, "usx_cu_demodulate: more than 255 filter taps");
  if (dec > 32) return fail(USX_ERR_UNSUPPORTED, "usx_cu_demodulate: decimation above 32");
  usx_cu_design_lowpass(cfg->filter_taps, cfg->cutoff_fraction * fdem / fs, p.h, kMaxTaps, &n_taps);
  p.rf = rf;
  p.iq = reinterpret_cast<float2*>(iq);
  p.n_traces = static_cast<long>(cd->n_events) * cd->probe.n_elements;
  p.n_in = cd->acq.n_samples;
  p.n_out = (p.n_in + dec - 1) / dec;
  p.dec = dec;
  p.n_taps = n_taps;
  p.gd = n_taps / 2;
  p.neg_two_pi_f = -2.0f * kPi * fdem;
  p.t0 = cd->acq.t0;
  p.fs = fs;
  if (out_fdem) *out_fdem = fdem;
  if (dec == 1 && (n_taps == 33 || n_taps == 21)) {
    const long gx = (p.n_traces + kSlideWarps - 1) / kSlideWarps;
    const int gy = ceil_div(p.n_out, kSlideOut);
    if (gx > 0x7fffffffL || gy > 65535) return fail(USX_ERR_UNSUPPORTED, "usx_cu_demodulate: acquisition too large");
    dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
    prof_begin(ctx, "demod_slide_kernel");
    if (n_taps == 33)
      demod_slide_kernel<33><<<grid, 32 * kSlideWarps, 0, ctx->stream>>>(p);
    else
      demod_slide_kernel<21><<<grid, 32 * kSlideWarps, 0, ctx->stream>>>(p);
    prof_end(ctx);
    USX_CHECK_LAUNCH("demod_slide_kernel");
    return USX_OK;
  }
  const int span = kOut * dec + n_taps - 1;
  const size_t smem = sizeof(float2) * static_cast<size_t>(span) * (1 + kTraces);
  if (smem > 48 * 1024)
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(demod_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  const long gx = (p.n_traces + kTraces - 1) / kTraces;
  const int gy = ceil_div(p.n_out, kOut);
  if (gx > 0x7fffffffL || gy > 65535) return fail(USX_ERR_UNSUPPORTED, "usx_cu_demodulate: acquisition too large");
  dim3 grid(static_cast<unsigned>(gx), static_cast<unsigned>(gy));
  prof_begin(ctx, "demod_kernel");
  demod_kernel<<<grid, kOut, smem, ctx->stream>>>(p);
  prof_end(ctx);
  USX_CHECK_LAUNCH("demod_kernel");
  return USX_OK;
}
