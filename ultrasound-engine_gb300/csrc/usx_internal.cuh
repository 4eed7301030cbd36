// usx_internal.cuh — shared device helpers and the context behind the C-ABI.
//
// Every translation unit of libusx_cu.so is compiled for sm_103a with
// -fmad=false: a plain `a * b + c` is then two IEEE-rounded operations, exactly
// as the reference's x86-64 float code evaluates it, so the geometry, index and
// phase chains reproduce the reference bit for bit. Kernels that may contract
// (tensor-core epilogues, the learned combiner) call fmaf() explicitly.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/usx_cu.h"

namespace usxcu {

// --------------------------------------------------------------- host side

// Thread-local last error (usx_cu_last_error).
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);
int cuda_fail(cudaError_t e, const char* where);

#define USX_CUDA(call)                                   \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return ::usxcu::cuda_fail(_e, #call); \
  } while (0)

#define USX_CHECK_LAUNCH(name)                           \
  do {                                                   \
    cudaError_t _e = cudaGetLastError();                 \
    if (_e != cudaSuccess) return ::usxcu::cuda_fail(_e, name); \
  } while (0)

}  // namespace usxcu

#include <vector>

// One timed kernel launch (profiling mode only).
struct usx_prof_rec {
  const char* name;
  cudaEvent_t start, stop;
};

// The context: one device, one stream, and a grow-only scratch arena so that a
// steady-state frame allocates nothing.
struct usx_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  void* scratch = nullptr;
  size_t scratch_bytes = 0;
  int* d_status = nullptr;     // device-side status word written by kernels
  void* mv_cov = nullptr;      // minimum variance: covariances between the tcgen05 and solve stages
  size_t mv_cov_bytes = 0;
  int sm_count = 0;
  bool profiling = false;      // record CUDA events around every launch
  std::vector<usx_prof_rec> prof;
  std::vector<cudaEvent_t> event_pool;
};

namespace usxcu {

// Scratch memory of at least `bytes` on the context's device (grows, never shrinks).
int scratch(usx_ctx* ctx, size_t bytes, void** out);

// Profiling: when enabled, events are recorded on the context's stream before
// and after each launch, so per-kernel device time is measured on the stream
// the kernel runs on. No-ops otherwise.
void prof_begin(usx_ctx* ctx, const char* name);
void prof_end(usx_ctx* ctx);

// Launch-configuration queries, cached per device and kernel so that a plan
// that has run once makes no attribute or occupancy call again (its launches
// can then be captured into a CUDA graph): smem_limit raises a kernel's
// dynamic shared-memory limit only when `bytes` exceeds what was set before;
// occupancy returns cudaOccupancyMaxActiveBlocksPerMultiprocessor.
int smem_limit(const void* func, size_t bytes);
int occupancy(const void* func, int threads, size_t smem, int* blocks_per_sm);

// ------------------------------------------------------------- device side

constexpr float kPi = 3.14159265358979323846f;

struct cplx {
  float re, im;
};

__device__ __forceinline__ cplx mk(float re, float im) { return cplx{re, im}; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return mk(a.re + b.re, a.im + b.im); }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return mk(a.re - b.re, a.im - b.im); }
// std::complex<float> product as GCC expands it: (ac - bd, ad + bc).
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return mk(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ cplx cscale(cplx a, float s) { return mk(a.re * s, a.im * s); }
__device__ __forceinline__ cplx cdivr(cplx a, float s) { return mk(a.re / s, a.im / s); }
__device__ __forceinline__ cplx cconj(cplx a) { return mk(a.re, -a.im); }
__device__ __forceinline__ float cnorm(cplx a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ float cabsf_(cplx a) { return hypotf(a.re, a.im); }
// libgcc divides std::complex<float> in double precision; so do we where the
// reference divides by a complex value.
__device__ __forceinline__ cplx cdiv_wide(cplx a, cplx b) {
  const double aa = a.re, bb = a.im, cc = b.re, dd = b.im;
  const double den = cc * cc + dd * dd;
  return mk(static_cast<float>((aa * cc + bb * dd) / den), static_cast<float>((bb * cc - aa * dd) / den));
}

__device__ __forceinline__ float fclamp(float v, float lo, float hi) {
  return v < lo ? lo : (hi < v ? hi : v);
}

// Window value at u in [-1, 1] (reference types.cpp:126-148).
__device__ __forceinline__ float window_value(int w, float u, float alpha) {
  if (u < -1.0f || u > 1.0f) return 0.0f;
  const float t = 0.5f * (u + 1.0f);
  const float two_pi = 2.0f * kPi;
  switch (w) {
    case USX_WIN_RECT: return 1.0f;
    case USX_WIN_HANN: return 0.5f * (1.0f - cosf(two_pi * t));
    case USX_WIN_HAMMING: return 0.54f - 0.46f * cosf(two_pi * t);
    case USX_WIN_BLACKMAN:
      return 0.42f - 0.5f * cosf(two_pi * t) + 0.08f * cosf(4.0f * kPi * t);
    case USX_WIN_TUKEY: {
      const float a = fclamp(alpha, 0.0f, 1.0f);
      if (a <= 0.0f) return 1.0f;
      if (t < a * 0.5f) return 0.5f * (1.0f + cosf(two_pi / a * (t - a * 0.5f)));
      if (t > 1.0f - a * 0.5f) return 0.5f * (1.0f + cosf(two_pi / a * (t - 1.0f + a * 0.5f)));
      return 1.0f;
    }
  }
  return 1.0f;
}

// Receive aperture weight of an element at (ex, 0, 0) for a pixel
// (reference geometry.cpp:123-130).
__device__ __forceinline__ float aperture_weight(float ex, float px, float pz, float f_number,
                                                 int w, float alpha) {
  const float depth = pz - 0.0f;
  if (depth <= 0.0f) return 0.0f;
  const float half = 0.5f * depth / fmaxf(f_number, 1e-3f);
  const float u = (ex - px) / fmaxf(half, 1e-9f);
  return window_value(w, u, alpha);
}

// |a - b| with the reference's summation order (types.hpp:52-56).
__device__ __forceinline__ float dist3(float ax, float ay, float az, float bx, float by, float bz) {
  const float x = ax - bx, y = ay - by, z = az - bz;
  return sqrtf(x * x + y * y + z * z);
}

// Element directivity (reference geometry.cpp:111-121).
__device__ __forceinline__ float directivity(float width, float lambda, float sin_theta) {
  const float st = fclamp(sin_theta, -1.0f, 1.0f);
  const float ct = sqrtf(fmaxf(0.0f, 1.0f - st * st));
  const float x = kPi * width * st / lambda;
  const float s = (fabsf(x) < 1e-6f) ? 1.0f - x * x / 6.0f : sinf(x) / x;
  return ct * s;
}

// Per-event transmit description, precomputed on the host with the host's
// libm so the trigonometry matches the reference exactly.
struct TxDev {
  int type;
  int valid;        // the transmit has at least one firing element
  float ox;         // beam origin x
  float sin_a, cos_a, tan_a;
  float fx, fy, fz;
  float x_lo, x_hi; // firing aperture extent (beamformer.cpp:238-247)
  float axis_len, dx, dy, dz;  // focused: unit axis from origin to focus
  float d_origin_focus;        // diverging: |O - focus|
  // For the fast paths' illumination weight: 1 / max(x_hi - x_lo, pitch) and
  // the focused/diverging band's edge slopes (fx - x_lo) / fz, (fx - x_hi) / fz.
  float inv_aperture, slope_lo, slope_hi;
};

// Ideal transmit arrival time at a point (reference geometry.cpp:82-109).
__device__ __forceinline__ float tx_arrival(const TxDev& t, float px, float py, float pz, float c) {
  if (t.type == USX_TX_PLANE_WAVE) {
    return ((px - t.ox) * t.sin_a + (pz - 0.0f) * t.cos_a) / c;
  } else if (t.type == USX_TX_FOCUSED) {
    if (t.axis_len < 1e-9f) return sqrtf(px * px + py * py + pz * pz) / c;
    const float rx = px - t.fx, ry = py - t.fy, rz = pz - t.fz;
    const float proj = rx * t.dx + ry * t.dy + rz * t.dz;
    const float sign = (proj >= 0.0f) ? 1.0f : -1.0f;
    return (t.axis_len + sign * sqrtf(rx * rx + ry * ry + rz * rz)) / c;
  } else {
    return (dist3(px, py, pz, t.fx, t.fy, t.fz) - t.d_origin_focus) / c;
  }
}

// Transmit illumination weight (reference beamformer.cpp:249-288).
__device__ __forceinline__ float tx_sensitivity(const TxDev& t, float px, float pz, float lambda,
                                                float pitch) {
  if (!t.valid || pz <= 0.0f) return 0.0f;
  float a, b;
  if (t.type == USX_TX_PLANE_WAVE) {
    const float shift = pz * t.tan_a;
    a = t.x_lo + shift;
    b = t.x_hi + shift;
  } else {
    const float zf = t.fz;
    if (fabsf(zf) < 1e-9f) return 1.0f;
    a = t.x_lo + (t.fx - t.x_lo) * pz / zf;
    b = t.x_hi + (t.fx - t.x_hi) * pz / zf;
    if (a > b) { const float s = a; a = b; b = s; }
  }
  const float aperture = fmaxf(t.x_hi - t.x_lo, pitch);
  const float f_num_eff = fclamp(pz / aperture, 0.5f, 20.0f);
  const float diffraction = f_num_eff * lambda;
  a -= diffraction;
  b += diffraction;
  const float centre = 0.5f * (a + b);
  const float half = 0.5f * (b - a);
  if (half <= 0.0f) return 0.0f;
  return window_value(USX_WIN_TUKEY, (px - centre) / half, 0.4f);
}

// tx_sensitivity with the per-transmit divisions replaced by products with
// host-computed reciprocals, the per-pixel one by __fdividef and the Tukey
// taper's cosine by __cosf: the weight moves by ~1e-6 relative, the delay
// indices and phases (which do not use it) not at all. The fast
// delay-and-sum kernels (every launch shape) use it; the exact-order kernel
// keeps tx_sensitivity.
__device__ __forceinline__ float tx_sensitivity_fast(const TxDev& t, float px, float pz, float lambda) {
  if (!t.valid || pz <= 0.0f) return 0.0f;
  float a, b;
  if (t.type == USX_TX_PLANE_WAVE) {
    const float shift = pz * t.tan_a;
    a = t.x_lo + shift;
    b = t.x_hi + shift;
  } else {
    if (fabsf(t.fz) < 1e-9f) return 1.0f;
    a = t.x_lo + pz * t.slope_lo;
    b = t.x_hi + pz * t.slope_hi;
    if (a > b) { const float s = a; a = b; b = s; }
  }
  const float f_num_eff = fclamp(pz * t.inv_aperture, 0.5f, 20.0f);
  const float diffraction = f_num_eff * lambda;
  a -= diffraction;
  b += diffraction;
  const float centre = 0.5f * (a + b);
  const float half = 0.5f * (b - a);
  if (half <= 0.0f) return 0.0f;
  const float u = __fdividef(px - centre, half);
  if (u < -1.0f || u > 1.0f) return 0.0f;
  const float tt = 0.5f * (u + 1.0f);   // Tukey, alpha 0.4
  constexpr float kA = 0.4f, kW = 2.0f * kPi / kA;
  if (tt < 0.5f * kA) return 0.5f * (1.0f + __cosf(kW * (tt - 0.5f * kA)));
  if (tt > 1.0f - 0.5f * kA) return 0.5f * (1.0f + __cosf(kW * (tt - 1.0f + 0.5f * kA)));
  return 1.0f;
}

// ChannelData::validate (reference types.cpp:8-124) on the metadata half.
int validate_channel(const usx_channel_desc& cd);

// Host-side construction of TxDev from a usx_transmit (bit-identical to the
// reference's float arithmetic; compiled by the host compiler).
TxDev make_txdev(const usx_probe& probe, const usx_transmit& tx);

inline int ceil_div(long a, long b) { return static_cast<int>((a + b - 1) / b); }

// Tensor-core minimum variance (mv_tc.cu). Optional extras: a device work
// list of (pixel, frame) pairs in place of every pixel of every frame, and a
// training export of the normalised Capon weights L w / sum(w)
// ([frame * n_pix + pix][2 * 64] floats, zero past L) with a per-pixel valid flag.
// Pixels of similar subarray length: the warp-per-pixel kernel sizes its
// shared memory for the class's largest L and active aperture.
struct MvClass {
  const int* pixels = nullptr;   // device list of pixel indices
  int count = 0;
  int lmax = 0, nmax = 0;
};
struct MvTcExtra {
  // 1 = covariance on tcgen05 (class mode; lists as 0), 0 = mma.sync in the
  // solve kernel, 2 = FP32 by the lag recurrence in the solve kernel.
  int cov_engine = 1;
  const int2* list = nullptr;
  const int* list_count = nullptr;
  int list_cap = 0;
  int list_lmax = 0, list_nmax = 0;  // limits of the listed pixels (0: the plan's L and all channels)
  float* w_export = nullptr;
  uint8_t* w_valid = nullptr;
  const MvClass* classes = nullptr;  // full frames by class (else the CTA-per-pixel kernel)
  int n_classes = 0;
  int* overflow_count = nullptr;     // device scratch: pixels past their class's limits
  int2* overflow = nullptr;
  int overflow_cap = 0;
};
int mv_tc_supported(int n_ch, int mv_subarray, int range_avg);
int launch_mv_tc(usx_ctx* ctx, const float2* y, const float* points, float2* out, long out_stride,
                 float* acc_out, int n_ch, int n_pix, int n1, int n_frames, int mv_subarray, int range_avg,
                 float loading, float f_number, float tukey_alpha, int rx_window, float half_nm1, float pitch,
                 int cf, int incoherent, int* stats, int* fallback_count, int2* fallback, int fallback_cap,
                 const MvTcExtra& extra = MvTcExtra());

// Learned minimum variance (learned.cu): per-pixel features of the compounded
// channel samples, and the gated apply of the network's weights.
constexpr int kLmvFeatures = 256;  // network inputs per pixel
// Gated pixels are listed per subarray class c (L in (16 c, 16 (c + 1)]).
constexpr int kLmvGateClasses = 4;
constexpr int kLmvClassWidth = 16;
constexpr int kLmvOutputs = 128;   // network outputs per pixel: 64 complex weights
struct LmvLaunch {
  const float2* y = nullptr;       // [frame][pix][n_ch]
  const float* points = nullptr;
  int n_ch = 0, n_pix = 0, n1 = 0, n_frames = 0, mv_subarray = 0, range_avg = 0;
  float f_number = 0, tukey_alpha = 0, half_nm1 = 0, pitch = 0;
  int rx_window = 0, cf = 0;
  void* feat16 = nullptr;          // BF16 [row][256] (inference)
  float* feat32 = nullptr;         // FP32 [row][256] (training export)
  float2* avg = nullptr;           // [row][64]
  float4* meta = nullptr;          // [row] (L, n_act, coherence factor, 0)
  float2* out = nullptr;           // frames (DAS for n_act < 4)
  long out_stride = 0;
};
int launch_lmv_features(usx_ctx* ctx, const LmvLaunch& l);
int launch_lmv_apply(usx_ctx* ctx, const float* net, const float2* avg, const float4* meta, float2* out,
                     long out_stride, int n_pix, int n_frames, float gate, int* gated_count, int2* gated,
                     int gated_cap, int* stats);
// Learned-subspace refinement: gate on the network's distortionless residual,
// then the exact Capon solve within span{1, network weights, n_beams DFT
// beams} through the pixel's snapshots, gated again on the share of the
// output-power reduction the network's direction carries (learned.cu).
// use_net = 0 leaves the network's direction out (the beams alone).
// level_gate: pixels whose tr(R) exceeds level_gate x the geometric mean of
// tr(R) over the lateral lines at their depth also go to the exact solver
// (+inf: off); `level` holds one float per (frame, depth).
int launch_lmv_subspace(usx_ctx* ctx, const LmvLaunch& l, const float* net, int n_beams, float loading,
                        float gate, int use_net, float share_gate, float level_gate, int level_lines, int level_depths, float* level,
                        int* gated_count, int2* gated, int gated_cap, int* stats, float* rec);
// Bytes per pixel of the scratch record launch_lmv_subspace passes between its two stages.
int lmv_subspace_record_bytes(int n_beams);

// Fifth-generation tensor-core GEMM (gemm_tc5.cu): C = act(A W + b) with A
// [M][K] and W^T [N][K] BF16 (K contiguous), FP32 accumulation in tensor
// memory, BF16 and / or FP32 output [M][N]; N = 128 or 256, K a multiple of
// 64, M a multiple of 128.
bool gemm_tc5_supported(int M, int N, int K);
int launch_gemm_tc5(usx_ctx* ctx, const void* A, const void* Bt, const float* bias, bool relu, void* C16, float* C32,
                    int M, int N, int K);
// wt[N][K] = w[K][N] (BF16).
int transpose_bf16(cudaStream_t st, const void* w, int K, int N, void* wt);

// The network (mlp.cu). mlp_infer runs `rows` (a multiple of 128) BF16 input
// rows through every layer with caller scratch t0, t1 (rows x widest BF16
// each) and writes the FP32 outputs.
int mlp_widest(const usx_mlp* n);
bool mlp_is_lmv(const usx_mlp* n);
int mlp_infer(usx_mlp* n, usx_ctx* ctx, const void* x16, long rows, void* t0, void* t1, float* out32);

}  // namespace usxcu
