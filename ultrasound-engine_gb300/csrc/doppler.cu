// doppler.cu — polynomial-regression wall filter, colour flow (Kasai/Loupas
// autocorrelation with coherence and power gates), power Doppler, two-stage
// axial displacement tracking and least-squares strain (reference
// doppler.cpp:15-305).
//
// Ensembles are [frame][pixel] complex. The (I - P) clutter projector depends
// only on the ensemble length and is built on the host with the reference's
// float Gram-Schmidt (bit-identical), then applied per pixel on the device.
// Every per-pixel sum runs in the reference's loop order (lateral offset,
// axial offset, frame), so the maps match the reference to the last ulp of
// the device's atan2f/hypotf.
#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kMaxEns = 64;

// doppler.cpp:15-47, host float arithmetic.
std::vector<float> reject_matrix(int n, int order) {
  order = std::min(std::max(order, 0), n - 1);
  const int p = order + 1;
  std::vector<std::vector<float>> basis;
  for (int d = 0; d < p; ++d) {
    std::vector<float> v(static_cast<size_t>(n));
    for (int k = 0; k < n; ++k) {
      const float x = (n == 1) ? 0.0f : 2.0f * static_cast<float>(k) / static_cast<float>(n - 1) - 1.0f;
      v[static_cast<size_t>(k)] = static_cast<float>(std::pow(static_cast<double>(x), static_cast<double>(d)));
    }
    for (const auto& b : basis) {
      float dot = 0;
      for (int k = 0; k < n; ++k) dot += v[static_cast<size_t>(k)] * b[static_cast<size_t>(k)];
      for (int k = 0; k < n; ++k) v[static_cast<size_t>(k)] -= dot * b[static_cast<size_t>(k)];
    }
    float norm = 0;
    for (float x : v) norm += x * x;
    norm = std::sqrt(norm);
    if (norm < 1e-8f) continue;
    for (float& x : v) x /= norm;
    basis.push_back(v);
  }
  std::vector<float> M(static_cast<size_t>(n) * n, 0.0f);
  for (int i = 0; i < n; ++i) M[static_cast<size_t>(i) * n + i] = 1.0f;
  for (const auto& b : basis)
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        M[static_cast<size_t>(i) * n + j] -= b[static_cast<size_t>(i)] * b[static_cast<size_t>(j)];
  return M;
}

struct WallArgs {
  const float2* ens;
  float2* out;          // filtered ensemble, or nullptr
  float* power;         // power Doppler sum, or nullptr
  long n_pix;
  int n;
  int identity;         // WallFilter::None: copy through
  float M[kMaxEns * kMaxEns];
};

__global__ void wall_kernel(const WallArgs a) {
  extern __shared__ float2 zs[];   // [n][blockDim]
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= a.n_pix) return;
  for (int j = 0; j < a.n; ++j) zs[j * blockDim.x + threadIdx.x] = a.ens[j * a.n_pix + k];
  float p = 0.0f;
  for (int i = 0; i < a.n; ++i) {
    cplx acc;
    if (a.identity) {
      const float2 z = zs[i * blockDim.x + threadIdx.x];
      acc = mk(z.x, z.y);
    } else {
      acc = mk(0.f, 0.f);
      for (int j = 0; j < a.n; ++j) {
        const float2 z = zs[j * blockDim.x + threadIdx.x];
        acc = cadd(acc, cscale(mk(z.x, z.y), a.M[i * a.n + j]));
      }
    }
    if (a.out) a.out[i * a.n_pix + k] = make_float2(acc.re, acc.im);
    p += cnorm(acc);
  }
  if (a.power) a.power[k] = p;
}

struct FlowArgs {
  const float2* filt;   // [n][n0*n1]
  int n, n0, n1, ka, kl, loupas;
  float dz, fdem, prf, c, coh_thr;
  float* velocity;
  float* power;
  float* variance;
  uint8_t* valid;
  unsigned* pmax_bits;
};

__device__ __forceinline__ void flow_pixel(const FlowArgs& a) {
  const long k0 = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  const long n_pix = static_cast<long>(a.n0) * a.n1;
  // Out-of-range lanes evaluate the last pixel but do not store, so that the
  // whole warp reaches the max reduction below.
  const bool in_range = k0 < n_pix;
  const long k = in_range ? k0 : n_pix - 1;
  const int i = static_cast<int>(k / a.n1), j = static_cast<int>(k - static_cast<long>(i) * a.n1);
  cplx R01 = mk(0.f, 0.f), R10 = mk(0.f, 0.f);
  float R00 = 0.0f;
  for (int di = -a.kl; di <= a.kl; ++di) {
    const int ii = i + di;
    if (ii < 0 || ii >= a.n0) continue;
    for (int dj = -a.ka; dj <= a.ka; ++dj) {
      const int jj = j + dj;
      if (jj < 0 || jj >= a.n1) continue;
      const long kk = static_cast<long>(ii) * a.n1 + jj;
      for (int e = 0; e < a.n; ++e) {
        const float2 zf = a.filt[e * n_pix + kk];
        const cplx z = mk(zf.x, zf.y);
        R00 += cnorm(z);
        if (e + 1 < a.n) {
          const float2 w = a.filt[(e + 1) * n_pix + kk];
          R01 = cadd(R01, cmul(cconj(z), mk(w.x, w.y)));
        }
        if (jj + 1 < a.n1) {
          const float2 w = a.filt[e * n_pix + kk + 1];
          R10 = cadd(R10, cmul(cconj(z), mk(w.x, w.y)));
        }
      }
    }
  }
  float vel = 0.0f, var = 0.0f;
  uint8_t ok = 0;
  if (R00 > 0.0f) {
    const float coherence = cabsf_(R01) / R00;
    var = fclamp(2.0f * (1.0f - coherence), 0.0f, 1.0f);
    if (!(coherence < a.coh_thr)) {
      const float phase_slow = atan2f(R01.im, R01.re);
      float f_centre = a.fdem;
      if (a.loupas) {
        const float phase_fast = atan2f(R10.im, R10.re);
        const float f_est = phase_fast * a.c / (4.0f * kPi * a.dz);
        if (f_est > 0.25f * a.fdem && f_est < 2.0f * a.fdem) f_centre = f_est;
      }
      if (f_centre > 0.0f) {
        vel = -phase_slow * a.c * a.prf / (4.0f * kPi * f_centre);
        ok = 1;
      }
    }
  }
  if (in_range) {
    a.velocity[k] = vel;
    a.power[k] = R00;
    a.variance[k] = var;
    a.valid[k] = ok;
  }
  // Power is non-negative, so its bit pattern orders like its value.
  unsigned m = __float_as_uint(fmaxf(R00, 0.0f));
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(a.pmax_bits, m);
}

__global__ void flow_kernel(const FlowArgs a) { flow_pixel(a); }

__global__ void power_gate_kernel(const float* power, uint8_t* valid, long n, float ratio,
                                  const unsigned* pmax_bits) {
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  const float pmax = __uint_as_float(*pmax_bits);
  if (pmax > 0.0f) {
    const float thr = pmax * ratio;
    if (power[k] < thr) valid[k] = 0;
  }
}

// Batched colour flow (usx_cu_color_flow_batch): all ensembles of one call
// in one wall-filter launch, one flow launch and one gate launch. blockIdx.y
// is the ensemble within a chunk; the per-ensemble lengths and offsets, and
// the clutter projector of every distinct length (they depend only on the
// length), ride in the kernel parameters. Per pixel the arithmetic is that
// of wall_kernel / flow_kernel / power_gate_kernel, so every map equals the
// one-ensemble path bit for bit.
constexpr int kBatchEns = 64;      // ensembles per launch
constexpr int kBatchPool = 6144;   // floats of projectors per launch (24 KB)

struct WallBatchArgs {
  const float2* ens;       // input frames, where the caller packed them
  float2* out;             // filtered frames, packed back to back
  long n_pix;
  int identity;
  int n[kBatchEns];
  int m_off[kBatchEns];    // projector offset in M
  long in_off[kBatchEns];  // first input frame of the ensemble
  long out_off[kBatchEns]; // first filtered frame of the ensemble
  float M[kBatchPool];
};

__global__ void wall_batch_kernel(const WallBatchArgs a) {
  extern __shared__ float2 zs[];   // [n][blockDim]
  const int e = blockIdx.y;
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= a.n_pix) return;
  const int n = a.n[e];
  const float2* src = a.ens + a.in_off[e] * a.n_pix;
  float2* dst = a.out + a.out_off[e] * a.n_pix;
  const float* M = a.M + a.m_off[e];
  for (int j = 0; j < n; ++j) zs[j * blockDim.x + threadIdx.x] = src[j * a.n_pix + k];
  for (int i = 0; i < n; ++i) {
    cplx acc;
    if (a.identity) {
      const float2 z = zs[i * blockDim.x + threadIdx.x];
      acc = mk(z.x, z.y);
    } else {
      acc = mk(0.f, 0.f);
      for (int j = 0; j < n; ++j) {
        const float2 z = zs[j * blockDim.x + threadIdx.x];
        acc = cadd(acc, cscale(mk(z.x, z.y), M[i * n + j]));
      }
    }
    dst[i * a.n_pix + k] = make_float2(acc.re, acc.im);
  }
}

struct FlowBatchArgs {
  FlowArgs base;         // filt = packed filtered frames; maps = [ensemble][pixel]
  int n[kBatchEns];
  int ens[kBatchEns];    // ensemble index of this chunk's entry (map row)
  long f_off[kBatchEns];
};

__global__ void flow_batch_kernel(const FlowBatchArgs b) {
  const int e = blockIdx.y;
  FlowArgs a = b.base;
  const long n_pix = static_cast<long>(a.n0) * a.n1;
  const long row = b.ens[e];
  a.n = b.n[e];
  a.filt = b.base.filt + b.f_off[e] * n_pix;
  a.velocity += row * n_pix;
  a.power += row * n_pix;
  a.variance += row * n_pix;
  a.valid += row * n_pix;
  a.pmax_bits += row;
  flow_pixel(a);
}

__global__ void power_gate_batch_kernel(const float* power, uint8_t* valid, long n, float ratio,
                                        const unsigned* pmax_bits) {
  const long row = blockIdx.y;
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= n) return;
  const float pmax = __uint_as_float(pmax_bits[row]);
  if (pmax > 0.0f) {
    const float thr = pmax * ratio;
    if (power[row * n + k] < thr) valid[row * n + k] = 0;
  }
}

struct DispArgs {
  const float2* a;
  const float2* b;
  int n0, n1, ka, kl, lag_max;
  float dz, fdem, c;
  float* axial;
  float* corr;
};

__global__ void displacement_kernel(const DispArgs p) {
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= static_cast<long>(p.n0) * p.n1) return;
  const int i = static_cast<int>(k / p.n1), j = static_cast<int>(k - static_cast<long>(i) * p.n1);
  p.axial[k] = 0.0f;
  p.corr[k] = 0.0f;
  cplx R10 = mk(0.f, 0.f);
  for (int di = -p.kl; di <= p.kl; ++di) {
    const int ii = i + di;
    if (ii < 0 || ii >= p.n0) continue;
    for (int dj = -p.ka; dj <= p.ka; ++dj) {
      const int jj = j + dj;
      if (jj < 0 || jj + 1 >= p.n1) continue;
      const long kk = static_cast<long>(ii) * p.n1 + jj;
      const float2 u = p.a[kk], v = p.a[kk + 1];
      R10 = cadd(R10, cmul(cconj(mk(u.x, u.y)), mk(v.x, v.y)));
    }
  }
  float f_centre = p.fdem;
  const float f_est = atan2f(R10.im, R10.re) * p.c / (4.0f * kPi * p.dz);
  if (f_est > 0.25f * p.fdem && f_est < 2.0f * p.fdem) f_centre = f_est;
  if (f_centre <= 0.0f) return;
  cplx best_R = mk(0.f, 0.f);
  float best_corr = -1.0f;
  int best_lag = 0;
  for (int lag = -p.lag_max; lag <= p.lag_max; ++lag) {
    cplx R = mk(0.f, 0.f);
    float ea = 0.0f, eb = 0.0f;
    for (int di = -p.kl; di <= p.kl; ++di) {
      const int ii = i + di;
      if (ii < 0 || ii >= p.n0) continue;
      for (int dj = -p.ka; dj <= p.ka; ++dj) {
        const int jj = j + dj;
        const int jl = jj + lag;
        if (jj < 0 || jj >= p.n1 || jl < 0 || jl >= p.n1) continue;
        const float2 u = p.a[static_cast<long>(ii) * p.n1 + jj];
        const float2 v = p.b[static_cast<long>(ii) * p.n1 + jl];
        const cplx A = mk(u.x, u.y), B = mk(v.x, v.y);
        R = cadd(R, cmul(cconj(A), B));
        ea += cnorm(A);
        eb += cnorm(B);
      }
    }
    if (ea <= 0.0f || eb <= 0.0f) continue;
    const float cr = cabsf_(R) / sqrtf(ea * eb);
    if (cr > best_corr) {
      best_corr = cr;
      best_R = R;
      best_lag = lag;
    }
  }
  if (best_corr < 0.0f) return;
  p.corr[k] = fclamp(best_corr, 0.0f, 1.0f);
  const float residual = -atan2f(best_R.im, best_R.re) * p.c / (4.0f * kPi * f_centre);
  p.axial[k] = static_cast<float>(best_lag) * p.dz + residual;
}

__global__ void strain_kernel(const float* axial, int n0, int n1, float dz, int half, float* strain) {
  const long k = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (k >= static_cast<long>(n0) * n1) return;
  const int i = static_cast<int>(k / n1), j = static_cast<int>(k - static_cast<long>(i) * n1);
  float sx = 0, sy = 0, sxx = 0, sxy = 0;
  int n = 0;
  for (int d = -half; d <= half; ++d) {
    const int jj = j + d;
    if (jj < 0 || jj >= n1) continue;
    const float x = static_cast<float>(d) * dz;
    const float y = axial[static_cast<long>(i) * n1 + jj];
    sx += x;
    sy += y;
    sxx += x * x;
    sxy += x * y;
    ++n;
  }
  float out = 0.0f;
  if (n >= 2) {
    const float denom = static_cast<float>(n) * sxx - sx * sx;
    if (!(fabsf(denom) < 1e-20f)) out = (static_cast<float>(n) * sxy - sx * sy) / denom;
  }
  strain[k] = out;
}

float axial_step(const float* axis1, int n1) {
  float dz = 1e-4f;
  if (n1 > 1 && axis1) dz = std::abs(axis1[1] - axis1[0]);
  return dz;
}

int launch_wall(usx_ctx* ctx, const float* ens, int n, long n_pix, int type, int order, float* out,
                float* power) {
  if (n > kMaxEns) return fail(USX_ERR_UNSUPPORTED, "ensembles longer than 64 frames are not supported");
  WallArgs a;
  a.ens = reinterpret_cast<const float2*>(ens);
  a.out = reinterpret_cast<float2*>(out);
  a.power = power;
  a.n_pix = n_pix;
  a.n = n;
  a.identity = type == USX_WALL_NONE;
  if (!a.identity) {
    const std::vector<float> M = reject_matrix(n, type == USX_WALL_MEAN ? 0 : order);
    std::copy(M.begin(), M.end(), a.M);
  }
  const int threads = 128;
  const size_t smem = sizeof(float2) * n * threads;
  if (smem > 48 * 1024)
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(wall_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  prof_begin(ctx, "wall_kernel");
  wall_kernel<<<ceil_div(n_pix, threads), threads, smem, ctx->stream>>>(a);
  prof_end(ctx);
  USX_CHECK_LAUNCH("wall_kernel");
  return USX_OK;
}

int launch_flow(usx_ctx* ctx, const float* filt, int n, int n0, int n1, float dz, float fdem,
                float prf, float c, const usx_doppler_config& cfg, float* velocity, float* power,
                float* variance, uint8_t* valid, unsigned* pmax_bits) {
  FlowArgs a;
  a.filt = reinterpret_cast<const float2*>(filt);
  a.n = n;
  a.n0 = n0;
  a.n1 = n1;
  a.ka = std::max(0, cfg.kernel_axial);
  a.kl = std::max(0, cfg.kernel_lateral);
  a.loupas = cfg.loupas;
  a.dz = dz;
  a.fdem = fdem;
  a.prf = prf;
  a.c = c;
  a.coh_thr = cfg.coherence_threshold;
  a.velocity = velocity;
  a.power = power;
  a.variance = variance;
  a.valid = valid;
  a.pmax_bits = pmax_bits;
  const long n_pix = static_cast<long>(n0) * n1;
  USX_CUDA(cudaMemsetAsync(pmax_bits, 0, sizeof(unsigned), ctx->stream));
  prof_begin(ctx, "flow_kernel");
  flow_kernel<<<ceil_div(n_pix, 128), 128, 0, ctx->stream>>>(a);
  prof_end(ctx);
  USX_CHECK_LAUNCH("flow_kernel");
  const float ratio = std::pow(10.0f, cfg.power_threshold_db / 10.0f);
  prof_begin(ctx, "power_gate_kernel");
  power_gate_kernel<<<ceil_div(n_pix, 256), 256, 0, ctx->stream>>>(power, valid, n_pix, ratio, pmax_bits);
  prof_end(ctx);
  USX_CHECK_LAUNCH("power_gate_kernel");
  return USX_OK;
}

}  // namespace

// ------------------------------------------------------------------------
// Colour flow without allocation (usx_cu_color_flow_noalloc).
//
// For callers that must not allocate device memory once they are running: a
// scanner's real-time loop with a fixed memory budget, or code that hands this
// library a stream but owns the device's allocator. Its working
// memory, the wall-filtered ensemble and the frame's maximum power, is this
// fixed array, reserved on every device that loads the library for as long
// as the process lives: kNoAllocSamples complex samples (8 MiB) plus one
// word. Host code must not pass the array's name to a kernel: on the host it
// only stands in for the symbol, so its device address is looked up once per
// device with cudaGetSymbolAddress.
namespace {

constexpr long kNoAllocSamples = 1L << 20;
static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocSamples + 32];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
float2* g_noalloc_addr[kNoAllocMaxDevices] = {};

// Device address of the scratch on the current device, looked up on the
// first call for that device.
int noalloc_scratch(float2** out) {
  int dev = 0;
  USX_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kNoAllocMaxDevices)
    return fail(USX_ERR_UNSUPPORTED, "usx_cu_color_flow_noalloc: device index above 63");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_addr[dev] = static_cast<float2*>(p);
  }
  *out = g_noalloc_addr[dev];
  return USX_OK;
}

}  // namespace
}  // namespace usxcu

using namespace usxcu;

extern "C" {

int usx_cu_wall_filter(usx_ctx* ctx, const float* ens, int n_frames, int64_t n_pix, int type,
                       int order, float* out) {
  if (!ctx || !ens || !out) return fail(USX_ERR_INVALID, "usx_cu_wall_filter: null argument");
  if (n_frames <= 0 || n_pix <= 0) return USX_OK;
  return launch_wall(ctx, ens, n_frames, n_pix, type, order, out, nullptr);
}

int usx_cu_power_doppler(usx_ctx* ctx, const float* ens, int n_frames, int64_t n_pix, int type,
                         int order, float* power) {
  if (!ctx || !ens || !power) return fail(USX_ERR_INVALID, "usx_cu_power_doppler: null argument");
  if (n_frames <= 0 || n_pix <= 0) return USX_OK;
  return launch_wall(ctx, ens, n_frames, n_pix, type, order, nullptr, power);
}

int usx_cu_color_flow(usx_ctx* ctx, const float* ens, int n_frames, int n0, int n1,
                      const float* axis1_host, float fdem, float prf, float speed_of_sound,
                      const usx_doppler_config* cfg, float* velocity, float* power,
                      float* variance, uint8_t* valid, float* nyquist) {
  if (!ctx || !ens || !cfg || !velocity || !power || !variance || !valid)
    return fail(USX_ERR_INVALID, "usx_cu_color_flow: null argument");
  if (n_frames < 2) return fail(USX_ERR_INVALID, "color_flow: need at least 2 frames in the ensemble");
  if (n0 <= 0 || n1 <= 0) return fail(USX_ERR_INVALID, "color_flow: empty grid");
  const long n_pix = static_cast<long>(n0) * n1;
  void* ws = nullptr;
  if (int rc = scratch(ctx, sizeof(float2) * n_pix * n_frames, &ws)) return rc;
  float* filt = static_cast<float*>(ws);
  if (int rc = launch_wall(ctx, ens, n_frames, n_pix, cfg->wall_filter, cfg->polynomial_order, filt, nullptr))
    return rc;
  if (nyquist) *nyquist = (fdem > 0.0f) ? speed_of_sound * prf / (4.0f * fdem) : 0.0f;
  return launch_flow(ctx, filt, n_frames, n0, n1, axial_step(axis1_host, n1), fdem, prf,
                     speed_of_sound, *cfg, velocity, power, variance, valid,
                     reinterpret_cast<unsigned*>(ctx->d_status + 10));
}

int usx_cu_color_flow_batch(usx_ctx* ctx, const float* ens, int n_ens, const int* n_frames_host,
                            const int64_t* frame_offset_host, int n0, int n1,
                            const float* axis1_host, float fdem, float prf,
                            float speed_of_sound, const usx_doppler_config* cfg, float* velocity,
                            float* power, float* variance, uint8_t* valid) {
  if (!ctx || !ens || !n_frames_host || !frame_offset_host || !cfg)
    return fail(USX_ERR_INVALID, "usx_cu_color_flow_batch: null argument");
  if (n_ens <= 0) return USX_OK;
  if (n_ens > 65535) return fail(USX_ERR_UNSUPPORTED, "usx_cu_color_flow_batch: more than 65535 ensembles");
  if (!velocity || !power || !variance || !valid)
    return fail(USX_ERR_INVALID, "usx_cu_color_flow_batch: null argument");
  if (n0 <= 0 || n1 <= 0) return fail(USX_ERR_INVALID, "color_flow: empty grid");
  const long n_pix = static_cast<long>(n0) * n1;
  int max_frames = 0;
  long total_frames = 0;
  for (int e = 0; e < n_ens; ++e) {
    if (n_frames_host[e] < 2) return fail(USX_ERR_INVALID, "color_flow: need at least 2 frames in the ensemble");
    if (frame_offset_host[e] < 0) return fail(USX_ERR_INVALID, "usx_cu_color_flow_batch: negative frame offset");
    max_frames = std::max(max_frames, n_frames_host[e]);
    total_frames += n_frames_host[e];
  }
  if (max_frames > kMaxEns) return fail(USX_ERR_UNSUPPORTED, "ensembles longer than 64 frames are not supported");
  // Filtered ensembles packed back to back, then one power maximum per ensemble.
  const size_t filt_bytes = sizeof(float2) * static_cast<size_t>(n_pix) * static_cast<size_t>(total_frames);
  void* ws = nullptr;
  if (int rc = scratch(ctx, filt_bytes + sizeof(unsigned) * n_ens + 256, &ws)) return rc;
  float2* filt = static_cast<float2*>(ws);
  unsigned* pmax = reinterpret_cast<unsigned*>(static_cast<char*>(ws) + filt_bytes);
  USX_CUDA(cudaMemsetAsync(pmax, 0, sizeof(unsigned) * n_ens, ctx->stream));

  const int type = cfg->wall_filter;
  const int order = type == USX_WALL_MEAN ? 0 : cfg->polynomial_order;
  const int threads = 128;
  FlowBatchArgs fb;
  FlowArgs& f = fb.base;
  f.filt = filt;
  f.n0 = n0;
  f.n1 = n1;
  f.ka = std::max(0, cfg->kernel_axial);
  f.kl = std::max(0, cfg->kernel_lateral);
  f.loupas = cfg->loupas;
  f.dz = axial_step(axis1_host, n1);
  f.fdem = fdem;
  f.prf = prf;
  f.c = speed_of_sound;
  f.coh_thr = cfg->coherence_threshold;
  f.velocity = velocity;
  f.power = power;
  f.variance = variance;
  f.valid = valid;
  f.pmax_bits = pmax;

  // Chunks of at most kBatchEns ensembles whose distinct projectors fit the pool.
  long packed = 0;  // first filtered frame of the next ensemble
  int e0 = 0;
  while (e0 < n_ens) {
    WallBatchArgs w;
    w.ens = reinterpret_cast<const float2*>(ens);
    w.out = filt;
    w.n_pix = n_pix;
    w.identity = type == USX_WALL_NONE;
    int pool = 0, count = 0, chunk_max = 0, n_have = 0;
    int have_n[kBatchEns], have_off[kBatchEns];
    for (int e = e0; e < n_ens && count < kBatchEns; ++e) {
      const int n = n_frames_host[e];
      int off = 0;
      if (!w.identity) {
        off = -1;
        for (int q = 0; q < n_have; ++q)
          if (have_n[q] == n) off = have_off[q];
        if (off < 0) {
          if (pool + n * n > kBatchPool) break;  // 64 x 64 alone always fits
          const std::vector<float> M = reject_matrix(n, order);
          std::copy(M.begin(), M.end(), w.M + pool);
          off = pool;
          have_n[n_have] = n;
          have_off[n_have++] = pool;
          pool += n * n;
        }
      }
      w.n[count] = n;
      w.m_off[count] = off;
      w.in_off[count] = frame_offset_host[e];
      w.out_off[count] = packed;
      fb.n[count] = n;
      fb.ens[count] = e;
      fb.f_off[count] = packed;
      packed += n;
      chunk_max = std::max(chunk_max, n);
      ++count;
    }
    const size_t smem = sizeof(float2) * static_cast<size_t>(chunk_max) * threads;
    if (smem > 48 * 1024)
      if (int rc_ = smem_limit(reinterpret_cast<const void*>(wall_batch_kernel), smem)) return rc_;
    prof_begin(ctx, "wall_batch_kernel");
    wall_batch_kernel<<<dim3(ceil_div(n_pix, threads), count), threads, smem, ctx->stream>>>(w);
    prof_end(ctx);
    USX_CHECK_LAUNCH("wall_batch_kernel");
    prof_begin(ctx, "flow_batch_kernel");
    flow_batch_kernel<<<dim3(ceil_div(n_pix, 128), count), 128, 0, ctx->stream>>>(fb);
    prof_end(ctx);
    USX_CHECK_LAUNCH("flow_batch_kernel");
    e0 += count;
  }
  const float ratio = std::pow(10.0f, cfg->power_threshold_db / 10.0f);
  prof_begin(ctx, "power_gate_batch_kernel");
  power_gate_batch_kernel<<<dim3(ceil_div(n_pix, 256), n_ens), 256, 0, ctx->stream>>>(power, valid, n_pix, ratio,
                                                                                       pmax);
  prof_end(ctx);
  USX_CHECK_LAUNCH("power_gate_batch_kernel");
  return USX_OK;
}

int usx_cu_color_flow_noalloc(void* stream, const float* ens, int n_frames, int n0, int n1,
                              const float* axis1_host, float fdem, float prf, float speed_of_sound,
                              const usx_doppler_config* cfg, float* velocity, float* power,
                              float* variance, uint8_t* valid, float* nyquist) {
  if (!ens || !cfg || !velocity || !power || !variance || !valid)
    return fail(USX_ERR_INVALID, "usx_cu_color_flow_noalloc: null argument");
  if (n_frames < 2) return fail(USX_ERR_INVALID, "color_flow: need at least 2 frames in the ensemble");
  if (n0 <= 0 || n1 <= 0) return fail(USX_ERR_INVALID, "color_flow: empty grid");
  if (n_frames > kMaxEns) return fail(USX_ERR_UNSUPPORTED, "ensembles longer than 64 frames are not supported");
  const long n_pix = static_cast<long>(n0) * n1;
  if (n_pix * n_frames > kNoAllocSamples)
    return fail(USX_ERR_INVALID,
                "usx_cu_color_flow_noalloc: n_frames * n0 * n1 exceeds the 1048576 complex samples of its "
                "static scratch; use usx_cu_color_flow");
  float2* scratch = nullptr;
  if (int rc = noalloc_scratch(&scratch)) return rc;
  float2* filt = scratch;
  unsigned* pmax_bits = reinterpret_cast<unsigned*>(scratch + kNoAllocSamples);
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  WallArgs w;
  w.ens = reinterpret_cast<const float2*>(ens);
  w.out = filt;
  w.power = nullptr;
  w.n_pix = n_pix;
  w.n = n_frames;
  w.identity = cfg->wall_filter == USX_WALL_NONE;
  if (!w.identity) {
    const std::vector<float> M = reject_matrix(n_frames, cfg->wall_filter == USX_WALL_MEAN ? 0 : cfg->polynomial_order);
    std::copy(M.begin(), M.end(), w.M);
  }
  const int threads = 128;
  const size_t smem = sizeof(float2) * n_frames * threads;
  if (smem > 48 * 1024)
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(wall_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  wall_kernel<<<ceil_div(n_pix, threads), threads, smem, st>>>(w);
  USX_CHECK_LAUNCH("wall_kernel");

  FlowArgs f;
  f.filt = filt;
  f.n = n_frames;
  f.n0 = n0;
  f.n1 = n1;
  f.ka = std::max(0, cfg->kernel_axial);
  f.kl = std::max(0, cfg->kernel_lateral);
  f.loupas = cfg->loupas;
  f.dz = axial_step(axis1_host, n1);
  f.fdem = fdem;
  f.prf = prf;
  f.c = speed_of_sound;
  f.coh_thr = cfg->coherence_threshold;
  f.velocity = velocity;
  f.power = power;
  f.variance = variance;
  f.valid = valid;
  f.pmax_bits = pmax_bits;
  // The scratch keeps the previous call's contents: the running maximum must start at zero.
  USX_CUDA(cudaMemsetAsync(pmax_bits, 0, sizeof(unsigned), st));
  flow_kernel<<<ceil_div(n_pix, 128), 128, 0, st>>>(f);
  USX_CHECK_LAUNCH("flow_kernel");
  const float ratio = std::pow(10.0f, cfg->power_threshold_db / 10.0f);
  power_gate_kernel<<<ceil_div(n_pix, 256), 256, 0, st>>>(power, valid, n_pix, ratio, pmax_bits);
  USX_CHECK_LAUNCH("power_gate_kernel");
  if (nyquist) *nyquist = (fdem > 0.0f) ? speed_of_sound * prf / (4.0f * fdem) : 0.0f;
  return USX_OK;
}

int usx_cu_axial_displacement(usx_ctx* ctx, const float* before, const float* after, int n0,
                              int n1, const float* axis1_host, float fdem, float speed_of_sound,
                              int kernel_axial, int kernel_lateral, int max_lag, float* axial,
                              float* correlation) {
  if (!ctx || !before || !after || !axial || !correlation)
    return fail(USX_ERR_INVALID, "usx_cu_axial_displacement: null argument");
  const long n = static_cast<long>(n0) * n1;
  if (n <= 0) return USX_OK;
  DispArgs p;
  p.a = reinterpret_cast<const float2*>(before);
  p.b = reinterpret_cast<const float2*>(after);
  p.n0 = n0;
  p.n1 = n1;
  p.ka = std::max(1, kernel_axial);
  p.kl = std::max(0, kernel_lateral);
  p.lag_max = std::max(0, max_lag);
  p.dz = axial_step(axis1_host, n1);
  p.fdem = fdem;
  p.c = speed_of_sound;
  p.axial = axial;
  p.corr = correlation;
  prof_begin(ctx, "displacement_kernel");
  displacement_kernel<<<ceil_div(n, 128), 128, 0, ctx->stream>>>(p);
  prof_end(ctx);
  USX_CHECK_LAUNCH("displacement_kernel");
  return USX_OK;
}

int usx_cu_axial_strain(usx_ctx* ctx, const float* axial, int n0, int n1,
                        const float* axis1_host, int fit_length, float* strain) {
  if (!ctx || !axial || !strain) return fail(USX_ERR_INVALID, "usx_cu_axial_strain: null argument");
  const long n = static_cast<long>(n0) * n1;
  if (n <= 0) return USX_OK;
  prof_begin(ctx, "strain_kernel");
  strain_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(axial, n0, n1, axial_step(axis1_host, n1),
                                                           std::max(1, fit_length / 2), strain);
  prof_end(ctx);
  USX_CHECK_LAUNCH("strain_kernel");
  return USX_OK;
}

}  // extern "C"
