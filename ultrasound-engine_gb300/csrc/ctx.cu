// ctx.cu — context, memory and error plumbing of the C-ABI, plus the host-side
// helpers (transmit tables, pulse, low-pass design) whose float arithmetic must
// match the reference exactly and therefore runs on the host's libm.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <map>
#include <mutex>
#include <tuple>

#include "usx_internal.cuh"

namespace usxcu {

namespace {
thread_local std::string g_last_error;
}

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* where) {
  g_last_error = std::string(where) + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? USX_ERR_NOMEM : USX_ERR_CUDA;
}

int scratch(usx_ctx* ctx, size_t bytes, void** out) {
  if (bytes == 0) bytes = 256;
  if (bytes > ctx->scratch_bytes) {
    if (ctx->scratch) {
      USX_CUDA(cudaStreamSynchronize(ctx->stream));
      USX_CUDA(cudaFree(ctx->scratch));
      ctx->scratch = nullptr;
      ctx->scratch_bytes = 0;
    }
    const size_t grow = bytes + bytes / 4;
    USX_CUDA(cudaMalloc(&ctx->scratch, grow));
    ctx->scratch_bytes = grow;
  }
  *out = ctx->scratch;
  return USX_OK;
}

// Element x position (reference types.hpp:77-80).
static float elem_x(const usx_probe& p, int i) {
  return (static_cast<float>(i) - 0.5f * static_cast<float>(p.n_elements - 1)) * p.pitch;
}

TxDev make_txdev(const usx_probe& probe, const usx_transmit& tx) {
  TxDev t;
  std::memset(&t, 0, sizeof(t));
  t.type = tx.type;
  t.ox = tx.origin[0];
  t.sin_a = std::sin(tx.angle);
  t.cos_a = std::cos(tx.angle);
  t.tan_a = std::tan(tx.angle);
  t.fx = tx.focus[0];
  t.fy = tx.focus[1];
  t.fz = tx.focus[2];
  // Firing aperture extent (beamformer.cpp:238-247).
  t.valid = 0;
  for (int i = 0; i < probe.n_elements; ++i) {
    if (tx.apodization && tx.apodization[i] == 0.0f) continue;
    const float x = elem_x(probe, i);
    if (!t.valid) {
      t.x_lo = t.x_hi = x;
      t.valid = 1;
    } else {
      t.x_lo = std::min(t.x_lo, x);
      t.x_hi = std::max(t.x_hi, x);
    }
  }
  // Focused: unit axis from the beam origin to the focus (geometry.cpp:95-101).
  const float ax = t.fx - t.ox, ay = t.fy - 0.0f, az = t.fz - 0.0f;
  t.axis_len = std::sqrt(ax * ax + ay * ay + az * az);
  if (t.axis_len >= 1e-9f) {
    t.dx = ax / t.axis_len;
    t.dy = ay / t.axis_len;
    t.dz = az / t.axis_len;
  }
  // Diverging: |O - focus| (geometry.cpp:104-106).
  const float ox = t.ox - t.fx, oy = 0.0f - t.fy, oz = 0.0f - t.fz;
  t.d_origin_focus = std::sqrt(ox * ox + oy * oy + oz * oz);
  // Reciprocal and slopes for tx_sensitivity_fast.
  t.inv_aperture = 1.0f / std::max(t.x_hi - t.x_lo, probe.pitch);
  if (std::fabs(t.fz) >= 1e-9f) {
    t.slope_lo = (t.fx - t.x_lo) / t.fz;
    t.slope_hi = (t.fx - t.x_hi) / t.fz;
  }
  return t;
}

static cudaEvent_t take_event(usx_ctx* ctx) {
  if (!ctx->event_pool.empty()) {
    cudaEvent_t e = ctx->event_pool.back();
    ctx->event_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

void prof_begin(usx_ctx* ctx, const char* name) {
  if (!ctx->profiling) return;
  usx_prof_rec r{name, take_event(ctx), take_event(ctx)};
  cudaEventRecord(r.start, ctx->stream);
  ctx->prof.push_back(r);
}

void prof_end(usx_ctx* ctx) {
  if (!ctx->profiling || ctx->prof.empty()) return;
  cudaEventRecord(ctx->prof.back().stop, ctx->stream);
}

namespace {
std::mutex g_launch_mu;
std::map<std::pair<int, const void*>, size_t> g_smem_set;
std::map<std::tuple<int, const void*, int, size_t>, int> g_occupancy;
}  // namespace

int smem_limit(const void* func, size_t bytes) {
  int dev = 0;
  USX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_launch_mu);
  size_t& have = g_smem_set[{dev, func}];
  if (bytes <= have) return USX_OK;
  USX_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
  have = bytes;
  return USX_OK;
}

int occupancy(const void* func, int threads, size_t smem, int* blocks_per_sm) {
  int dev = 0;
  USX_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_launch_mu);
  const auto key = std::make_tuple(dev, func, threads, smem);
  auto it = g_occupancy.find(key);
  if (it == g_occupancy.end()) {
    int n = 0;
    USX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, func, threads, smem));
    it = g_occupancy.emplace(key, n).first;
  }
  *blocks_per_sm = it->second;
  return USX_OK;
}

int validate_channel(const usx_channel_desc& cd) {
  const usx_probe& p = cd.probe;
  if (p.n_elements <= 0) return fail(USX_ERR_INVALID, "Probe.n_elements must be > 0");
  if (p.pitch <= 0) return fail(USX_ERR_INVALID, "Probe.pitch must be > 0");
  if (p.element_width <= 0) return fail(USX_ERR_INVALID, "Probe.element_width must be > 0");
  if (p.element_width > p.pitch * 1.001f)
    return fail(USX_ERR_INVALID, "Probe.element_width exceeds pitch (elements would overlap)");
  if (p.center_frequency <= 0) return fail(USX_ERR_INVALID, "Probe.center_frequency must be > 0");
  if (p.bandwidth <= 0) return fail(USX_ERR_INVALID, "Probe.bandwidth must be > 0");
  if (cd.medium.speed_of_sound <= 0) return fail(USX_ERR_INVALID, "Medium.speed_of_sound must be > 0");
  if (cd.medium.attenuation < 0) return fail(USX_ERR_INVALID, "Medium.attenuation must be >= 0");
  if (cd.acq.sampling_frequency <= 0)
    return fail(USX_ERR_INVALID, "Acquisition.sampling_frequency must be > 0");
  if (cd.acq.n_samples <= 0) return fail(USX_ERR_INVALID, "Acquisition.n_samples must be > 0");
  if (cd.acq.prf <= 0) return fail(USX_ERR_INVALID, "Acquisition.prf must be > 0");
  if (cd.n_events <= 0 || !cd.transmits) return fail(USX_ERR_INVALID, "ChannelData has no transmit events");
  if (cd.is_iq && cd.demodulation_frequency <= 0)
    return fail(USX_ERR_INVALID, "IQ ChannelData needs a positive demodulation_frequency");
  return USX_OK;
}

// Never launched: its attributes tell which device code the library carries.
__global__ void binary_version_kernel() {}

}  // namespace usxcu

using namespace usxcu;

extern "C" {

int usx_cu_abi_version(void) { return USX_CU_ABI_VERSION; }

int usx_cu_binary_version(int* version) {
  if (!version) return fail(USX_ERR_INVALID, "usx_cu_binary_version: version is NULL");
  cudaFuncAttributes a{};
  USX_CUDA(cudaFuncGetAttributes(&a, binary_version_kernel));
  *version = a.binaryVersion;
  return USX_OK;
}

const char* usx_cu_last_error(void) { return g_last_error.c_str(); }

int usx_cu_ctx_create(int device, void* stream, usx_ctx** out) {
  if (!out) return fail(USX_ERR_INVALID, "usx_cu_ctx_create: out is NULL");
  int n = 0;
  USX_CUDA(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return fail(USX_ERR_INVALID, "usx_cu_ctx_create: no such device");
  USX_CUDA(cudaSetDevice(device));
  usx_ctx* c = new usx_ctx();
  c->device = device;
  if (stream) {
    c->stream = static_cast<cudaStream_t>(stream);
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete c;
      return cuda_fail(e, "cudaStreamCreate");
    }
    c->own_stream = true;
  }
  cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  cudaError_t e = cudaMalloc(&c->d_status, sizeof(int) * 16);
  if (e != cudaSuccess) {
    if (c->own_stream) cudaStreamDestroy(c->stream);
    delete c;
    return cuda_fail(e, "cudaMalloc(status)");
  }
  cudaMemset(c->d_status, 0, sizeof(int) * 16);
  *out = c;
  return USX_OK;
}

int usx_cu_ctx_destroy(usx_ctx* ctx) {
  if (!ctx) return USX_OK;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (auto& r : ctx->prof) {
    cudaEventDestroy(r.start);
    cudaEventDestroy(r.stop);
  }
  for (auto e : ctx->event_pool) cudaEventDestroy(e);
  if (ctx->scratch) cudaFree(ctx->scratch);
  if (ctx->mv_cov) cudaFree(ctx->mv_cov);
  if (ctx->d_status) cudaFree(ctx->d_status);
  if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
  return USX_OK;
}

void* usx_cu_ctx_stream(usx_ctx* ctx) { return ctx ? static_cast<void*>(ctx->stream) : nullptr; }

int usx_cu_ctx_set_stream(usx_ctx* ctx, void* stream) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (!stream) return fail(USX_ERR_INVALID, "usx_cu_ctx_set_stream: stream is NULL");
  if (ctx->own_stream) {
    USX_CUDA(cudaStreamSynchronize(ctx->stream));
    USX_CUDA(cudaStreamDestroy(ctx->stream));
    ctx->own_stream = false;
  }
  ctx->stream = static_cast<cudaStream_t>(stream);
  return USX_OK;
}

int usx_cu_synchronize(usx_ctx* ctx) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  return USX_OK;
}

int usx_cu_malloc(usx_ctx* ctx, size_t bytes, void** dev) {
  if (!ctx || !dev) return fail(USX_ERR_INVALID, "usx_cu_malloc: null argument");
  USX_CUDA(cudaSetDevice(ctx->device));
  USX_CUDA(cudaMalloc(dev, bytes ? bytes : 1));
  return USX_OK;
}

int usx_cu_free(usx_ctx* ctx, void* dev) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (dev) USX_CUDA(cudaFree(dev));
  return USX_OK;
}

int usx_cu_host_alloc(usx_ctx* ctx, size_t bytes, void** host) {
  if (!ctx || !host) return fail(USX_ERR_INVALID, "usx_cu_host_alloc: null argument");
  USX_CUDA(cudaMallocHost(host, bytes ? bytes : 1));
  return USX_OK;
}

int usx_cu_host_free(usx_ctx* ctx, void* host) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (host) USX_CUDA(cudaFreeHost(host));
  return USX_OK;
}

int usx_cu_memcpy_h2d(usx_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (bytes == 0) return USX_OK;
  USX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, ctx->stream));
  return USX_OK;
}

int usx_cu_memcpy_d2h(usx_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (bytes == 0) return USX_OK;
  USX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  return USX_OK;
}

int usx_cu_memcpy_d2d(usx_ctx* ctx, void* dst, const void* src, size_t bytes) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (bytes == 0) return USX_OK;
  USX_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, ctx->stream));
  return USX_OK;
}

int usx_cu_memset(usx_ctx* ctx, void* dst, int value, size_t bytes) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  if (bytes == 0) return USX_OK;
  USX_CUDA(cudaMemsetAsync(dst, value, bytes, ctx->stream));
  return USX_OK;
}

int usx_cu_profile_enable(usx_ctx* ctx, int on) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  ctx->profiling = on != 0;
  return USX_OK;
}

int usx_cu_profile_reset(usx_ctx* ctx) {
  if (!ctx) return fail(USX_ERR_INVALID, "null context");
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  for (auto& r : ctx->prof) {
    ctx->event_pool.push_back(r.start);
    ctx->event_pool.push_back(r.stop);
  }
  ctx->prof.clear();
  return USX_OK;
}

int usx_cu_profile_read(usx_ctx* ctx, int index, char* name, int name_cap, double* total_ms,
                        int64_t* launches) {
  if (!ctx || !name || name_cap <= 0 || !total_ms || !launches)
    return fail(USX_ERR_INVALID, "usx_cu_profile_read: null argument");
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  std::vector<std::string> names;
  for (auto& r : ctx->prof) {
    bool seen = false;
    for (auto& n : names) seen = seen || n == r.name;
    if (!seen) names.push_back(r.name);
  }
  if (index < 0 || index >= static_cast<int>(names.size()))
    return fail(USX_ERR_INVALID, "usx_cu_profile_read: no such kernel index");
  double ms = 0.0;
  int64_t n = 0;
  for (auto& r : ctx->prof) {
    if (names[static_cast<size_t>(index)] != r.name) continue;
    float t = 0.0f;
    USX_CUDA(cudaEventElapsedTime(&t, r.start, r.stop));
    ms += t;
    ++n;
  }
  std::snprintf(name, static_cast<size_t>(name_cap), "%s", names[static_cast<size_t>(index)].c_str());
  *total_ms = ms;
  *launches = n;
  return USX_OK;
}

// Simulator::pulse (reference simulator.cpp:140-154), host arithmetic.
int usx_cu_pulse(const usx_probe* probe, const usx_acquisition* acq,
                 const usx_simulator_config* cfg, float* out, int cap, int* n_taps,
                 float* half_duration) {
  if (!probe || !acq || !cfg) return fail(USX_ERR_INVALID, "usx_cu_pulse: null argument");
  const float f0 = probe->center_frequency;
  const float ln2 = 0.69314718f;
  const float sigma = std::sqrt(2.0f * ln2) / (kPi * probe->bandwidth * f0);
  const float half = 3.0f * sigma;
  const int os = cfg->oversampling < 1 ? 1 : cfg->oversampling;
  const float fs_os = acq->sampling_frequency * static_cast<float>(os);
  const int n_half = static_cast<int>(std::ceil(half * fs_os));
  const int n = 2 * n_half + 1;
  if (n_taps) *n_taps = n;
  if (half_duration) *half_duration = static_cast<float>(n_half) / fs_os;
  if (out) {
    if (cap < n) return fail(USX_ERR_INVALID, "usx_cu_pulse: output too small");
    for (int i = -n_half; i <= n_half; ++i) {
      const float t = static_cast<float>(i) / fs_os;
      out[i + n_half] = std::exp(-0.5f * (t * t) / (sigma * sigma)) * std::cos(2.0f * kPi * f0 * t);
    }
  }
  return USX_OK;
}

// design_lowpass (reference demodulate.cpp:13-34), host arithmetic.
int usx_cu_design_lowpass(int n_taps, float normalized_cutoff, float* h, int cap, int* n_out) {
  if (n_taps < 3) n_taps = 3;
  if (n_taps % 2 == 0) ++n_taps;
  if (n_out) *n_out = n_taps;
  if (!h) return USX_OK;
  if (cap < n_taps) return fail(USX_ERR_INVALID, "usx_cu_design_lowpass: output too small");
  const float fc = std::min(std::max(normalized_cutoff, 1e-4f), 0.499f);
  const int m = n_taps / 2;
  float sum = 0.0f;
  for (int i = 0; i < n_taps; ++i) {
    const int k = i - m;
    const float sinc = (k == 0) ? 2.0f * fc
                                : std::sin(2.0f * kPi * fc * static_cast<float>(k)) /
                                      (kPi * static_cast<float>(k));
    const float w = 0.54f - 0.46f * std::cos(2.0f * kPi * static_cast<float>(i) /
                                             static_cast<float>(n_taps - 1));
    h[i] = sinc * w;
    sum += sinc * w;
  }
  if (sum != 0.0f)
    for (int i = 0; i < n_taps; ++i) h[i] /= sum;
  return USX_OK;
}

}  // extern "C"
