// simulate.cu — point-scatterer forward model (reference simulator.cpp:213-419),
// in two stages per group of transmit events, with no floating-point atomics
// (runs are bit-identical):
//
//   incident_kernel  one warp per (scatterer, event): the incident field at
//            the (moved) scatterer, a sum over firing elements of the delayed,
//            weighted two-way pulse linearly interpolated onto an oversampled
//            time axis, built in the warp's shared-memory buffer. Per element
//            the lanes split the buffer slots the pulse covers; each slot adds
//            the "next sample" term of the previous tap and then the "this
//            sample" term of its own tap, which is exactly the order in which
//            the reference's serial tap loop updates each buffer position, so
//            the buffer is bit-identical. Its -40 dB tails are trimmed (warp
//            max + ballots) and the trimmed field goes to global memory with a
//            header (start time, length, position, amplitude);
//   echo_kernel      one CTA per (group of elements, event, slice of the
//            scatterer list), one warp per element: the lanes take 32
//            scatterers at a time, each setting up its echo on the warp's
//            element (distance, amplitude, delay, sample window) and adding
//            its echo samples (linear interpolation of the trimmed incident
//            field) into the element's row in shared memory. The row holds
//            64-bit fixed-point integers (the samples times 2^s, s chosen from
//            a bound on every sum so nothing overflows), so the additions are
//            exact and their order does not matter: every run gives the same
//            bits. Rows are added (as integers) into a global accumulator;
//   fixed_to_float_kernel converts the accumulator to the float RF.
//
// The reference reduces per-thread buffers in `omp critical` order, which is
// arbitrary; here each RF sample is the exact sum of its contributions, each
// rounded to the fixed-point step (2^-61 of the bound on any sum: for 100,000
// scatterers about 1e-13 of one scatterer's largest echo, far below the float
// rounding of a sample).
//
// Receive noise is added by a third kernel once an event's echoes are
// complete: sigma = peak|RF| * 10^(noise_db/20), RF += z * sigma, with z the
// host-generated standard normals of the reference's per-event generator.
#include <algorithm>
#include <cmath>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kSimWarps = 4;       // incident_kernel: warps (scatterers) per CTA
constexpr int kEchoWarps = 4;      // echo_kernel: warps (elements) per CTA
constexpr int kMaxElem = 256;
constexpr int kMaxPulse = 1024;

struct SimArgs {
  const usx_scatterer* scat;
  long n_scat;
  const float* delays;     // [ev][n_el]
  const float* apod;       // [ev][n_el] (1 where the transmit has no apodization)
  const int* active;       // [ev][n_el] active element list
  const int* n_active;     // [ev]
  const float* pulse;      // [pulse_n]
  float* rf;               // [ev][n_el][n_smp]
  unsigned long long* counter;
  float* inc;              // [ev - ev0][n_scat][inc_cap] trimmed incident fields
  unsigned long long* acc; // [ev - ev0][n_el][n_smp] 64-bit fixed-point RF of the group
  unsigned* bound_bits;    // bound on one scatterer's contribution to any sample (float bits)
  long slice_len;          // scatterers per slice
  float4* hdr;             // [ev - ev0][n_scat][2]: (t0, length bits, amplitude, -), (x, y, z, -)
  int ev0;                 // first event of this group
  int n_el, n_smp, n_ev, pulse_n, inc_cap;
  float c, fs, t0, fs_os, lambda, width, prf, half_nm1, pitch;
  float pulse_half, max_window_s, trim_amp, atten_db_per_m;
  int spreading, directivity_on, motion, full;
};

__device__ __forceinline__ float elem_amp(const SimArgs& a, float base_amp, float px, float ex, float r) {
  float amp = base_amp;
  if (a.spreading) amp /= r;
  if (a.directivity_on) {
    const float sin_th = (px - ex) / r;
    amp *= directivity(a.width, a.lambda, sin_th);
  }
  if (a.atten_db_per_m > 0.0f) amp *= powf(10.0f, -a.atten_db_per_m * r / 20.0f);
  return amp;
}

__global__ void __launch_bounds__(32 * kSimWarps) incident_kernel(const SimArgs a) {
  extern __shared__ float4 sim_smem[];
  float* pulse = reinterpret_cast<float*>(sim_smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per_warp = a.inc_cap + 4 * kMaxElem;
  float* mine = pulse + kMaxPulse + warp * per_warp;
  float* inc = mine;                            // [inc_cap]
  float* e_r = inc + a.inc_cap;                 // distance to each element
  float* e_amp = e_r + kMaxElem;                // stage-1 amplitude (active order)
  float* e_ctr = e_amp + kMaxElem;              // stage-1 centre index (active order)
  int* e_base = reinterpret_cast<int*>(e_ctr + kMaxElem);
  for (int k = threadIdx.x; k < a.pulse_n; k += blockDim.x) pulse[k] = a.pulse[k];
  __syncthreads();

  const int evl = blockIdx.y, ev = a.ev0 + evl;
  const float event_time = static_cast<float>(ev) / a.prf;
  const int n_act = a.n_active[ev];
  const int* act = a.active + static_cast<long>(ev) * a.n_el;
  const float* dly = a.delays + static_cast<long>(ev) * a.n_el;
  const float* apd = a.apod + static_cast<long>(ev) * a.n_el;

  for (long si = static_cast<long>(blockIdx.x) * kSimWarps + warp; si < a.n_scat;
       si += static_cast<long>(gridDim.x) * kSimWarps) {
    __syncwarp();  // the previous scatterer's buffers are no longer read
    float4* hd = a.hdr + 2 * (static_cast<long>(evl) * a.n_scat + si);
    const usx_scatterer sc = a.scat[si];
    int trim_n = 0;
    float trim_t0 = 0.0f;
    float px = sc.x, py = sc.y, pz = sc.z;
    if (a.motion) {
      px = px + sc.vx * event_time;
      py = py + sc.vy * event_time;
      pz = pz + sc.vz * event_time;
    }
    if (sc.amplitude != 0.0f && pz > 0.0f) {
      // Distances to every element.
      for (int e = lane; e < a.n_el; e += 32) {
        const float ex = (static_cast<float>(e) - a.half_nm1) * a.pitch;
        e_r[e] = dist3(px, py, pz, ex, 0.0f, 0.0f);
      }
      __syncwarp();
      // ---- arrival span over firing elements ------------------------------
      float t_min = INFINITY, t_max = -INFINITY;
      for (int q = lane; q < n_act; q += 32) {
        const int e = act[q];
        const float t = dly[e] + e_r[e] / a.c;
        t_min = fminf(t_min, t);
        t_max = fmaxf(t_max, t);
      }
      for (int o = 16; o > 0; o >>= 1) {
        t_min = fminf(t_min, __shfl_xor_sync(0xffffffffu, t_min, o));
        t_max = fmaxf(t_max, __shfl_xor_sync(0xffffffffu, t_max, o));
      }
      float span = (t_max - t_min) + 2.0f * a.pulse_half;
      span = fminf(span, a.max_window_s + 2.0f * a.pulse_half);
      const float inc_t0 = t_min - a.pulse_half;
      const int inc_n = static_cast<int>(ceilf(span * a.fs_os)) + 2;
      if (inc_n <= a.inc_cap && inc_n > 0) {  // the cap bounds the window: always
        for (int k = lane; k < inc_n; k += 32) inc[k] = 0.0f;
        // Per firing element: amplitude and pulse placement.
        for (int q = lane; q < n_act; q += 32) {
          const int e = act[q];
          const float r = e_r[e];
          float amp = 0.0f;
          float centre = 0.0f;
          if (!(r < 1e-6f)) {
            const float ex = (static_cast<float>(e) - a.half_nm1) * a.pitch;
            amp = elem_amp(a, apd[e], px, ex, r);
            const float t_arr = dly[e] + r / a.c;
            centre = (t_arr - inc_t0) * a.fs_os;
          }
          e_amp[q] = (r < 1e-6f) ? 0.0f : amp;
          e_ctr[q] = centre;
          e_base[q] = static_cast<int>(floorf(centre)) - a.pulse_n / 2;
        }
        __syncwarp();
        for (int q = 0; q < n_act; ++q) {
          const float amp = e_amp[q];
          if (amp == 0.0f) continue;
          const float centre = e_ctr[q];
          const int base = e_base[q];
          const float frac = centre - floorf(centre);
          const float omf = 1.0f - frac;
          // One lane per buffer slot s = base + j: first the "next sample"
          // term of tap j - 1, then the "this sample" term of tap j.
          for (int j = lane; j <= a.pulse_n; j += 32) {
            const int s = base + j;
            const bool nx = j >= 1 && s >= 1 && s < inc_n;          // tap j - 1 at index s - 1
            const bool th = j < a.pulse_n && s >= 0 && s + 1 < inc_n; // tap j at index s
            if (!nx && !th) continue;
            float t = inc[s];
            if (nx) t += (amp * pulse[j - 1]) * frac;
            if (th) t += (amp * pulse[j]) * omf;
            inc[s] = t;
          }
          __syncwarp();
          if (!a.full) break;
        }
        // ---- trim the -40 dB tails -----------------------------------------
        float peak = 0.0f;
        for (int k = lane; k < inc_n; k += 32) peak = fmaxf(peak, fabsf(inc[k]));
        for (int o = 16; o > 0; o >>= 1) peak = fmaxf(peak, __shfl_xor_sync(0xffffffffu, peak, o));
        if (peak > 0.0f) {
          const float thr = peak * a.trim_amp;
          int lo = inc_n, hi = -1;
          for (int k0 = 0; k0 < inc_n; k0 += 32) {
            const int k = k0 + lane;
            const bool keep = k < inc_n && !(fabsf(inc[k]) < thr);
            const unsigned m = __ballot_sync(0xffffffffu, keep);
            if (m) {
              lo = min(lo, k0 + __ffs(m) - 1);
              hi = max(hi, k0 + 31 - __clz(m));
            }
          }
          if (lo < inc_n && hi > lo) {
            trim_t0 = inc_t0 + static_cast<float>(lo) / a.fs_os;
            trim_n = hi - lo + 1;
            float* dst = a.inc + (static_cast<long>(evl) * a.n_scat + si) * a.inc_cap;
            for (int k = lane; k < trim_n; k += 32) dst[k] = inc[lo + k];
            // Largest contribution of this scatterer to any RF sample:
            // |amplitude| x peak of the field x the largest element factor
            // (directivity and attenuation are at most 1; spreading 1 / r).
            float r_min = INFINITY;
            for (int e = lane; e < a.n_el; e += 32) r_min = fminf(r_min, e_r[e]);
            for (int o = 16; o > 0; o >>= 1) r_min = fminf(r_min, __shfl_xor_sync(0xffffffffu, r_min, o));
            const float spread = a.spreading ? 1.0f / fmaxf(r_min, 1e-6f) : 1.0f;
            const float bnd = fabsf(sc.amplitude) * peak * spread * 1.001f;
            if (lane == 0 && bnd > 0.0f) atomicMax(a.bound_bits, __float_as_uint(bnd));
          }
        }
      }
    }
    if (lane == 0) {
      hd[0] = make_float4(trim_t0, __int_as_float(trim_n), sc.amplitude, 0.0f);
      hd[1] = make_float4(px, py, pz, 0.0f);
    }
  }
}

// Fixed-point shift of a group: samples are stored times 2^(61 - e) with
// n_scat x bound < 2^e, so no sum of contributions reaches 2^61 in
// magnitude. The same on every thread.
__device__ __forceinline__ int fixed_shift(const SimArgs& a) {
  const float bound = __uint_as_float(*a.bound_bits);
  int e = 0;
  frexp(static_cast<double>(bound) * static_cast<double>(a.n_scat), &e);
  return 61 - e;
}

__global__ void __launch_bounds__(32 * kEchoWarps) echo_kernel(const SimArgs a) {
  extern __shared__ float4 echo_smem[];
  unsigned long long* rows = reinterpret_cast<unsigned long long*>(echo_smem);   // [warps][n_smp]
  float* t_axis = reinterpret_cast<float*>(rows + kEchoWarps * a.n_smp);       // [n_smp]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Sample times t0 + n / fs of the RF axis, each computed as the reference
  // does (float division).
  for (int n = threadIdx.x; n < a.n_smp; n += blockDim.x) t_axis[n] = a.t0 + static_cast<float>(n) / a.fs;
  for (int k = threadIdx.x; k < kEchoWarps * a.n_smp; k += blockDim.x) rows[k] = 0ull;
  __syncthreads();
  // 2^shift as two float factors, each within float range whatever the bound.
  const int shift = fixed_shift(a);
  const float scale1 = ldexpf(1.0f, shift / 2), scale2 = ldexpf(1.0f, shift - shift / 2);
  const int evl = blockIdx.y, slice = blockIdx.z;
  const int e = blockIdx.x * kEchoWarps + warp;
  const long s_begin = static_cast<long>(slice) * a.slice_len;
  const long s_end = min(a.n_scat, s_begin + a.slice_len);
  unsigned long long samples = 0;
  if (e < a.n_el) {
    unsigned long long* row = rows + warp * a.n_smp;
    const float ex = (static_cast<float>(e) - a.half_nm1) * a.pitch;
    const float4* hdr = a.hdr + 2 * static_cast<long>(evl) * a.n_scat;
    const float* incs = a.inc + static_cast<long>(evl) * a.n_scat * a.inc_cap;
    for (long s0 = s_begin; s0 < s_end; s0 += 32) {
      // Lane = scatterer: its echo on this element.
      const long si = s0 + lane;
      int n0 = 1, n1 = 0;
      float amp = 0.0f, delay = 0.0f, trim_t0 = 0.0f;
      int trim_n = 0;
      if (si < s_end) {
        const float4 h0 = __ldg(hdr + 2 * si);
        trim_n = __float_as_int(h0.y);
        if (trim_n > 0) {
          const float4 h1 = __ldg(hdr + 2 * si + 1);
          const float r = dist3(h1.x, h1.y, h1.z, ex, 0.0f, 0.0f);
          if (!(r < 1e-6f)) {
            amp = elem_amp(a, h0.z, h1.x, ex, r);
            if (amp != 0.0f) {
              trim_t0 = h0.x;
              delay = r / a.c;
              const float span_t = static_cast<float>(trim_n - 1) / a.fs_os;
              const float t_start = trim_t0 + delay;
              const float t_end = t_start + span_t;
              n0 = max(static_cast<int>(ceilf((t_start - a.t0) * a.fs)), 0);
              n1 = min(static_cast<int>(floorf((t_end - a.t0) * a.fs)), a.n_smp - 1);
            }
          }
        }
      }
      if (n0 <= n1) {
        samples += static_cast<unsigned long long>(n1 - n0 + 1);
        const float* tr = incs + si * a.inc_cap;
        for (int n = n0; n <= n1; ++n) {
          const float t = t_axis[n] - delay;
          const float u = (t - trim_t0) * a.fs_os;
          const int k = static_cast<int>(u);
          if (k < 0 || k + 1 >= trim_n) continue;
          const float f = u - static_cast<float>(k);
          const float va = __ldg(tr + k), vb = __ldg(tr + k + 1);
          const float v = amp * (va + (vb - va) * f);
          atomicAdd(row + n, static_cast<unsigned long long>(__float2ll_rn((v * scale1) * scale2)));
        }
      }
    }
    __syncwarp();
    unsigned long long* dst = a.acc + (static_cast<long>(evl) * a.n_el + e) * a.n_smp;
    for (int n = lane; n < a.n_smp; n += 32)
      if (row[n]) atomicAdd(dst + n, row[n]);
  }
  for (int o = 16; o > 0; o >>= 1) samples += __shfl_xor_sync(0xffffffffu, samples, o);
  if (lane == 0 && samples) atomicAdd(a.counter, samples);
}

// RF of the group's events from the fixed-point accumulator.
__global__ void fixed_to_float_kernel(const SimArgs a, int n_ev_group) {
  const long per_ev = static_cast<long>(a.n_el) * a.n_smp;
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= per_ev * n_ev_group) return;
  const double inv = ldexp(1.0, -fixed_shift(a));
  const long evl = i / per_ev, k = i - evl * per_ev;
  const long long v = static_cast<long long>(a.acc[i]);
  a.rf[(a.ev0 + evl) * per_ev + k] = static_cast<float>(static_cast<double>(v) * inv);
}

__global__ void event_peak_kernel(const float* rf, long ev_size, unsigned* peak_bits) {
  const int ev = blockIdx.y;
  const float* x = rf + ev * ev_size;
  float m = 0.0f;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < ev_size;
       i += static_cast<long>(gridDim.x) * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && m > 0.0f) atomicMax(peak_bits + ev, __float_as_uint(m));
}

__global__ void add_noise_kernel(float* rf, const float* z, long ev_size, const unsigned* peak_bits,
                                 float noise_amp) {
  const int ev = blockIdx.y;
  const float peak = __uint_as_float(peak_bits[ev]);
  if (!(peak > 0.0f)) return;
  const float sigma = peak * noise_amp;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < ev_size;
       i += static_cast<long>(gridDim.x) * blockDim.x) {
    const long k = ev * ev_size + i;
    rf[k] = rf[k] + (z[k] * sigma + 0.0f);
  }
}

}  // namespace
}  // namespace usxcu

using namespace usxcu;

extern "C" int usx_cu_simulate(usx_ctx* ctx, const usx_channel_desc* cd,
                               const usx_simulator_config* cfg, const usx_scatterer* scat,
                               int64_t n_scat, const float* noise_z, float* rf, double* stats) {
  if (!ctx || !cd || !cfg || !rf) return fail(USX_ERR_INVALID, "usx_cu_simulate: null argument");
  if (n_scat > 0 && !scat) return fail(USX_ERR_INVALID, "usx_cu_simulate: null scatterers");
  if (int rc = validate_channel(*cd)) return rc;
  const int n_el = cd->probe.n_elements, n_smp = cd->acq.n_samples, n_ev = cd->n_events;
  if (n_el > kMaxElem) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: more than 256 elements");
  if (n_ev > 65535) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: more than 65535 events");
  const long ev_size = static_cast<long>(n_el) * n_smp;

  // Host-side constants with the reference's float arithmetic.
  int pulse_n = 0;
  float pulse_half = 0.0f;
  usx_cu_pulse(&cd->probe, &cd->acq, cfg, nullptr, 0, &pulse_n, &pulse_half);
  if (pulse_n > kMaxPulse) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: pulse longer than 1024 taps");
  std::vector<float> pulse(static_cast<size_t>(pulse_n));
  usx_cu_pulse(&cd->probe, &cd->acq, cfg, pulse.data(), pulse_n, &pulse_n, &pulse_half);
  const int os = cfg->oversampling < 1 ? 1 : cfg->oversampling;
  const float fs = cd->acq.sampling_frequency;
  const float fs_os = fs * static_cast<float>(os);
  const float f0_mhz = cd->probe.center_frequency * 1e-6f;
  const float atten = cfg->apply_attenuation ? cd->medium.attenuation * f0_mhz * 100.0f : 0.0f;
  const float max_window_s = cfg->max_incident_window_us * 1e-6f;
  const float trim_amp = std::pow(10.0f, cfg->incident_trim_db / 20.0f);
  // Largest incident buffer the window clamp allows.
  const double cap_d = std::ceil((static_cast<double>(max_window_s) + 2.0 * pulse_half) * fs_os) + 8.0;
  if (!(cap_d < 65536.0)) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: incident window too long");
  const int inc_cap = static_cast<int>(cap_d);

  std::vector<float> delays(static_cast<size_t>(n_ev) * n_el, 0.0f), apod(delays.size(), 1.0f);
  std::vector<int> active(delays.size(), 0), n_active(static_cast<size_t>(n_ev), 0);
  for (int e = 0; e < n_ev; ++e) {
    const usx_transmit& t = cd->transmits[e];
    int na = 0;
    for (int i = 0; i < n_el; ++i) {
      delays[static_cast<size_t>(e) * n_el + i] = t.delays ? t.delays[i] : 0.0f;
      apod[static_cast<size_t>(e) * n_el + i] = t.apodization ? t.apodization[i] : 1.0f;
      if (t.apodization && t.apodization[i] != 0.0f) active[static_cast<size_t>(e) * n_el + na++] = i;
    }
    if (na == 0)
      for (int i = 0; i < n_el; ++i) active[static_cast<size_t>(e) * n_el + na++] = i;
    n_active[static_cast<size_t>(e)] = na;
  }
  const size_t tbl = delays.size();
  // Event groups whose trimmed incident fields (inc_cap floats per scatterer
  // and event, of which only the trimmed part is written) fit about 2 GB.
  const long n_sc = std::max<long>(1, n_scat);
  const size_t per_event = static_cast<size_t>(n_sc) * (static_cast<size_t>(inc_cap) * sizeof(float) + 2 * sizeof(float4));
  const int group = static_cast<int>(std::max<size_t>(1, std::min<size_t>(n_ev, (size_t(2) << 30) / per_event)));
  // The echo stage in scatterer slices: enough CTAs for about four waves of
  // the GPU; the slices' fixed-point rows add exactly into one accumulator.
  // Each CTA keeps kEchoWarps fixed-point rows and the sample-time axis in
  // shared memory.
  const size_t smem_echo = sizeof(unsigned long long) * kEchoWarps * static_cast<size_t>(n_smp) +
                           sizeof(float) * static_cast<size_t>(n_smp);
  if (smem_echo > 227 * 1024) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: more than 6,900 samples per trace");
  const long base_ctas = static_cast<long>(ceil_div(n_el, kEchoWarps)) * group;
  const int n_slices = static_cast<int>(std::max<long>(1, std::min<long>({static_cast<long>(ctx->sm_count) * 12 /
                                                                             std::max<long>(1, base_ctas),
                                                                         (n_sc + 31) / 32, 4096})));
  const long slice_len = ((n_sc + n_slices - 1) / n_slices + 31) / 32 * 32;
  const size_t acc_bytes = sizeof(unsigned long long) * static_cast<size_t>(group) * n_el * n_smp;
  const size_t bytes = sizeof(float) * (2 * tbl + pulse.size()) + sizeof(int) * (tbl + n_ev) +
                       sizeof(unsigned long long) + sizeof(unsigned) * (n_ev + 1) + per_event * group + acc_bytes +
                       4096;
  void* ws = nullptr;
  if (int rc = scratch(ctx, bytes, &ws)) return rc;
  char* w = static_cast<char*>(ws);
  auto take = [&](size_t b) {
    char* p = w;
    w += (b + 255) / 256 * 256;
    return p;
  };
  unsigned long long* d_counter = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  unsigned* d_peak = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * n_ev));
  float* d_delays = reinterpret_cast<float*>(take(sizeof(float) * tbl));
  float* d_apod = reinterpret_cast<float*>(take(sizeof(float) * tbl));
  int* d_active = reinterpret_cast<int*>(take(sizeof(int) * tbl));
  int* d_nact = reinterpret_cast<int*>(take(sizeof(int) * n_ev));
  float* d_pulse = reinterpret_cast<float*>(take(sizeof(float) * pulse.size()));
  float4* d_hdr = reinterpret_cast<float4*>(take(sizeof(float4) * 2 * static_cast<size_t>(n_sc) * group));
  float* d_inc = reinterpret_cast<float*>(take(sizeof(float) * static_cast<size_t>(inc_cap) * n_sc * group));
  unsigned long long* d_acc = reinterpret_cast<unsigned long long*>(take(acc_bytes));
  unsigned* d_bound = reinterpret_cast<unsigned*>(take(sizeof(unsigned)));
  if (static_cast<size_t>(w - static_cast<char*>(ws)) > ctx->scratch_bytes)
    return fail(USX_ERR_INVALID, "usx_cu_simulate: scratch layout overflow");
  USX_CUDA(cudaMemsetAsync(d_counter, 0, sizeof(unsigned long long), ctx->stream));
  USX_CUDA(cudaMemcpyAsync(d_delays, delays.data(), sizeof(float) * tbl, cudaMemcpyHostToDevice, ctx->stream));
  USX_CUDA(cudaMemcpyAsync(d_apod, apod.data(), sizeof(float) * tbl, cudaMemcpyHostToDevice, ctx->stream));
  USX_CUDA(cudaMemcpyAsync(d_active, active.data(), sizeof(int) * tbl, cudaMemcpyHostToDevice, ctx->stream));
  USX_CUDA(cudaMemcpyAsync(d_nact, n_active.data(), sizeof(int) * n_ev, cudaMemcpyHostToDevice, ctx->stream));
  USX_CUDA(cudaMemcpyAsync(d_pulse, pulse.data(), sizeof(float) * pulse.size(), cudaMemcpyHostToDevice,
                           ctx->stream));

  SimArgs a;
  a.scat = scat;
  a.n_scat = n_scat;
  a.delays = d_delays;
  a.apod = d_apod;
  a.active = d_active;
  a.n_active = d_nact;
  a.pulse = d_pulse;
  a.rf = rf;
  a.counter = d_counter;
  a.inc = d_inc;
  a.acc = d_acc;
  a.bound_bits = d_bound;
  a.slice_len = slice_len;
  a.hdr = d_hdr;
  a.ev0 = 0;
  a.n_el = n_el;
  a.n_smp = n_smp;
  a.n_ev = n_ev;
  a.pulse_n = pulse_n;
  a.inc_cap = inc_cap;
  a.c = cd->medium.speed_of_sound;
  a.fs = fs;
  a.t0 = cd->acq.t0;
  a.fs_os = fs_os;
  a.lambda = cd->medium.speed_of_sound / cd->probe.center_frequency;
  a.width = cd->probe.element_width;
  a.prf = cd->acq.prf;
  a.half_nm1 = 0.5f * static_cast<float>(n_el - 1);
  a.pitch = cd->probe.pitch;
  a.pulse_half = pulse_half;
  a.max_window_s = max_window_s;
  a.trim_amp = trim_amp;
  a.atten_db_per_m = atten;
  a.spreading = cfg->apply_spreading;
  a.directivity_on = cfg->apply_directivity;
  a.motion = cfg->enable_motion;
  a.full = cfg->full_transmit_diffraction;
  const size_t smem_inc = sizeof(float) * (kMaxPulse + static_cast<size_t>(kSimWarps) * (inc_cap + 4 * kMaxElem));
  if (smem_inc > 227 * 1024) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: incident window too long");
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(incident_kernel), smem_inc)) return rc_;
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(echo_kernel), smem_echo)) return rc_;
  if (n_scat > 0) {
    int per_sm = 0;
    if (int rc_ = occupancy(reinterpret_cast<const void*>(incident_kernel), 32 * kSimWarps, smem_inc, &per_sm))
      return rc_;
    for (int e0 = 0; e0 < n_ev; e0 += group) {
      const int ng = std::min(group, n_ev - e0);
      a.ev0 = e0;
      const long want = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count * 4 / ng;
      const long need = (n_scat + kSimWarps - 1) / kSimWarps;
      const unsigned gx = static_cast<unsigned>(std::max(1L, std::min(want, need)));
      USX_CUDA(cudaMemsetAsync(d_bound, 0, sizeof(unsigned), ctx->stream));
      USX_CUDA(cudaMemsetAsync(d_acc, 0, sizeof(unsigned long long) * static_cast<size_t>(ng) * n_el * n_smp,
                               ctx->stream));
      prof_begin(ctx, "incident_kernel");
      incident_kernel<<<dim3(gx, ng), 32 * kSimWarps, smem_inc, ctx->stream>>>(a);
      prof_end(ctx);
      USX_CHECK_LAUNCH("incident_kernel");
      prof_begin(ctx, "echo_kernel");
      echo_kernel<<<dim3(static_cast<unsigned>(ceil_div(n_el, kEchoWarps)), ng, n_slices), 32 * kEchoWarps,
                    smem_echo, ctx->stream>>>(a);
      prof_end(ctx);
      USX_CHECK_LAUNCH("echo_kernel");
      prof_begin(ctx, "fixed_to_float_kernel");
      fixed_to_float_kernel<<<static_cast<unsigned>(ceil_div(static_cast<long>(ng) * n_el * n_smp, 256)), 256, 0,
                              ctx->stream>>>(a, ng);
      prof_end(ctx);
      USX_CHECK_LAUNCH("fixed_to_float_kernel");
    }
  } else {
    USX_CUDA(cudaMemsetAsync(rf, 0, sizeof(float) * ev_size * n_ev, ctx->stream));
  }
  if (cfg->noise_db > -200.0f && noise_z) {
    USX_CUDA(cudaMemsetAsync(d_peak, 0, sizeof(unsigned) * n_ev, ctx->stream));
    const int bx = std::max(1, std::min(ceil_div(ev_size, 256), 64));
    event_peak_kernel<<<dim3(bx, n_ev), 256, 0, ctx->stream>>>(rf, ev_size, d_peak);
    USX_CHECK_LAUNCH("event_peak_kernel");
    const float noise_amp = std::pow(10.0f, cfg->noise_db / 20.0f);
    add_noise_kernel<<<dim3(bx, n_ev), 256, 0, ctx->stream>>>(rf, noise_z, ev_size, d_peak, noise_amp);
    USX_CHECK_LAUNCH("add_noise_kernel");
  }
  // Host tables must outlive their asynchronous copies.
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  if (stats) {
    unsigned long long n = 0;
    USX_CUDA(cudaMemcpy(&n, d_counter, sizeof(n), cudaMemcpyDeviceToHost));
    stats[0] = static_cast<double>(n);
    // 4 flops per accumulated echo sample (lerp + scaled accumulate).
    stats[1] = 4.0 * static_cast<double>(n);
  }
  return USX_OK;
}
