// simulate.cu — point-scatterer forward model (reference simulator.cpp:213-419).
//
// One warp owns one (scatterer, transmit event) at a time (eight warps per
// CTA):
//   stage 1  the incident field at the scatterer, a sum over firing elements of
//            the delayed, weighted two-way pulse linearly interpolated onto an
//            oversampled time axis, built in the warp's shared-memory buffer.
//            Per element the lanes split the buffer slots the pulse covers;
//            each slot adds the "next sample" term of the previous tap and
//            then the "this sample" term of its own tap, which is exactly the
//            order in which the reference's serial tap loop updates each
//            buffer position, so the buffer is bit-identical;
//   trim     the buffer's -40 dB tails are cut (warp max + ballots);
//   stage 2  the echo set-up of every receive element, one element per lane
//            (amplitude, delay, sample window), then per element the lanes
//            produce the delayed, weighted echo samples.
// Each echo sample is added to a 64-bit fixed-point accumulator of the RF
// (fire-and-forget integer reductions): the sample times 2^s, with s chosen
// from a bound on every RF sum (sim_bound_kernel) so that nothing overflows.
// Integer addition is exact and commutative, so the RF is the same bit for
// bit on every run whatever order the warps add their echoes in (the
// reference reduces its per-thread float buffers in `omp critical` order,
// which is arbitrary). fixed_to_float_kernel converts the accumulator; the
// fixed-point step is 2^-61 of the bound on any sum (for realistic phantoms
// well below the float rounding of a sample).
//
// Occupancy: a warp keeps a 1,536-sample incident buffer and element tables
// sized to the probe in shared memory (8 KB at 128 elements), so that eight
// warps per CTA and three CTAs per SM fit; windows longer than the buffer
// (up to the 30 us clamp) use the warp's slot of a global buffer through the
// same generic pointer, and the grid is persistent over (event, block of
// scatterers) items so that there is one slot per resident warp. Against
// buffers sized for the clamp (10 warps per SM): 509 -> 311 ms for 100,000
// scatterers. The fixed-point scale (a power of two) is folded into each
// element's amplitude, which gives the same scaled samples exactly. A
// 960-sample buffer with a register cap for four CTAs per SM (58 registers)
// measured slower (356 ms).
//
// Measured and dropped (100,000 scatterers, 75 events x 128 elements, 509 ms
// for the kernel at the time): the incident waveforms of a batch written to a pool and
// an echo kernel whose warps each own one element's RF row in shared memory
// and add every scatterer's echo in ascending order (no atomics, bit-exact
// order): 834 ms, the waveform reads going to L2 once per element because
// the rows leave little L1.
//
// Receive noise is added by a second kernel once an event's echoes are
// complete: sigma = peak|RF| * 10^(noise_db/20), RF += z * sigma, with z the
// host-generated standard normals of the reference's per-event generator.
#include <algorithm>
#include <cmath>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kSimWarps = 8;
constexpr int kMaxElem = 256;
constexpr int kMaxPulse = 1024;
constexpr int kMaxTimeTable = 8192;
// Incident samples a warp keeps in shared memory; a longer window (up to the
// clamp) uses the warp's slot of a global-memory buffer instead.
constexpr int kIncSmall = 1536;

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
  unsigned long long* acc; // [ev][n_el][n_smp] 64-bit fixed-point RF
  const unsigned* bound_bits;  // bound on one scatterer's contribution to any sample (float bits)
  float apod_sum_max;      // largest sum of transmit apodisation over the events
  float pulse_max;         // largest |pulse tap|
  int n_el, n_smp, n_ev, pulse_n, inc_cap, scat_per_block;
  int pulse_pad, tbl_pad, inc_small;  // shared-memory layout (floats)
  long n_sblocks, n_items;  // scatterer blocks per event; work items (events x blocks)
  float* inc_global;       // [block][warp][inc_cap] incident buffers for long windows
  float c, fs, t0, fs_os, lambda, width, prf, half_nm1, pitch;
  float pulse_half, max_window_s, trim_amp, atten_db_per_m;
  int spreading, directivity_on, motion, full;
  int t_table;             // the block holds the sample-time table (n_smp <= kMaxTimeTable)
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

// A bound on one scatterer's contribution to any RF sample: the incident
// field is at most sum(apodisation) x max|pulse| x (1 / r with spreading),
// the echo at most |amplitude| x that x (1 / r); directivity and attenuation
// are at most 1, and r is at least the scatterer's smallest depth over the
// events (the elements lie at z = 0). Thread per scatterer; the maximum goes
// to bound_bits (an order-free atomic maximum).
__global__ void sim_bound_kernel(const SimArgs a) {
  const long si = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (si >= a.n_scat) return;
  const usx_scatterer sc = a.scat[si];
  float z_min = sc.z;
  if (a.motion) z_min = fminf(z_min, sc.z + sc.vz * (static_cast<float>(a.n_ev - 1) / a.prf));
  const float inv_r = a.spreading ? 1.0f / fmaxf(z_min, 1e-6f) : 1.0f;
  const float b = fabsf(sc.amplitude) * a.apod_sum_max * a.pulse_max * inv_r * inv_r * 1.01f;
  if (b > 0.0f) atomicMax(const_cast<unsigned*>(a.bound_bits), __float_as_uint(b));
}

// Fixed-point shift: samples are stored times 2^(61 - e) with
// n_scat x bound < 2^e, so no RF sum reaches 2^61 in magnitude.
__device__ __forceinline__ int fixed_shift(const SimArgs& a) {
  const float bound = __uint_as_float(*a.bound_bits);
  int e = 0;
  frexp(static_cast<double>(bound) * static_cast<double>(a.n_scat), &e);
  return 61 - e;
}

__global__ void __launch_bounds__(32 * kSimWarps) simulate_kernel(const SimArgs a) {
  extern __shared__ float4 sim_smem[];
  // Shared memory: the pulse, the sample-time table, then per warp a small
  // incident buffer and four element tables (sized to the probe).
  float* pulse = reinterpret_cast<float*>(sim_smem);
  float* t_axis = pulse + a.pulse_pad;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int per_warp = a.inc_small + 4 * a.tbl_pad;
  float* mine = t_axis + (a.t_table ? a.n_smp + (4 - a.n_smp % 4) % 4 : 0) + warp * per_warp;
  float* inc_smem = mine;                       // [inc_small]
  float* inc_glob = a.inc_global + (static_cast<long>(blockIdx.x) * kSimWarps + warp) * a.inc_cap;
  float* e_r = inc_smem + a.inc_small;          // distance to each element
  float* e_amp = e_r + a.tbl_pad;               // stage-1 amplitude (active order)
  float* e_ctr = e_amp + a.tbl_pad;             // stage-1 centre index (active order)
  int* e_base = reinterpret_cast<int*>(e_ctr + a.tbl_pad);
  for (int k = threadIdx.x; k < a.pulse_n; k += blockDim.x) pulse[k] = a.pulse[k];
  // Sample times t0 + n / fs of the RF axis, each computed as the reference
  // does (float division), once per block instead of once per echo sample.
  if (a.t_table)
    for (int n = threadIdx.x; n < a.n_smp; n += blockDim.x) t_axis[n] = a.t0 + static_cast<float>(n) / a.fs;
  __syncthreads();

  // 2^shift as two float factors, each within float range whatever the bound.
  const int shift = fixed_shift(a);
  const float scale1 = ldexpf(1.0f, shift / 2), scale2 = ldexpf(1.0f, shift - shift / 2);
  unsigned long long samples = 0;

  // Work items (event, block of scatterers), the grid persistent over them
  // (so that the global incident buffers are per resident CTA).
  for (long item = blockIdx.x; item < a.n_items; item += gridDim.x) {
  const int ev = static_cast<int>(item / a.n_sblocks);
  const long sb = item - static_cast<long>(ev) * a.n_sblocks;
  const float event_time = static_cast<float>(ev) / a.prf;
  const int n_act = a.n_active[ev];
  const int* act = a.active + static_cast<long>(ev) * a.n_el;
  const float* dly = a.delays + static_cast<long>(ev) * a.n_el;
  const float* apd = a.apod + static_cast<long>(ev) * a.n_el;
  unsigned long long* acc_ev = a.acc + static_cast<long>(ev) * a.n_el * a.n_smp;
  const long s_begin = sb * a.scat_per_block;
  const long s_end = min(a.n_scat, s_begin + a.scat_per_block);
  for (long si = s_begin + warp; si < s_end; si += kSimWarps) {
    __syncwarp();  // the previous scatterer's buffers are no longer read
    const usx_scatterer sc = a.scat[si];
    if (sc.amplitude == 0.0f) continue;
    float px = sc.x, py = sc.y, pz = sc.z;
    if (a.motion) {
      px = px + sc.vx * event_time;
      py = py + sc.vy * event_time;
      pz = pz + sc.vz * event_time;
    }
    if (pz <= 0.0f) continue;

    // Distances to every element.
    for (int e = lane; e < a.n_el; e += 32) {
      const float ex = (static_cast<float>(e) - a.half_nm1) * a.pitch;
      e_r[e] = dist3(px, py, pz, ex, 0.0f, 0.0f);
    }
    __syncwarp();

    // ---- stage 1: arrival span over firing elements -----------------------
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
    if (inc_n > a.inc_cap || inc_n <= 0) continue;  // cannot happen: cap bounds the window
    // The window in shared memory when it fits, else in the warp's global slot
    // (the same code through a generic pointer).
    float* inc = inc_n <= a.inc_small ? inc_smem : inc_glob;
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
      } else {
        amp = 0.0f;
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
      // One lane per buffer slot s = base + j: first the "next sample" term of
      // tap j - 1, then the "this sample" term of tap j, which is the order in
      // which the reference's serial tap loop updates slot s (see header).
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

    // ---- trim ----------------------------------------------------------------
    float peak = 0.0f;
    for (int k = lane; k < inc_n; k += 32) peak = fmaxf(peak, fabsf(inc[k]));
    for (int o = 16; o > 0; o >>= 1) peak = fmaxf(peak, __shfl_xor_sync(0xffffffffu, peak, o));
    if (peak <= 0.0f) continue;
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
    if (lo >= inc_n || hi <= lo) continue;
    const float trim_t0 = inc_t0 + static_cast<float>(lo) / a.fs_os;
    const int trim_n = hi - lo + 1;
    const float* tr = inc + lo;

    // ---- stage 2: echo on every receive element ---------------------------------
    // Per receive element, one lane each: amplitude, delay and the echo's
    // sample window (the stage-1 tables are free again; e_r[e] is read by
    // the lane that then overwrites it with the window's last sample).
    const float span_t = static_cast<float>(trim_n - 1) / a.fs_os;
    for (int e = lane; e < a.n_el; e += 32) {
      const float r = e_r[e];
      float amp = 0.0f, delay = 0.0f;
      int n0 = 1, n1 = 0;
      if (!(r < 1e-6f)) {
        const float ex = (static_cast<float>(e) - a.half_nm1) * a.pitch;
        amp = elem_amp(a, sc.amplitude, px, ex, r);
        if (amp != 0.0f) {
          delay = r / a.c;
          const float t_start = trim_t0 + delay;
          const float t_end = t_start + span_t;
          n0 = max(static_cast<int>(ceilf((t_start - a.t0) * a.fs)), 0);
          n1 = min(static_cast<int>(floorf((t_end - a.t0) * a.fs)), a.n_smp - 1);
        }
      }
      if (n0 > n1) {
        n0 = 1;
        n1 = 0;
      } else {
        samples += static_cast<unsigned long long>(n1 - n0 + 1);
      }
      // The fixed-point scale is a power of two, so scaling the amplitude
      // gives the scaled sample exactly: amp 2^s x lerp = (amp x lerp) 2^s.
      e_amp[e] = (amp * scale1) * scale2;
      e_ctr[e] = delay;
      e_base[e] = n0;
      e_r[e] = __int_as_float(n1);
    }
    __syncwarp();
    for (int e = 0; e < a.n_el; ++e) {
      const int n0 = e_base[e], n1 = __float_as_int(e_r[e]);
      if (n0 > n1) continue;
      const float amp = e_amp[e], delay = e_ctr[e];
      unsigned long long* dst = acc_ev + static_cast<long>(e) * a.n_smp;
      for (int n = n0 + lane; n <= n1; n += 32) {
        const float t = (a.t_table ? t_axis[n] : (a.t0 + static_cast<float>(n) / a.fs)) - delay;
        const float u = (t - trim_t0) * a.fs_os;
        const int k = static_cast<int>(u);
        if (k < 0 || k + 1 >= trim_n) continue;
        const float f = u - static_cast<float>(k);
        const float va = tr[k], vb = tr[k + 1];
        const float v = amp * (va + (vb - va) * f);
        atomicAdd(dst + n, static_cast<unsigned long long>(__float2ll_rn(v)));
      }
    }
    __syncwarp();
  }
  }  // work items
  for (int o = 16; o > 0; o >>= 1) samples += __shfl_xor_sync(0xffffffffu, samples, o);
  if (lane == 0 && samples) atomicAdd(a.counter, samples);
}

// RF from the fixed-point accumulator.
__global__ void fixed_to_float_kernel(const SimArgs a, long n) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const double inv = ldexp(1.0, -fixed_shift(a));
  a.rf[i] = static_cast<float>(static_cast<double>(static_cast<long long>(a.acc[i])) * inv);
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
  const size_t acc_bytes = sizeof(unsigned long long) * static_cast<size_t>(ev_size) * n_ev;
  // Work items: blocks of scatterers per event, enough to fill the GPU several
  // times over; the grid is persistent over them (at most eight CTAs per SM).
  const long target_blocks = std::max<long>(1, static_cast<long>(ctx->sm_count) * 8 / std::max(1, n_ev));
  const int scat_per_block = static_cast<int>(
      std::min<long>(256, std::max<long>(kSimWarps, (n_scat + target_blocks - 1) / target_blocks)));
  const long gx = std::max<long>(1, (n_scat + scat_per_block - 1) / scat_per_block);
  const long grid_max = std::max<long>(1, std::min<long>(gx * n_ev, 8L * ctx->sm_count));
  // Incident buffers for windows longer than the shared-memory one: one per
  // warp of the persistent grid.
  const size_t incg_bytes = sizeof(float) * static_cast<size_t>(grid_max) * kSimWarps * inc_cap;
  const size_t bytes = acc_bytes + incg_bytes + 512 + sizeof(float) * (2 * tbl + pulse.size()) +
                       sizeof(int) * (tbl + n_ev) + sizeof(unsigned long long) + sizeof(unsigned) * n_ev + 1024;
  void* ws = nullptr;
  if (int rc = scratch(ctx, bytes, &ws)) return rc;
  char* w = static_cast<char*>(ws);
  auto take = [&](size_t b) {
    char* p = w;
    w += (b + 255) / 256 * 256;
    return p;
  };
  unsigned long long* d_counter = reinterpret_cast<unsigned long long*>(take(sizeof(unsigned long long)));
  unsigned* d_peak = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * (n_ev + 1)));
  unsigned* d_bound = d_peak + n_ev;
  unsigned long long* d_acc = reinterpret_cast<unsigned long long*>(take(acc_bytes));
  float* d_incg = reinterpret_cast<float*>(take(incg_bytes));
  float* d_delays = reinterpret_cast<float*>(take(sizeof(float) * tbl));
  float* d_apod = reinterpret_cast<float*>(take(sizeof(float) * tbl));
  int* d_active = reinterpret_cast<int*>(take(sizeof(int) * tbl));
  int* d_nact = reinterpret_cast<int*>(take(sizeof(int) * n_ev));
  float* d_pulse = reinterpret_cast<float*>(take(sizeof(float) * pulse.size()));
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
  a.acc = d_acc;
  a.bound_bits = d_bound;
  {
    float apod_max = 0.0f;
    for (int e = 0; e < n_ev; ++e) {
      float sum = 0.0f;
      for (int i = 0; i < n_el; ++i) sum += std::fabs(apod[static_cast<size_t>(e) * n_el + i]);
      apod_max = std::max(apod_max, sum);
    }
    float pmax = 0.0f;
    for (float v : pulse) pmax = std::max(pmax, std::fabs(v));
    a.apod_sum_max = apod_max;
    a.pulse_max = pmax;
  }
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
  a.scat_per_block = scat_per_block;
  a.inc_global = d_incg;
  a.n_sblocks = gx;
  a.n_items = gx * n_ev;
  a.t_table = n_smp <= kMaxTimeTable ? 1 : 0;
  a.pulse_pad = (pulse_n + 3) / 4 * 4;
  a.tbl_pad = (n_el + 3) / 4 * 4;
  a.inc_small = std::min(kIncSmall, (inc_cap + 3) / 4 * 4);
  const size_t smem = sizeof(float) * (a.pulse_pad + (a.t_table ? (n_smp + 3) / 4 * 4 : 0) +
                                       static_cast<size_t>(kSimWarps) * (a.inc_small + 4 * a.tbl_pad));
  if (smem > 227 * 1024) return fail(USX_ERR_UNSUPPORTED, "usx_cu_simulate: incident window too long");
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(simulate_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  int per_sm = 0;
  if (int rc_ = occupancy(reinterpret_cast<const void*>(simulate_kernel), 32 * kSimWarps, smem, &per_sm)) return rc_;
  const long grid = std::max<long>(1, std::min<long>(grid_max, static_cast<long>(std::max(1, per_sm)) * ctx->sm_count));

  if (n_scat > 0) {
    prof_begin(ctx, "simulate_kernel");
    USX_CUDA(cudaMemsetAsync(d_bound, 0, sizeof(unsigned), ctx->stream));
    USX_CUDA(cudaMemsetAsync(d_acc, 0, acc_bytes, ctx->stream));
    sim_bound_kernel<<<static_cast<unsigned>(ceil_div(n_scat, 256)), 256, 0, ctx->stream>>>(a);
    USX_CHECK_LAUNCH("sim_bound_kernel");
    simulate_kernel<<<static_cast<unsigned>(grid), 32 * kSimWarps, smem, ctx->stream>>>(a);
    prof_end(ctx);
    USX_CHECK_LAUNCH("simulate_kernel");
    fixed_to_float_kernel<<<static_cast<unsigned>(ceil_div(ev_size * n_ev, 256)), 256, 0, ctx->stream>>>(
        a, ev_size * n_ev);
    USX_CHECK_LAUNCH("fixed_to_float_kernel");
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
