// beamform.cu — delay-and-sum with dynamic receive aperture, plane-wave /
// focused / diverging transmit compounding, and the DAS, DMAS, coherence-factor
// and minimum-variance combiners (reference beamformer.cpp:297-549).
//
// Kernel structure (das_kernel): one thread per pixel, pixels ordered with the
// depth axis fastest so a warp is 32 consecutive depths of one line; at a fixed
// (event, channel) its 32 delayed reads fall in one ~45-sample window of the
// trace, i.e. 2-3 cache lines, so the gather is served by L1/L2 with little
// waste. Channels are processed in groups of kGroup: for a group the receive
// geometry (aperture weight, receive delay, receive phasor) is computed once
// into registers, then every transmit event is visited in order and its
// geometry (illumination weight, transmit delay, transmit phasor) computed
// once per group; the kGroup per-channel sums stay in registers. This keeps
// the reference's summation order exactly — each channel sums its events in
// ascending order, channels are then combined in ascending order — so DAS,
// DMAS and CF reproduce the reference C++ bit for bit (to the last ulp of
// the device's sincosf/cosf), and it lets the non-linear combiners consume one
// finished channel at a time.
//
// Minimum variance exports the compounded per-channel samples Y[pixel][ch]
// and runs mv_kernel on them (one warp per pixel): spatially smoothed and
// range-averaged covariance, diagonal loading, Cholesky solve of R w = 1 and
// the weighted subarray average, in the reference's operation order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kGroup = 8;
constexpr int kBfThreads = 128;
constexpr int kMaxL = 64;
constexpr int kMaxCh = 256;
constexpr int kMvWarps = 2;
constexpr int kMaxRangeAvg = 4;

struct BfArgs {
  const float2* iq;      // IQ path: [ev][ch][smp]
  const float* rf;       // RF path
  long data_stride;      // elements between frames of a batch
  const float* points;   // [pix][3]
  const TxDev* tx;       // [n_events]
  float2* out;           // [pix] per frame
  long out_stride;
  float2* y_out;         // MV: [frame][pix][n_ch]
  float* acc_out;        // incoherent MV: per-pixel |out|^2 accumulator
  int n_ch, n_smp, n_pix, n1;
  int ev_begin, ev_end;
  int seq_epf;           // > 0: frame f uses events ev_begin + [f*seq_epf, (f+1)*seq_epf)
  int pass;              // >= 0: export only event (first event of the frame) + pass
  float c, fs, t0, fdem, two_pi_f, lambda, pitch, half_nm1;
  float f_number, tukey_alpha;
  int rx_window, combiner, compounding, tx_weighting, cf, is_mv;
  int mv_subarray, mv_range_average;
  float mv_loading;
  int* status;           // context status word (set when a bounded wait gives up)
};

__device__ __forceinline__ float elem_x(const BfArgs& a, int ch) {
  return (static_cast<float>(ch) - a.half_nm1) * a.pitch;
}

template <bool IQ>
__global__ void __launch_bounds__(kBfThreads) das_kernel(const BfArgs a) {
  const int pix = blockIdx.x * kBfThreads + threadIdx.x;
  if (pix >= a.n_pix) return;
  const long frame = blockIdx.y;
  const float px = __ldg(a.points + 3 * pix), py = __ldg(a.points + 3 * pix + 1),
              pz = __ldg(a.points + 3 * pix + 2);
  int ev_first = a.ev_begin, ev_last = a.ev_end;
  if (a.seq_epf > 0) {
    ev_first = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_last = ev_first + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_first += a.pass;
    ev_last = ev_first + 1;
  }
  const bool incoherent = a.compounding == USX_COMP_INCOHERENT && a.pass < 0;
  const bool select = a.compounding == USX_COMP_SELECT;

  int best_ev = -1;
  float best_w = 0.0f;
  if (select) {
    for (int ev = ev_first; ev < ev_last; ++ev) {
      const float tw = tx_sensitivity(a.tx[ev], px, pz, a.lambda, a.pitch);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }

  const int n_pass = incoherent ? (ev_last - ev_first) : 1;
  float inc_acc = 0.0f;
  cplx result = mk(0.f, 0.f);
  const float2* iq = IQ ? a.iq + frame * a.data_stride : nullptr;
  const float* rf = IQ ? nullptr : a.rf + frame * a.data_stride;

  for (int pass = 0; pass < max(1, n_pass); ++pass) {
    const int ev_lo = incoherent ? ev_first + pass : ev_first;
    const int ev_hi = incoherent ? ev_lo + 1 : ev_last;
    cplx das = mk(0.f, 0.f), s = mk(0.f, 0.f), q = mk(0.f, 0.f), coh = mk(0.f, 0.f);
    float incs = 0.0f;
    int n_active = 0;

    for (int g = 0; g < a.n_ch; g += kGroup) {
      float ap[kGroup], rt[kGroup], rc[kGroup], rs[kGroup];
      bool any = false;
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        const int ch = g + k;
        ap[k] = 0.0f;
        rt[k] = 0.0f;
        rc[k] = 1.0f;
        rs[k] = 0.0f;
        if (ch < a.n_ch) {
          const float ex = elem_x(a, ch);
          const float w = aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha);
          ap[k] = a.is_mv ? (w > 0.0f ? 1.0f : 0.0f) : w;
          if (w > 0.0f) {
            any = true;
            rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
            if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs[k], &rc[k]);
          }
        }
      }
      cplx Y[kGroup];
#pragma unroll
      for (int k = 0; k < kGroup; ++k) Y[k] = mk(0.f, 0.f);

      if (any) {
        for (int ev = ev_lo; ev < ev_hi; ++ev) {
          const TxDev& t = a.tx[ev];
          float tw;
          if (select) {
            tw = (best_ev == ev) ? best_w : 0.0f;
            if (tw > 0.0f) tw = 1.0f;
          } else if (a.tx_weighting) {
            tw = tx_sensitivity(t, px, pz, a.lambda, a.pitch);
          } else {
            tw = 1.0f;
          }
          if (tw <= 0.0f) continue;
          const float tau = tx_arrival(t, px, py, pz, a.c);
          float tc = 1.0f, ts = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
          const long trace0 = (static_cast<long>(ev) * a.n_ch + g) * a.n_smp;
#pragma unroll
          for (int k = 0; k < kGroup; ++k) {
            if (ap[k] <= 0.0f) continue;
            const float idx = (tau + rt[k] - a.t0) * a.fs;
            const int kk = static_cast<int>(floorf(idx));
            const float wt = ap[k] * tw;
            if (IQ) {
              cplx v = mk(0.f, 0.f);
              if (kk >= 0 && kk + 1 < a.n_smp) {
                const float f = idx - static_cast<float>(kk);
                const float2* tr = iq + trace0 + static_cast<long>(k) * a.n_smp;
                const float2 s0 = __ldg(tr + kk), s1 = __ldg(tr + kk + 1);
                const float w0 = 1.0f - f;
                v = mk(s0.x * w0 + s1.x * f, s0.y * w0 + s1.y * f);
              }
              const cplx rot = mk(tc * rc[k] - ts * rs[k], ts * rc[k] + tc * rs[k]);
              Y[k] = cadd(Y[k], cscale(cmul(v, rot), wt));
            } else {
              float v = 0.0f;
              if (kk >= 0 && kk + 1 < a.n_smp) {
                const float f = idx - static_cast<float>(kk);
                const float* tr = rf + trace0 + static_cast<long>(k) * a.n_smp;
                v = __ldg(tr + kk) * (1.0f - f) + __ldg(tr + kk + 1) * f;
              }
              Y[k] = cadd(Y[k], mk(v * wt, 0.0f * wt));
            }
          }
        }
      }

      // Combine the finished channels of this group in ascending order.
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        const int ch = g + k;
        if (ch >= a.n_ch) break;
        const bool act = ap[k] > 0.0f;
        const cplx y = act ? Y[k] : mk(0.f, 0.f);
        if (a.is_mv) {
          a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = make_float2(y.re, y.im);
          continue;
        }
        n_active += act ? 1 : 0;
        if (a.combiner == USX_COMB_DMAS) {
          const float m = cabsf_(y);
          if (m > 0.0f) {
            const cplx v = cdivr(y, sqrtf(m));
            s = cadd(s, v);
            q = cadd(q, cmul(v, v));
          }
        } else {
          das = cadd(das, y);
        }
        if (a.cf && act) {
          coh = cadd(coh, y);
          incs += cnorm(y);
        }
      }
    }
    if (a.is_mv) continue;

    cplx out;
    if (n_active == 0) {
      out = mk(0.f, 0.f);
      if (incoherent) continue;
    } else if (a.combiner == USX_COMB_DMAS) {
      const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
      const float norm = 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1));
      out = cdivr(acc, norm);
    } else {
      out = das;
    }
    if (a.cf && n_active > 0)
      out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
    if (incoherent)
      inc_acc += cnorm(out);
    else
      result = out;
  }
  if (a.is_mv) return;
  if (incoherent) result = mk(sqrtf(inc_acc), 0.0f);
  a.out[frame * a.out_stride + pix] = make_float2(result.re, result.im);
}


// ------------------------------------------------------------------------
// das_fast_kernel: the default beamformer (USX_BF_FAST).
//
// Same delay indices and phase arguments as the reference, bit for bit (an
// error of one ulp in a sample index near 2000 moves the interpolation by
// 1e-4 samples, which on speckle is a 5e-5 relative error, so these chains
// are kept in the reference's order without contraction). Everything else
// is rearranged for throughput:
//   * the receive phasor and aperture weight do not depend on the event and
//     are applied once per channel after the event sum,
//     y_ch = (a e^{j th_rx}) * sum_ev (tw e^{j th_tx}) lerp(IQ, idx);
//   * the interpolation and the complex accumulation use FMA;
//   * 16 channels per group share each event's geometry (illumination,
//     transmit delay, transmit phasor);
//   * a block is a 4-line x 32-depth tile, so the four warps read
//     overlapping windows of every trace and share them in L1.
// The result differs from the reference's rounding by ~1e-7 relative L2.
//
// The group size G, the tile's line count TL (a CTA is TL warps), the
// register cap (MINB resident CTAs per SM) and the warp's shape within the
// tile (kWarpLines lines x 32 / kWarpLines depths: a warp spanning several
// lines and fewer depths gathers from a narrower window of each trace, the
// transmit-plus-receive delay changing less across lines than along depth)
// are template parameters; every variant computes the same sums in the same
// order (bit-identical frames), and the plan's autotuner picks the fastest
// for its geometry.
// One CTA tile (`tile` of frame `frame`) of the plan `a`: the body of
// das_fast_kernel, also run by das_queue_kernel for the tiles of many plans.
// rt_s: kRtShared's per-thread receive delays in shared memory.
template <bool IQ, int kFastGroup, int kTileLines, bool kRtShared, int kWarpLines, bool kDeepFirst>
__device__ __forceinline__ void das_fast_tile(const BfArgs& a, int tile, long frame, float* rt_s) {
  static_assert(kTileLines % kWarpLines == 0 && 32 % kWarpLines == 0, "warp shape must tile the CTA");
  const int n0 = a.n_pix / a.n1;
  const int tiles_depth = (a.n1 + 31) / 32;
  constexpr int kWarpDepths = 32 / kWarpLines;
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  // Tile order. Default: depth tiles of a group of lines, then the next lines.
  // kDeepFirst: every line group's deepest depth tile first, the shallowest
  // last. A pixel's work grows with depth (the aperture widens as z / F#), so
  // the CTAs dispatched last, which form the tail of the grid, are the
  // lightest (longest-processing-time-first order). Both orders visit each of
  // the n_line_tiles x tiles_depth tiles once.
  const int n_line_tiles = (n0 + kTileLines - 1) / kTileLines;
  const int line_tile = kDeepFirst ? tile % n_line_tiles : tile / tiles_depth;
  const int depth_tile = kDeepFirst ? tiles_depth - 1 - tile / n_line_tiles : tile % tiles_depth;
  const int line = line_tile * kTileLines + (w / kWarpLines) * kWarpLines + ln / kWarpDepths;
  const int depth = depth_tile * 32 + (w % kWarpLines) * kWarpDepths + ln % kWarpDepths;
  if (line >= n0 || depth >= a.n1) return;
  const int pix = line * a.n1 + depth;
  const float px = __ldg(a.points + 3 * pix), py = __ldg(a.points + 3 * pix + 1),
              pz = __ldg(a.points + 3 * pix + 2);
  int ev_first = a.ev_begin, ev_last = a.ev_end;
  if (a.seq_epf > 0) {
    ev_first = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_last = ev_first + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_first += a.pass;
    ev_last = ev_first + 1;
  }
  const bool incoherent = a.compounding == USX_COMP_INCOHERENT && a.pass < 0;
  const bool select = a.compounding == USX_COMP_SELECT;
  int best_ev = -1;
  float best_w = 0.0f;
  if (select) {
    for (int ev = ev_first; ev < ev_last; ++ev) {
      const float tw = tx_sensitivity_fast(a.tx[ev], px, pz, a.lambda);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }
  const float2* iq = IQ ? a.iq + frame * a.data_stride : nullptr;
  const float* rf = IQ ? nullptr : a.rf + frame * a.data_stride;
  const int n_pass = incoherent ? (ev_last - ev_first) : 1;
  float inc_acc = 0.0f;
  cplx result = mk(0.f, 0.f);
  const unsigned n_last = static_cast<unsigned>(a.n_smp - 1);

  for (int pass = 0; pass < max(1, n_pass); ++pass) {
    const int ev_lo = incoherent ? ev_first + pass : ev_first;
    const int ev_hi = incoherent ? ev_lo + 1 : ev_last;
    cplx das = mk(0.f, 0.f), s = mk(0.f, 0.f), q = mk(0.f, 0.f), coh = mk(0.f, 0.f);
    float incs = 0.0f;
    int n_active = 0;
    for (int g = 0; g < a.n_ch; g += kFastGroup) {
      float rt_r[kRtShared ? 1 : kFastGroup];
      float* rt = kRtShared ? rt_s + threadIdx.x * kFastGroup : rt_r;
      unsigned mask = 0u;
#pragma unroll
      for (int k = 0; k < kFastGroup; ++k) {
        const int ch = g + k;
        rt[k] = 0.0f;
        if (ch < a.n_ch) {
          const float ex = elem_x(a, ch);
          if (aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f) {
            mask |= 1u << k;
            rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
          }
        }
      }
      float ar[kFastGroup], ai[kFastGroup];
#pragma unroll
      for (int k = 0; k < kFastGroup; ++k) ar[k] = ai[k] = 0.0f;
      if (mask) {
        for (int ev = ev_lo; ev < ev_hi; ++ev) {
          const TxDev& t = a.tx[ev];
          float tw;
          if (select) {
            tw = (best_ev == ev && best_w > 0.0f) ? 1.0f : 0.0f;
          } else if (a.tx_weighting) {
            tw = tx_sensitivity_fast(t, px, pz, a.lambda);
          } else {
            tw = 1.0f;
          }
          if (tw <= 0.0f) continue;
          const float tau = tx_arrival(t, px, py, pz, a.c);
          float tc = 1.0f, ts = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
          const float wr = tw * tc, wi = tw * ts;
          const long trace0 = (static_cast<long>(ev) * a.n_ch + g) * a.n_smp;
#pragma unroll
          for (int k = 0; k < kFastGroup; ++k) {
            if (!(mask & (1u << k))) continue;
            const float idx = (tau + rt[k] - a.t0) * a.fs;
            const float fl = floorf(idx);
            const int kk = static_cast<int>(fl);
            if (static_cast<unsigned>(kk) >= n_last) continue;
            const float f = idx - fl;
            if (IQ) {
              const float2* tr = iq + trace0 + static_cast<long>(k) * a.n_smp + kk;
              const float2 s0 = __ldg(tr), s1 = __ldg(tr + 1);
              const float vr = fmaf(f, s1.x - s0.x, s0.x);
              const float vi = fmaf(f, s1.y - s0.y, s0.y);
              ar[k] = fmaf(wr, vr, fmaf(-wi, vi, ar[k]));
              ai[k] = fmaf(wr, vi, fmaf(wi, vr, ai[k]));
            } else {
              const float* tr = rf + trace0 + static_cast<long>(k) * a.n_smp + kk;
              const float s0 = __ldg(tr), s1 = __ldg(tr + 1);
              ar[k] = fmaf(wr, fmaf(f, s1 - s0, s0), ar[k]);
            }
          }
        }
      }
      // Apply each channel's aperture weight and receive phasor, combine in order.
#pragma unroll
      for (int k = 0; k < kFastGroup; ++k) {
        const int ch = g + k;
        if (ch >= a.n_ch) break;
        const bool act = (mask >> k) & 1u;
        cplx y = mk(0.f, 0.f);
        if (act) {
          const float w = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha);
          const float ap = a.is_mv ? 1.0f : w;
          float rc = 1.0f, rs = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
          const float gr = ap * rc, gi = ap * rs;
          y = mk(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
        }
        if (a.is_mv) {
          a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = make_float2(y.re, y.im);
          continue;
        }
        n_active += act ? 1 : 0;
        if (a.combiner == USX_COMB_DMAS) {
          const float m = cabsf_(y);
          if (m > 0.0f) {
            const cplx v = cdivr(y, sqrtf(m));
            s = cadd(s, v);
            q = cadd(q, cmul(v, v));
          }
        } else {
          das = cadd(das, y);
        }
        if (a.cf && act) {
          coh = cadd(coh, y);
          incs += cnorm(y);
        }
      }
    }
    if (a.is_mv) continue;
    cplx out;
    if (n_active == 0) {
      out = mk(0.f, 0.f);
      if (incoherent) continue;
    } else if (a.combiner == USX_COMB_DMAS) {
      const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
      out = cdivr(acc, 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1)));
    } else {
      out = das;
    }
    if (a.cf && n_active > 0)
      out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
    if (incoherent)
      inc_acc += cnorm(out);
    else
      result = out;
  }
  if (a.is_mv) return;
  if (incoherent) result = mk(sqrtf(inc_acc), 0.0f);
  a.out[frame * a.out_stride + pix] = make_float2(result.re, result.im);
}

template <bool IQ, int kFastGroup, int kTileLines, int MINB, bool kRtShared = false, int kWarpLines = 1,
          bool kDeepFirst = false>
__global__ void __launch_bounds__(32 * kTileLines, MINB) das_fast_kernel(const BfArgs a) {
  // kRtShared: the group's receive delays live in shared memory instead of
  // registers, so that a larger group fits the register cap.
  __shared__ float rt_s[kRtShared ? 32 * kTileLines * kFastGroup : 1];
  das_fast_tile<IQ, kFastGroup, kTileLines, kRtShared, kWarpLines, kDeepFirst>(a, blockIdx.x, blockIdx.y, rt_s);
}

// ------------------------------------------------------------------------
// das_export_kernel: the minimum-variance export (compounded channel samples
// y[frame][pixel][channel]) with the transmit side tabulated per pixel. A
// CTA is kPW pixel warps x kCQ channel warps: the tile is kPW x 32 pixels
// (das_fast_kernel's tile: kPW lines x 32 depths, warps of kWL lines x 32 /
// kWL depths), and channel warp cq takes channels cq, cq + kCQ, ... in groups
// of kG, so the kPW pixel warps that share a channel read the same trace
// windows through L1. Per pass (one group of kG channels per channel warp)
// the events go in chunks of kExpEv: the CTA first tabulates (transmit delay,
// weighted transmit phasor, illumination weight) for its pixels and the
// chunk's events, each thread for its own pixel, then every thread runs its
// kG channels over the chunk. The transmit side is evaluated once per pixel,
// event and pass instead of once per channel group; the per-channel sums are
// das_fast_kernel's expressions in the same order, so the exported samples
// are the same bit for bit.
// das_csum_kernel is the same body for the plain sums (delay-and-sum, DMAS,
// coherence factor): after each pass the channel warps stage their channel
// values in the table's shared memory and channel warp 0's thread of each
// pixel combines the pass's channels in ascending order, exactly as
// das_fast_kernel's channel loop, so its frames are the same bit for bit;
// the combine state lives in shared memory between passes. At 128 channels,
// 75 plane waves, 512 x 1024: 4.20 ms per frame against 4.97 for
// das_fast_kernel's best shape (three CTAs per SM; two, at 64 registers,
// measured 5.6). Warps of 2 or 1 lines (x 16 or 32 depths) instead of 4:
// 4.26 and 4.34 ms; 2 pixel warps x 8 channel warps (32 channels per pass,
// half the passes and tables, half the pixel warps sharing a trace): 4.43.
// Measured on the learned frame (128 ch, 75 plane waves, 512 x 1024): export
// 4.83 ms with (kG, kPW, kCQ, kWL) = (4, 4, 4, 4) against 5.08 for
// das_fast_kernel's best shape; (8, 4, 4, 4) 5.1, (8, 4, 4, 1) 5.6,
// (8, 4, 2, 4) 5.3. The gathers' latency, not the transmit terms, bounds it.
// Skipping the passes outside every pixel's aperture: 4.83 -> 4.38 ms; the
// deepest tiles first: 4.38 -> 4.13 ms; chunks of 32 events instead of 16
// (half the table barriers, the table in 64 KB of dynamic shared memory):
// 4.13 -> 4.10 ms, and 4.21 -> 4.18 ms for das_csum_kernel.
constexpr int kExpEv = 32;
// Dynamic shared memory of the channel-warp kernels (the transmit table).
__host__ __device__ constexpr size_t exp_table_bytes(int pixel_warps) {
  return sizeof(float4) * kExpEv * 32 * pixel_warps;
}

template <int kG, int kPW, int kCQ, int kWL, bool kSum>
__device__ __forceinline__ void das_export_body(const BfArgs& a, int tile, long frame) {
  static_assert(32 % kWL == 0 && kPW % kWL == 0, "warp shape must tile the CTA");
  static_assert(sizeof(float2) * kCQ * kG <= sizeof(float4) * kExpEv, "a pass's channel values fit the table");
  extern __shared__ float4 das_exp_smem[];
  float4 (*tab)[32 * kPW] = reinterpret_cast<float4 (*)[32 * kPW]>(das_exp_smem);   // [kExpEv][pixel slot]
  // kSum: a pass's channel values [channel of the pass][pixel slot] in the
  // table's space once the pass's events are done, and each channel warp's
  // aperture mask per pixel.
  __shared__ unsigned act_s[kSum ? kCQ : 1][32 * kPW];
  // kSum: each pixel's combine state (das, s, q, coh, incs, n_active), kept
  // in shared memory rather than in registers through the event loops.
  __shared__ float cs[kSum ? 10 : 1][32 * kPW];
  float2* ys = reinterpret_cast<float2*>(das_exp_smem);
  constexpr int kWD = 32 / kWL;
  const int n0 = a.n_pix / a.n1;
  const int tiles_depth = (a.n1 + 31) / 32;
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31;
  const int pw = w % kPW, cq = w / kPW;
  const int pl = pw * 32 + ln;   // pixel slot in the tile
  // Deepest depth tiles first: the aperture, and with it a tile's active
  // passes, grows with depth, so the last CTAs of the grid are the lightest.
  const int n_line_tiles = (n0 + kPW - 1) / kPW;
  const int line_tile = tile % n_line_tiles, depth_tile = tiles_depth - 1 - tile / n_line_tiles;
  const int line = line_tile * kPW + (pw / kWL) * kWL + ln / kWD;
  const int depth = depth_tile * 32 + (pw % kWL) * kWD + ln % kWD;
  const bool valid = line < n0 && depth < a.n1;
  const int pix = valid ? line * a.n1 + depth : 0;
  const float px = __ldg(a.points + 3 * pix), py = __ldg(a.points + 3 * pix + 1), pz = __ldg(a.points + 3 * pix + 2);
  int ev_lo = a.ev_begin, ev_hi = a.ev_end;
  if (a.seq_epf > 0) {
    ev_lo = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_hi = ev_lo + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_lo += a.pass;
    ev_hi = ev_lo + 1;
  }
  const bool select = a.compounding == USX_COMP_SELECT;
  int best_ev = -1;
  float best_w = 0.0f;
  if (select && valid) {
    for (int ev = ev_lo; ev < ev_hi; ++ev) {
      const float tw = tx_sensitivity_fast(a.tx[ev], px, pz, a.lambda);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }
  const float2* iq = a.iq + frame * a.data_stride;
  const unsigned n_last = static_cast<unsigned>(a.n_smp - 1);
  const int n_groups = (a.n_ch + kG - 1) / kG;
  const int n_pass = (n_groups + kCQ - 1) / kCQ;
  // kSum: the channel combine of das_fast_tile, run by channel warp 0's
  // thread of each pixel over the channels in ascending order.
  if (kSum && cq == 0)
#pragma unroll
    for (int i = 0; i < 10; ++i) cs[i][pl] = 0.0f;
  for (int pass = 0; pass < n_pass; ++pass) {
    const int grp = pass * kCQ + cq;
    const int g = grp * kG;
    float rt[kG];
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < kG; ++k) {
      const int ch = g + k;
      rt[k] = 0.0f;
      if (valid && ch < a.n_ch) {
        const float ex = elem_x(a, ch);
        if (aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f) {
          mask |= 1u << k;
          rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
        }
      }
    }
    float ar[kG], ai[kG];
#pragma unroll
    for (int k = 0; k < kG; ++k) ar[k] = ai[k] = 0.0f;
    // A pass whose kCQ x kG channels are outside every pixel's aperture (the
    // shallow tiles') skips the transmit table and the events; its samples
    // are written as zeros below.
    const int c_end = __syncthreads_or(mask != 0u) ? ev_hi : ev_lo;
    for (int c0 = ev_lo; c0 < c_end; c0 += kExpEv) {
      const int c1 = min(c_end, c0 + kExpEv);
      // The chunk's table: (tau, tw cos, tw sin, tw) for this thread's pixel.
      __syncthreads();
      for (int e = c0 + cq; e < c1; e += kCQ) {
        const TxDev& t = a.tx[e];
        float tw;
        if (!valid)
          tw = 0.0f;
        else if (select)
          tw = (best_ev == e && best_w > 0.0f) ? 1.0f : 0.0f;
        else if (a.tx_weighting)
          tw = tx_sensitivity_fast(t, px, pz, a.lambda);
        else
          tw = 1.0f;
        float4 ent = make_float4(0.f, 0.f, 0.f, tw);
        if (tw > 0.0f) {
          const float tau = tx_arrival(t, px, py, pz, a.c);
          float tc = 1.0f, ts = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
          ent = make_float4(tau, tw * tc, tw * ts, tw);
        }
        tab[e - c0][pl] = ent;
      }
      __syncthreads();
      if (!mask) continue;
      for (int e = c0; e < c1; ++e) {
        const float4 ent = tab[e - c0][pl];
        if (ent.w <= 0.0f) continue;
        const float tau = ent.x, wr = ent.y, wi = ent.z;
        const float2* trace = iq + (static_cast<long>(e) * a.n_ch + g) * a.n_smp;
#pragma unroll
        for (int k = 0; k < kG; ++k) {
          if (!(mask & (1u << k))) continue;
          const float idx = (tau + rt[k] - a.t0) * a.fs;
          const float fl = floorf(idx);
          const int kk = static_cast<int>(fl);
          if (static_cast<unsigned>(kk) >= n_last) continue;
          const float f = idx - fl;
          const float2* tr = trace + static_cast<long>(k) * a.n_smp + kk;
          const float2 s0 = __ldg(tr), s1 = __ldg(tr + 1);
          const float vr = fmaf(f, s1.x - s0.x, s0.x);
          const float vi = fmaf(f, s1.y - s0.y, s0.y);
          ar[k] = fmaf(wr, vr, fmaf(-wi, vi, ar[k]));
          ai[k] = fmaf(wr, vi, fmaf(wi, vr, ai[k]));
        }
      }
    }
    if (kSum) {
      __syncthreads();   // the table is read for the last time
#pragma unroll
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        float2 y = make_float2(0.f, 0.f);
        if ((mask >> k) & 1u) {
          const float ap = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha);
          float rc = 1.0f, rs = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
          const float gr = ap * rc, gi = ap * rs;
          y = make_float2(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
        }
        ys[(cq * kG + k) * (32 * kPW) + pl] = y;
      }
      act_s[cq][pl] = mask;
      __syncthreads();
      // (The next pass's __syncthreads_or keeps the table's writers out of
      // these values until the combine is done.)
      if (cq == 0 && valid) {
        cplx das = mk(cs[0][pl], cs[1][pl]), s = mk(cs[2][pl], cs[3][pl]), q = mk(cs[4][pl], cs[5][pl]),
             coh = mk(cs[6][pl], cs[7][pl]);
        float incs = cs[8][pl];
        int n_active = __float_as_int(cs[9][pl]);
        for (int c = 0; c < kCQ * kG; ++c) {
          const int ch = pass * kCQ * kG + c;
          if (ch >= a.n_ch) break;
          const bool act = (act_s[c / kG][pl] >> (c % kG)) & 1u;
          const float2 yv = ys[c * (32 * kPW) + pl];
          const cplx y = mk(yv.x, yv.y);
          n_active += act ? 1 : 0;
          if (a.combiner == USX_COMB_DMAS) {
            const float m = cabsf_(y);
            if (m > 0.0f) {
              const cplx v = cdivr(y, sqrtf(m));
              s = cadd(s, v);
              q = cadd(q, cmul(v, v));
            }
          } else {
            das = cadd(das, y);
          }
          if (a.cf && act) {
            coh = cadd(coh, y);
            incs += cnorm(y);
          }
        }
        cs[0][pl] = das.re;
        cs[1][pl] = das.im;
        cs[2][pl] = s.re;
        cs[3][pl] = s.im;
        cs[4][pl] = q.re;
        cs[5][pl] = q.im;
        cs[6][pl] = coh.re;
        cs[7][pl] = coh.im;
        cs[8][pl] = incs;
        cs[9][pl] = __int_as_float(n_active);
      }
      continue;
    }
    if (!valid) continue;
#pragma unroll
    for (int k = 0; k < kG; ++k) {
      const int ch = g + k;
      if (ch >= a.n_ch) break;
      const bool act = (mask >> k) & 1u;
      float2 y = make_float2(0.f, 0.f);
      if (act) {
        float rc = 1.0f, rs = 0.0f;
        if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
        const float gr = 1.0f * rc, gi = 1.0f * rs;   // the export carries no aperture weight
        y = make_float2(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
      }
      a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = y;
    }
  }
  if (kSum && cq == 0 && valid) {
    const cplx das = mk(cs[0][pl], cs[1][pl]), s = mk(cs[2][pl], cs[3][pl]), q = mk(cs[4][pl], cs[5][pl]),
               coh = mk(cs[6][pl], cs[7][pl]);
    const float incs = cs[8][pl];
    const int n_active = __float_as_int(cs[9][pl]);
    cplx out;
    if (n_active == 0) {
      out = mk(0.f, 0.f);
    } else if (a.combiner == USX_COMB_DMAS) {
      const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
      out = cdivr(acc, 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1)));
    } else {
      out = das;
    }
    if (a.cf && n_active > 0)
      out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
    a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
  }
}

template <int kG, int kPW, int kCQ, int kWL>
__global__ void __launch_bounds__(32 * kPW * kCQ) das_export_kernel(const BfArgs a) {
  das_export_body<kG, kPW, kCQ, kWL, false>(a, blockIdx.x, blockIdx.y);
}
// The channel-combining instance (delay-and-sum, DMAS, coherence factor):
// three CTAs per SM, as the export's fastest shape runs.
template <int kG, int kPW, int kCQ, int kWL>
__global__ void __launch_bounds__(32 * kPW * kCQ, 3) das_csum_kernel(const BfArgs a) {
  das_export_body<kG, kPW, kCQ, kWL, true>(a, blockIdx.x, blockIdx.y);
}

// ------------------------------------------------------------------------
// das_queue_kernel: frames of many plans (any probe, grid, transmit set and
// plain combiner) in one persistent launch. Each CTA takes the next tile
// from a device counter, finds its (plan, frame) from the entries' tile
// prefix, and runs das_fast_tile with that plan's arguments (kernel
// parameters, indexed by entry). Tiles of every entry are the same as in the
// plan's own launch, so each frame equals its plan's execution bit for bit.
constexpr int kQueueMax = 48;

struct DasQueueArgs {
  BfArgs args[kQueueMax];
  int tiles[kQueueMax];        // tiles per frame
  int first[kQueueMax + 1];    // first work item of each entry (tiles x frames)
  int n;
  unsigned* next;              // work counter (zero at launch)
};

template <bool IQ, int kFastGroup, int kTileLines, int MINB, bool kRtShared = false, int kWarpLines = 1,
          bool kDeepFirst = false>
__global__ void __launch_bounds__(32 * kTileLines, MINB) das_queue_kernel(const DasQueueArgs q) {
  __shared__ float rt_s[kRtShared ? 32 * kTileLines * kFastGroup : 1];
  __shared__ int s_item;
  const int total = q.first[q.n];
  for (;;) {
    if (threadIdx.x == 0) s_item = static_cast<int>(atomicAdd(q.next, 1u));
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= total) break;
    int e = 0;
    while (e + 1 < q.n && item >= q.first[e + 1]) ++e;
    const int local = item - q.first[e];
    const int frame = local / q.tiles[e], tile = local - frame * q.tiles[e];
    das_fast_tile<IQ, kFastGroup, kTileLines, kRtShared, kWarpLines, kDeepFirst>(q.args[e], tile, frame, rt_s);
  }
}

// The same queue over das_csum_kernel's body (IQ plans): CTAs of 4 pixel
// warps x 4 channel warps on the same 4-line x 32-depth tiles.
__global__ void __launch_bounds__(512, 3) das_csum_queue_kernel(const DasQueueArgs q) {
  __shared__ int s_item;
  const int total = q.first[q.n];
  for (;;) {
    if (threadIdx.x == 0) s_item = static_cast<int>(atomicAdd(q.next, 1u));
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= total) break;
    int e = 0;
    while (e + 1 < q.n && item >= q.first[e + 1]) ++e;
    const int local = item - q.first[e];
    const int frame = local / q.tiles[e], tile = local - frame * q.tiles[e];
    das_export_body<4, 4, 4, 4, true>(q.args[e], tile, frame);
  }
}

// ------------------------------------------------------------------------
// das_table_kernel: the fast delay-and-sum with the transmit side computed
// once per (pixel, event). A CTA is 32 pixels (kWL lines x 32 / kWL depths,
// one per lane) and one warp per group of G channels (all warps share the
// lanes' pixels). For each chunk of events the warps first fill a table of
// (transmit delay, weighted transmit phasor, illumination weight) for the 32
// pixels in shared memory, each warp its share of the events; then every
// warp runs its channels over the chunk's events, reading one table entry per
// event instead of evaluating the illumination weight, the transmit delay and
// its phasor once per channel group as das_fast_kernel does. The per-channel
// sums, the receive phasor and aperture weight are das_fast_kernel's
// expressions in the same order, so the per-channel values are the same bit
// for bit; they are staged in shared memory [pixel][channel] and either
// written out as rows (the minimum-variance export: 32 contiguous rows of
// n_ch samples instead of one sample per pixel and channel) or combined by
// the first warp, channel by channel in ascending order as das_fast_kernel
// does. IQ data, coherent and select compounding, n_ch <= 256.
// Measured at 128 channels, 75 plane waves, 512 x 1024 (ms per frame against
// 4.98 for das_fast_kernel's best shape): G = 8 with 1, 2, 4 lines per CTA
// and two CTAs per SM 8.63, 8.39, 8.29; G = 8, three CTAs 7.87; G = 4, one
// CTA of 32 warps 9.21; G = 4, two CTAs (64 warps per SM) 6.06. The warps of a
// CTA read different traces, so none of the L1 reuse that das_fast_kernel's
// warps get from sharing each trace window remains, and the gathers' latency
// outweighs the transmit work saved. G = 4 with two CTAs stays a candidate.
constexpr int kTableEv = 32;    // events per table chunk (16 KB)
constexpr int kTableMaxCh = 256;

__host__ __device__ inline int table_warps(int group, int n_ch) {
  const int cap = group >= 8 ? 16 : 32;
  const int need = (n_ch + group - 1) / group;
  return need < cap ? need : cap;
}
__host__ __device__ inline size_t table_stage_off() { return sizeof(float4) * kTableEv * 32; }
__host__ __device__ inline size_t table_smem_bytes(int n_ch) {
  return table_stage_off() + sizeof(float2) * 33 * n_ch + 32 * n_ch;
}

template <int G, int kWL, int MINB>
__global__ void __launch_bounds__(32 * (G >= 8 ? 16 : 32), MINB) das_table_kernel(const BfArgs a) {
  extern __shared__ float4 table_smem[];
  float4* tab = table_smem;                                                    // [event in chunk][lane]
  // Staged channel values [channel][33] (one pad column: rows of a pixel read
  // along channels stay conflict-free) and active flags [channel][32].
  float2* ys = reinterpret_cast<float2*>(reinterpret_cast<char*>(table_smem) + table_stage_off());
  unsigned char* act_s = reinterpret_cast<unsigned char*>(ys + 33 * a.n_ch);
  constexpr int kWD = 32 / kWL;
  const int n0 = a.n_pix / a.n1;
  const int tiles_depth = (a.n1 + kWD - 1) / kWD;
  const int w = threadIdx.x >> 5, ln = threadIdx.x & 31, n_warps = blockDim.x >> 5;
  const long frame = blockIdx.y;
  const int line = (static_cast<int>(blockIdx.x) / tiles_depth) * kWL + ln / kWD;
  const int depth = (static_cast<int>(blockIdx.x) % tiles_depth) * kWD + ln % kWD;
  const bool valid = line < n0 && depth < a.n1;
  const int pix = valid ? line * a.n1 + depth : 0;
  const float px = __ldg(a.points + 3 * pix), py = __ldg(a.points + 3 * pix + 1), pz = __ldg(a.points + 3 * pix + 2);
  int ev_lo = a.ev_begin, ev_hi = a.ev_end;
  if (a.seq_epf > 0) {
    ev_lo = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_hi = ev_lo + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_lo += a.pass;
    ev_hi = ev_lo + 1;
  }
  const bool select = a.compounding == USX_COMP_SELECT;
  int best_ev = -1;
  float best_w = 0.0f;
  if (select) {
    for (int ev = ev_lo; ev < ev_hi; ++ev) {
      const float tw = tx_sensitivity_fast(a.tx[ev], px, pz, a.lambda);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }
  const float2* iq = a.iq + frame * a.data_stride;
  const unsigned n_last = static_cast<unsigned>(a.n_smp - 1);
  const int ch_stride = G * n_warps;
  const bool one_chunk = ev_hi - ev_lo <= kTableEv;

  for (int g = G * w, g_first = 0; g_first < a.n_ch; g += ch_stride, g_first += ch_stride) {
    float rt[G];
    unsigned mask = 0u;
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const int ch = g + k;
      rt[k] = 0.0f;
      if (valid && ch < a.n_ch) {
        const float ex = elem_x(a, ch);
        if (aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f) {
          mask |= 1u << k;
          rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
        }
      }
    }
    float ar[G], ai[G];
#pragma unroll
    for (int k = 0; k < G; ++k) ar[k] = ai[k] = 0.0f;
    for (int c0 = ev_lo; c0 < ev_hi; c0 += kTableEv) {
      const int c1 = min(ev_hi, c0 + kTableEv);
      if (g_first == 0 || !one_chunk) {
        // The chunk's table: (tau, tw cos, tw sin, tw) for this lane's pixel.
        __syncthreads();
        for (int e = c0 + w; e < c1; e += n_warps) {
          const TxDev& t = a.tx[e];
          float tw;
          if (select)
            tw = (best_ev == e && best_w > 0.0f) ? 1.0f : 0.0f;
          else if (a.tx_weighting)
            tw = tx_sensitivity_fast(t, px, pz, a.lambda);
          else
            tw = 1.0f;
          float4 ent = make_float4(0.f, 0.f, 0.f, tw);
          if (tw > 0.0f) {
            const float tau = tx_arrival(t, px, py, pz, a.c);
            float tc = 1.0f, ts = 0.0f;
            if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
            ent = make_float4(tau, tw * tc, tw * ts, tw);
          }
          tab[(e - c0) * 32 + ln] = ent;
        }
        __syncthreads();
      }
      if (!mask) continue;
      for (int e = c0; e < c1; ++e) {
        const float4 ent = tab[(e - c0) * 32 + ln];
        if (ent.w <= 0.0f) continue;
        const float tau = ent.x, wr = ent.y, wi = ent.z;
        const float2* trace = iq + (static_cast<long>(e) * a.n_ch + g) * a.n_smp;
#pragma unroll
        for (int k = 0; k < G; ++k) {
          if (!(mask & (1u << k))) continue;
          const float idx = (tau + rt[k] - a.t0) * a.fs;
          const float fl = floorf(idx);
          const int kk = static_cast<int>(fl);
          if (static_cast<unsigned>(kk) >= n_last) continue;
          const float f = idx - fl;
          const float2* tr = trace + static_cast<long>(k) * a.n_smp + kk;
          const float2 s0 = __ldg(tr), s1 = __ldg(tr + 1);
          const float vr = fmaf(f, s1.x - s0.x, s0.x);
          const float vi = fmaf(f, s1.y - s0.y, s0.y);
          ar[k] = fmaf(wr, vr, fmaf(-wi, vi, ar[k]));
          ai[k] = fmaf(wr, vi, fmaf(wi, vr, ai[k]));
        }
      }
    }
    // Each channel's aperture weight and receive phasor; staged per pixel.
#pragma unroll
    for (int k = 0; k < G; ++k) {
      const int ch = g + k;
      if (ch >= a.n_ch) break;
      const bool act = (mask >> k) & 1u;
      float2 y = make_float2(0.f, 0.f);
      if (act) {
        const float wt = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha);
        const float ap = a.is_mv ? 1.0f : wt;
        float rc = 1.0f, rs = 0.0f;
        if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
        const float gr = ap * rc, gi = ap * rs;
        y = make_float2(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
      }
      ys[ch * 33 + ln] = y;
      act_s[ch * 32 + ln] = act ? 1 : 0;
    }
  }
  __syncthreads();
  if (a.is_mv) {
    // 32 rows of n_ch samples, written by the whole CTA.
    for (int i = threadIdx.x; i < 32 * a.n_ch; i += blockDim.x) {
      const int p = i / a.n_ch, ch = i - p * a.n_ch;
      const int pl = (static_cast<int>(blockIdx.x) / tiles_depth) * kWL + p / kWD;
      const int pd = (static_cast<int>(blockIdx.x) % tiles_depth) * kWD + p % kWD;
      if (pl < n0 && pd < a.n1)
        a.y_out[(frame * a.n_pix + static_cast<long>(pl) * a.n1 + pd) * a.n_ch + ch] = ys[ch * 33 + p];
    }
    return;
  }
  if (w != 0 || !valid) return;
  cplx das = mk(0.f, 0.f), s = mk(0.f, 0.f), q = mk(0.f, 0.f), coh = mk(0.f, 0.f);
  float incs = 0.0f;
  int n_active = 0;
  for (int ch = 0; ch < a.n_ch; ++ch) {
    const float2 yv = ys[ch * 33 + ln];
    const cplx y = mk(yv.x, yv.y);
    const bool act = act_s[ch * 32 + ln] != 0;
    n_active += act ? 1 : 0;
    if (a.combiner == USX_COMB_DMAS) {
      const float m = cabsf_(y);
      if (m > 0.0f) {
        const cplx v = cdivr(y, sqrtf(m));
        s = cadd(s, v);
        q = cadd(q, cmul(v, v));
      }
    } else {
      das = cadd(das, y);
    }
    if (a.cf && act) {
      coh = cadd(coh, y);
      incs += cnorm(y);
    }
  }
  cplx out;
  if (n_active == 0) {
    out = mk(0.f, 0.f);
  } else if (a.combiner == USX_COMB_DMAS) {
    const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
    out = cdivr(acc, 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1)));
  } else {
    out = das;
  }
  if (a.cf && n_active > 0)
    out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
  a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
}

// ------------------------------------------------------------------------
// das_staged_kernel: the fast delay-and-sum with the IQ windows of every
// (channel group, kE transmits) step staged in shared memory by the tensor
// memory accelerator (cp.async.bulk, one 1-D bulk copy per channel row,
// completion on an mbarrier), double-buffered so that step i+1's copies fly
// while step i is computed. At 128 channels and 75 plane waves it measured
// 14.7 ms per 512 x 1024 frame with one transmit per step and 21-22 ms with
// four or five, against 6.0 ms for das_fast_kernel's L1 gathers (the
// per-step barrier and the single issuing thread serialise the CTA); it stays
// one of the autotuner's candidates. Plane waves only: the window of a channel over the CTA's tile
// is bounded from the tile's pixel extent (the transmit delay is linear in x
// and z; the receive delay is smallest at the tile point nearest the element
// and largest at the farthest corner). The per-pixel delay index is the
// reference's, bit for bit, as in das_fast_kernel; a pixel whose samples fall
// outside the staged window (rounding at the window's edge, an unusually
// wide tile) reads them from global memory, so the frame is identical to
// das_fast_kernel's. Coherent and select compounding.
constexpr int kStageW = 64;   // staged samples per channel row (512 bytes)

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

template <int kG, int kTL, int kE>
__global__ void __launch_bounds__(32 * kTL) das_staged_kernel(const BfArgs a) {
  // A step is one channel group and kE consecutive transmits.
  __shared__ __align__(16) float2 win[2][kE][kG][kStageW];
  __shared__ __align__(8) uint64_t bar[2];
  __shared__ int s_lo[2][kE][kG];
  __shared__ float s_rmin[kG];
  __shared__ float bnd[4][kTL];   // per warp: x min, x max, z min, z max
  __shared__ unsigned s_mask;
  const int n0 = a.n_pix / a.n1;
  const int tiles_depth = (a.n1 + 31) / 32;
  const int tile = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int line = (tile / tiles_depth) * kTL + warp;
  const int depth = (tile % tiles_depth) * 32 + lane;
  const bool live = line < n0 && depth < a.n1;
  const int pix = live ? line * a.n1 + depth : 0;
  const long frame = blockIdx.y;
  const float px = live ? __ldg(a.points + 3 * pix) : 0.f, py = live ? __ldg(a.points + 3 * pix + 1) : 0.f,
              pz = live ? __ldg(a.points + 3 * pix + 2) : 0.f;
  // The tile's extent.
  {
    float xl = live ? px : INFINITY, xh = live ? px : -INFINITY, zl = live ? pz : INFINITY,
          zh = live ? pz : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      xl = fminf(xl, __shfl_xor_sync(0xffffffffu, xl, o));
      xh = fmaxf(xh, __shfl_xor_sync(0xffffffffu, xh, o));
      zl = fminf(zl, __shfl_xor_sync(0xffffffffu, zl, o));
      zh = fmaxf(zh, __shfl_xor_sync(0xffffffffu, zh, o));
    }
    if (lane == 0) {
      bnd[0][warp] = xl;
      bnd[1][warp] = xh;
      bnd[2][warp] = zl;
      bnd[3][warp] = zh;
    }
  }
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  float x_min = bnd[0][0], x_max = bnd[1][0], z_min = bnd[2][0], z_max = bnd[3][0];
#pragma unroll
  for (int w = 1; w < kTL; ++w) {
    x_min = fminf(x_min, bnd[0][w]);
    x_max = fmaxf(x_max, bnd[1][w]);
    z_min = fminf(z_min, bnd[2][w]);
    z_max = fmaxf(z_max, bnd[3][w]);
  }
  int ev_first = a.ev_begin, ev_last = a.ev_end;
  if (a.seq_epf > 0) {
    ev_first = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_last = ev_first + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_first += a.pass;
    ev_last = ev_first + 1;
  }
  const bool select = a.compounding == USX_COMP_SELECT;
  int best_ev = -1;
  float best_w = 0.0f;
  if (select && live) {
    for (int ev = ev_first; ev < ev_last; ++ev) {
      const float tw = tx_sensitivity_fast(a.tx[ev], px, pz, a.lambda);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }
  const float2* iq = a.iq + frame * a.data_stride;
  const unsigned n_last = static_cast<unsigned>(a.n_smp - 1);
  const int n_ev = max(0, ev_last - ev_first);
  const int n_groups = (a.n_ch + kG - 1) / kG;
  const int n_chunks = (n_ev + kE - 1) / kE;   // steps per group
  const int n_steps = n_groups * n_chunks;
  unsigned phase[2] = {0u, 0u};

  // Thread 0: channel windows of step i and their bulk copies into stage i & 1.
  auto issue = [&](int i) {
    const int st = i & 1;
    const int g = (i / n_chunks) * kG, e0 = ev_first + (i % n_chunks) * kE;
    const long row_base = frame * a.data_stride;
    unsigned bytes = 0;
    for (int e = 0; e < kE; ++e) {
      const int ev = e0 + e;
      float tmin = 0.0f;
      if (ev < ev_last) {
        const TxDev& t = a.tx[ev];
        const float tx0 = ((x_min - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
        const float tx1 = ((x_max - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
        const float tx2 = ((x_min - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
        const float tx3 = ((x_max - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
        tmin = fminf(fminf(tx0, tx1), fminf(tx2, tx3));
      }
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        int lo = -1;
        if (ev < ev_last && ch < a.n_ch && ((s_mask >> k) & 1u)) {
          lo = static_cast<int>(floorf((tmin + s_rmin[k] - a.t0) * a.fs)) - 2;
          lo = max(0, min(lo, a.n_smp - kStageW - 1));
          const long el = row_base + (static_cast<long>(ev) * a.n_ch + ch) * a.n_smp + lo;
          if (el & 1L) lo = lo > 0 ? lo - 1 : lo + 1;   // 16-byte aligned source
          bytes += kStageW * sizeof(float2);
        }
        s_lo[st][e][k] = lo;
      }
    }
    mbar_arrive_expect_tx(&bar[st], bytes);
    for (int e = 0; e < kE; ++e)
      for (int k = 0; k < kG; ++k) {
        const int lo = s_lo[st][e][k];
        if (lo < 0) continue;
        const float2* src = iq + (static_cast<long>(e0 + e) * a.n_ch + g + k) * a.n_smp + lo;
        bulk_copy_g2s(&win[st][e][k][0], src, kStageW * sizeof(float2), &bar[st]);
      }
  };

  cplx das = mk(0.f, 0.f), s = mk(0.f, 0.f), q = mk(0.f, 0.f), coh = mk(0.f, 0.f);
  float incs = 0.0f;
  int n_active = 0;
  float rt[kG], ar[kG], ai[kG];
  unsigned mask = 0u;
  bool timed_out = false;
  for (int i = 0; i < n_steps; ++i) {
    const int g = (i / n_chunks) * kG, e0 = ev_first + (i % n_chunks) * kE;
    const int st = i & 1;
    if (i % n_chunks == 0) {
      // A new channel group: receive delays and the tile's channel mask.
      mask = 0u;
#pragma unroll
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        rt[k] = 0.0f;
        ar[k] = ai[k] = 0.0f;
        if (live && ch < a.n_ch) {
          const float ex = elem_x(a, ch);
          if (aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f) {
            mask |= 1u << k;
            rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
          }
        }
      }
      unsigned m = mask;
      for (int o = 16; o > 0; o >>= 1) m |= __shfl_xor_sync(0xffffffffu, m, o);
      if (threadIdx.x == 0) s_mask = 0u;
      __syncthreads();
      if (lane == 0) atomicOr(&s_mask, m);
      __syncthreads();
      // The group's first step is issued once the tile's channel mask is known.
      if (threadIdx.x == 0) {
        for (int k = 0; k < kG; ++k) {  // receive delay of channel g + k at the tile point nearest it
          const float ex = elem_x(a, min(g + k, a.n_ch - 1));
          const float xc = fminf(fmaxf(ex, x_min), x_max);
          s_rmin[k] = sqrtf((ex - xc) * (ex - xc) + z_min * z_min) / a.c;
        }
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        issue(i);
      }
    }
    // Prefetch the next step (its stage was released by the barrier closing step i - 1).
    if (threadIdx.x == 0 && i + 1 < n_steps && (i + 1) % n_chunks != 0) {
      asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
      issue(i + 1);
    }
    // Wait for this step's windows (bounded: on a timeout the samples are read
    // from global memory and the context's status word records it).
    {
      long spins = 0;
      while (!mbar_try_wait(&bar[st], phase[st])) {
        if (++spins > (1L << 24)) {
          timed_out = true;
          break;
        }
      }
      phase[st] ^= 1u;
    }
    if (mask) {
      for (int e = 0; e < kE; ++e) {
        const int ev = e0 + e;
        if (ev >= ev_last) break;
        const TxDev& t = a.tx[ev];
        float tw;
        if (select) {
          tw = (best_ev == ev && best_w > 0.0f) ? 1.0f : 0.0f;
        } else if (a.tx_weighting) {
          tw = tx_sensitivity_fast(t, px, pz, a.lambda);
        } else {
          tw = 1.0f;
        }
        if (!(tw > 0.0f)) continue;
        const float tau = tx_arrival(t, px, py, pz, a.c);
        float tc = 1.0f, ts = 0.0f;
        if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
        const float wr = tw * tc, wi = tw * ts;
        const long trace0 = (static_cast<long>(ev) * a.n_ch + g) * a.n_smp;
#pragma unroll
        for (int k = 0; k < kG; ++k) {
          if (!(mask & (1u << k))) continue;
          const float idx = (tau + rt[k] - a.t0) * a.fs;
          const float fl = floorf(idx);
          const int kk = static_cast<int>(fl);
          if (static_cast<unsigned>(kk) >= n_last) continue;
          const float f = idx - fl;
          const int lo = s_lo[st][e][k];
          const int loc = kk - lo;
          float2 s0, s1;
          if (!timed_out && lo >= 0 && loc >= 0 && loc + 1 < kStageW) {
            s0 = win[st][e][k][loc];
            s1 = win[st][e][k][loc + 1];
          } else {
            const float2* tr = iq + trace0 + static_cast<long>(k) * a.n_smp + kk;
            s0 = __ldg(tr);
            s1 = __ldg(tr + 1);
          }
          const float vr = fmaf(f, s1.x - s0.x, s0.x);
          const float vi = fmaf(f, s1.y - s0.y, s0.y);
          ar[k] = fmaf(wr, vr, fmaf(-wi, vi, ar[k]));
          ai[k] = fmaf(wr, vi, fmaf(wi, vr, ai[k]));
        }
      }
    }
    __syncthreads();   // stage st is free for step i + 2
    if ((i + 1) % n_chunks == 0) {
      // The group is complete: receive phasor and aperture weight, combine.
#pragma unroll
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        if (ch >= a.n_ch || !live) continue;
        const bool act = (mask >> k) & 1u;
        cplx y = mk(0.f, 0.f);
        if (act) {
          const float w = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha);
          const float ap = a.is_mv ? 1.0f : w;
          float rc = 1.0f, rs = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
          const float gr = ap * rc, gi = ap * rs;
          y = mk(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
        }
        if (a.is_mv) {
          a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = make_float2(y.re, y.im);
          continue;
        }
        n_active += act ? 1 : 0;
        if (a.combiner == USX_COMB_DMAS) {
          const float m = cabsf_(y);
          if (m > 0.0f) {
            const cplx v = cdivr(y, sqrtf(m));
            s = cadd(s, v);
            q = cadd(q, cmul(v, v));
          }
        } else {
          das = cadd(das, y);
        }
        if (a.cf && act) {
          coh = cadd(coh, y);
          incs += cnorm(y);
        }
      }
    }
  }
  if (timed_out && threadIdx.x == 0 && a.status) atomicExch(a.status, 1);
  if (!live || a.is_mv) return;
  cplx out;
  if (n_active == 0) {
    out = mk(0.f, 0.f);
  } else if (a.combiner == USX_COMB_DMAS) {
    const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
    out = cdivr(acc, 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1)));
  } else {
    out = das;
  }
  if (a.cf && n_active > 0)
    out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
  a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
}

// ------------------------------------------------------------------------
// das_ring_kernel: the staged delay-and-sum with a producer warp. The CTA is
// kTL consumer warps (one lateral line x 32 depths each, as das_staged_kernel)
// and one producer warp. Steps are (channel group of kG, transmit) in
// das_fast_kernel's order; the producer stages each step's channel windows
// (kStageW samples per channel, bounded analytically from the tile's extent
// for plane waves) into a ring of kS shared-memory stages with cp.async.bulk,
// each stage completing on its "full" mbarrier (transaction bytes), and
// reuses a stage once all consumer warps have arrived on its "empty"
// mbarrier. The consumers never meet at a CTA barrier inside the loop: each
// waits for its step's stage, computes, and releases it. Samples outside a
// staged window (rounding at its edge, a channel the tile's bound left out)
// are read from global memory, so the frame is das_fast_kernel's bit for bit.
// All waits are bounded; after a timeout the consumers read every sample
// from global memory, the context's status word records it, and the producer
// waits (bounded) for its copies in flight before it exits.
// Measured at 128 channels, 75 plane waves, 512 x 1024 (ms per frame against
// 4.98 for das_fast_kernel's best shape): (kG, kTL, kS) = (4, 4, 8) 12.1,
// (8, 4, 8) 9.9, (8, 8, 8) 8.1, (16, 4, 4) 9.7; with the producer's bounds
// per event and per channel group precomputed, (4, 4, 12) 11.5 and (8, 8, 8)
// 7.75. The consumers still evaluate each event's transmit terms once per
// channel group and now also wait on a stage per step; das_fast_kernel's L1
// already serves most gathers. (8, 8, 8) stays an autotuner candidate.
constexpr int kRingMaxEv = 128;   // events whose tile bound is kept in shared memory

__device__ __forceinline__ bool ring_wait(uint64_t* bar, unsigned parity) {
  for (long spin = 0; spin < (1L << 24); ++spin)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(smem_u32(bar)) : "memory");
}

template <int kG, int kTL, int kS>
__global__ void __launch_bounds__(32 * (kTL + 1)) das_ring_kernel(const BfArgs a) {
  __shared__ __align__(16) float2 win[kS][kG][kStageW];
  __shared__ __align__(8) uint64_t full[kS], empty[kS];
  __shared__ int s_lo[kS][kG];
  __shared__ float bnd[4][kTL];   // per consumer warp: x min, x max, z min, z max
  __shared__ float s_tmin[kRingMaxEv];
  const int n0 = a.n_pix / a.n1;
  const int tiles_depth = (a.n1 + 31) / 32;
  const int tile = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool producer = warp == kTL;
  const int line = (tile / tiles_depth) * kTL + warp;
  const int depth = (tile % tiles_depth) * 32 + lane;
  const bool live = !producer && line < n0 && depth < a.n1;
  const int pix = live ? line * a.n1 + depth : 0;
  const long frame = blockIdx.y;
  const float px = live ? __ldg(a.points + 3 * pix) : 0.f, py = live ? __ldg(a.points + 3 * pix + 1) : 0.f,
              pz = live ? __ldg(a.points + 3 * pix + 2) : 0.f;
  if (!producer) {
    float xl = live ? px : INFINITY, xh = live ? px : -INFINITY, zl = live ? pz : INFINITY,
          zh = live ? pz : -INFINITY;
    for (int o = 16; o > 0; o >>= 1) {
      xl = fminf(xl, __shfl_xor_sync(0xffffffffu, xl, o));
      xh = fmaxf(xh, __shfl_xor_sync(0xffffffffu, xh, o));
      zl = fminf(zl, __shfl_xor_sync(0xffffffffu, zl, o));
      zh = fmaxf(zh, __shfl_xor_sync(0xffffffffu, zh, o));
    }
    if (lane == 0) {
      bnd[0][warp] = xl;
      bnd[1][warp] = xh;
      bnd[2][warp] = zl;
      bnd[3][warp] = zh;
    }
  }
  if (threadIdx.x == 0) {
    for (int st = 0; st < kS; ++st) {
      mbar_init(&full[st], 1);
      mbar_init(&empty[st], kTL);
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  float x_min = bnd[0][0], x_max = bnd[1][0], z_min = bnd[2][0], z_max = bnd[3][0];
#pragma unroll
  for (int w = 1; w < kTL; ++w) {
    x_min = fminf(x_min, bnd[0][w]);
    x_max = fmaxf(x_max, bnd[1][w]);
    z_min = fminf(z_min, bnd[2][w]);
    z_max = fmaxf(z_max, bnd[3][w]);
  }
  int ev_first = a.ev_begin, ev_last = a.ev_end;
  if (a.seq_epf > 0) {
    ev_first = a.ev_begin + static_cast<int>(frame) * a.seq_epf;
    ev_last = ev_first + a.seq_epf;
  }
  if (a.pass >= 0) {
    ev_first += a.pass;
    ev_last = ev_first + 1;
  }
  const float2* iq = a.iq + frame * a.data_stride;
  const int n_ev = max(0, ev_last - ev_first);
  const int n_groups = (a.n_ch + kG - 1) / kG;
  const int n_steps = x_min <= x_max ? n_groups * n_ev : 0;   // no live pixel: no steps

  if (producer) {
    // Lane k < kG stages channel g + k of each step. The earliest transmit
    // arrival over the tile, per event, once (in shared memory).
    float* tmin_ev = reinterpret_cast<float*>(&s_tmin[0]);
    for (int e = lane; e < n_ev && e < kRingMaxEv; e += 32) {
      const TxDev& t = a.tx[ev_first + e];
      const float tx0 = ((x_min - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
      const float tx1 = ((x_max - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
      const float tx2 = ((x_min - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
      const float tx3 = ((x_max - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
      tmin_ev[e] = fminf(fminf(tx0, tx1), fminf(tx2, tx3));
    }
    __syncwarp();
    const float half_ap = 0.5f * z_max / fmaxf(a.f_number, 1e-3f) + a.pitch;
    const long row_base = frame * a.data_stride;
    bool ok = true;
    int issued = 0;
    float rmin = 0.0f;
    bool in_ap = false;
    for (int i = 0; i < n_steps; ++i) {
      const int st = i % kS;
      if (i >= kS) {
        bool got = true;
        if (lane == 0) got = ring_wait(&empty[st], static_cast<unsigned>((i / kS) - 1) & 1u);
        if (!__shfl_sync(0xffffffffu, got, 0)) {
          ok = false;
          break;
        }
      }
      const int g = (i / n_ev) * kG, e_rel = i % n_ev, ev = ev_first + e_rel;
      if (e_rel == 0 && lane < kG) {
        // A new channel group: this lane's channel, in the tile's aperture?
        const int ch = g + lane;
        in_ap = false;
        if (ch < a.n_ch) {
          const float ex = elem_x(a, ch);
          if (ex >= x_min - half_ap && ex <= x_max + half_ap) {
            const float xc = fminf(fmaxf(ex, x_min), x_max);
            rmin = sqrtf((ex - xc) * (ex - xc) + z_min * z_min) / a.c;
            in_ap = true;
          }
        }
      }
      float tmin;
      if (e_rel < kRingMaxEv) {
        tmin = tmin_ev[e_rel];
      } else {
        const TxDev& t = a.tx[ev];
        const float tx0 = ((x_min - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
        const float tx1 = ((x_max - t.ox) * t.sin_a + (z_min - 0.0f) * t.cos_a) / a.c;
        const float tx2 = ((x_min - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
        const float tx3 = ((x_max - t.ox) * t.sin_a + (z_max - 0.0f) * t.cos_a) / a.c;
        tmin = fminf(fminf(tx0, tx1), fminf(tx2, tx3));
      }
      int lo = -1;
      if (lane < kG) {
        const int ch = g + lane;
        if (in_ap) {
          {
            lo = static_cast<int>(floorf((tmin + rmin - a.t0) * a.fs)) - 2;
            lo = max(0, min(lo, a.n_smp - kStageW - 1));
            const long el = row_base + (static_cast<long>(ev) * a.n_ch + ch) * a.n_smp + lo;
            if (el & 1L) lo = lo > 0 ? lo - 1 : lo + 1;   // 16-byte aligned source
          }
        }
        s_lo[st][lane] = lo;
      }
      unsigned bytes = lo >= 0 ? static_cast<unsigned>(kStageW * sizeof(float2)) : 0u;
      for (int o = 16; o > 0; o >>= 1) bytes += __shfl_xor_sync(0xffffffffu, bytes, o);
      __syncwarp();
      if (lane == 0) {
        asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
        mbar_arrive_expect_tx(&full[st], bytes);
      }
      __syncwarp();
      if (lo >= 0) {
        const float2* src = iq + (static_cast<long>(ev) * a.n_ch + g + lane) * a.n_smp + lo;
        bulk_copy_g2s(&win[st][lane][0], src, kStageW * sizeof(float2), &full[st]);
      }
      ++issued;
    }
    if (lane == 0) {
      if (!ok && a.status) atomicExch(a.status, 1);
      // No copy may still be in flight when the CTA exits.
      for (int i = max(0, issued - kS); i < issued; ++i) ring_wait(&full[i % kS], static_cast<unsigned>(i / kS) & 1u);
    }
    return;
  }

  // ---- consumers ----------------------------------------------------------
  const bool select = a.compounding == USX_COMP_SELECT;
  int best_ev = -1;
  float best_w = 0.0f;
  if (select && live) {
    for (int ev = ev_first; ev < ev_last; ++ev) {
      const float tw = tx_sensitivity_fast(a.tx[ev], px, pz, a.lambda);
      if (tw > best_w) {
        best_w = tw;
        best_ev = ev;
      }
    }
  }
  const unsigned n_last = static_cast<unsigned>(a.n_smp - 1);
  cplx das = mk(0.f, 0.f), s = mk(0.f, 0.f), q = mk(0.f, 0.f), coh = mk(0.f, 0.f);
  float incs = 0.0f;
  int n_active = 0;
  float rt[kG], ar[kG], ai[kG];
  unsigned mask = 0u;
  bool timed_out = false;
  for (int i = 0; i < n_steps; ++i) {
    const int g = (i / n_ev) * kG, ev = ev_first + i % n_ev;
    const int st = i % kS;
    if (i % n_ev == 0) {
      mask = 0u;
#pragma unroll
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        rt[k] = 0.0f;
        ar[k] = ai[k] = 0.0f;
        if (live && ch < a.n_ch) {
          const float ex = elem_x(a, ch);
          if (aperture_weight(ex, px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f) {
            mask |= 1u << k;
            rt[k] = dist3(ex, 0.0f, 0.0f, px, py, pz) / a.c;
          }
        }
      }
    }
    if (!timed_out && !ring_wait(&full[st], static_cast<unsigned>(i / kS) & 1u)) timed_out = true;
    if (mask) {
      const TxDev& t = a.tx[ev];
      float tw;
      if (select) {
        tw = (best_ev == ev && best_w > 0.0f) ? 1.0f : 0.0f;
      } else if (a.tx_weighting) {
        tw = tx_sensitivity_fast(t, px, pz, a.lambda);
      } else {
        tw = 1.0f;
      }
      if (tw > 0.0f) {
        const float tau = tx_arrival(t, px, py, pz, a.c);
        float tc = 1.0f, ts = 0.0f;
        if (a.fdem > 0.0f) sincosf(a.two_pi_f * tau, &ts, &tc);
        const float wr = tw * tc, wi = tw * ts;
        const long trace0 = (static_cast<long>(ev) * a.n_ch + g) * a.n_smp;
#pragma unroll
        for (int k = 0; k < kG; ++k) {
          if (!(mask & (1u << k))) continue;
          const float idx = (tau + rt[k] - a.t0) * a.fs;
          const float fl = floorf(idx);
          const int kk = static_cast<int>(fl);
          if (static_cast<unsigned>(kk) >= n_last) continue;
          const float f = idx - fl;
          const int lo = s_lo[st][k];
          const int loc = kk - lo;
          float2 s0, s1;
          if (!timed_out && lo >= 0 && loc >= 0 && loc + 1 < kStageW) {
            s0 = win[st][k][loc];
            s1 = win[st][k][loc + 1];
          } else {
            const float2* tr = iq + trace0 + static_cast<long>(k) * a.n_smp + kk;
            s0 = __ldg(tr);
            s1 = __ldg(tr + 1);
          }
          const float vr = fmaf(f, s1.x - s0.x, s0.x);
          const float vi = fmaf(f, s1.y - s0.y, s0.y);
          ar[k] = fmaf(wr, vr, fmaf(-wi, vi, ar[k]));
          ai[k] = fmaf(wr, vi, fmaf(wi, vr, ai[k]));
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[st]);
    if ((i + 1) % n_ev == 0) {
      // The group is complete: receive phasor and aperture weight, combine.
#pragma unroll
      for (int k = 0; k < kG; ++k) {
        const int ch = g + k;
        if (ch >= a.n_ch || !live) continue;
        const bool act = (mask >> k) & 1u;
        cplx y = mk(0.f, 0.f);
        if (act) {
          const float w = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha);
          const float ap = a.is_mv ? 1.0f : w;
          float rc = 1.0f, rs = 0.0f;
          if (a.fdem > 0.0f) sincosf(a.two_pi_f * rt[k], &rs, &rc);
          const float gr = ap * rc, gi = ap * rs;
          y = mk(fmaf(gr, ar[k], -gi * ai[k]), fmaf(gr, ai[k], gi * ar[k]));
        }
        if (a.is_mv) {
          a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = make_float2(y.re, y.im);
          continue;
        }
        n_active += act ? 1 : 0;
        if (a.combiner == USX_COMB_DMAS) {
          const float m = cabsf_(y);
          if (m > 0.0f) {
            const cplx v = cdivr(y, sqrtf(m));
            s = cadd(s, v);
            q = cadd(q, cmul(v, v));
          }
        } else {
          das = cadd(das, y);
        }
        if (a.cf && act) {
          coh = cadd(coh, y);
          incs += cnorm(y);
        }
      }
    }
  }
  if (timed_out && lane == 0 && a.status) atomicExch(a.status, 1);
  if (!live) return;
  if (a.is_mv) {
    if (n_steps == 0)
      for (int ch = 0; ch < a.n_ch; ++ch) a.y_out[(frame * a.n_pix + pix) * a.n_ch + ch] = make_float2(0.f, 0.f);
    return;
  }
  cplx out;
  if (n_active == 0) {
    out = mk(0.f, 0.f);
  } else if (a.combiner == USX_COMB_DMAS) {
    const cplx acc = cscale(csub(cmul(s, s), q), 0.5f);
    out = cdivr(acc, 0.5f * fmaxf(1.0f, static_cast<float>(n_active - 1)));
  } else {
    out = das;
  }
  if (a.cf && n_active > 0)
    out = cscale(out, (incs > 0.0f) ? cnorm(coh) / (static_cast<float>(n_active) * incs) : 0.0f);
  a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
}

// The delay-and-sum variants the autotuner chooses from (index 0 is the
// default): (channel group, tile lines, minimum resident CTAs per SM, lines
// per warp).
struct DasVariant {
  int group, tile_lines, min_blocks, warp_lines;
  bool deep_first;  // deepest depth tiles dispatched first
  void (*iq)(BfArgs);
  void (*rf)(BfArgs);
  bool staged;   // das_staged_kernel (plane waves, IQ, 16-byte aligned data); else variant 0
  bool table;    // das_table_kernel (IQ, coherent or select, n_ch <= 256); else variant 0
  int producer_warps = 0;   // das_ring_kernel: one warp beside the tile's warps
  int channel_warps = 1;    // das_export_kernel: warps per pixel warp (IQ: MV exports, coherent sums; else variant 0)
  void (*sum)(BfArgs) = nullptr;   // das_csum_kernel, the channel-combining instance (plain IQ launches)
};
// RF input (the reference's interp_rf path) keeps the default shape in
// every variant.
template <int G, int TL, int MB, bool RTS = false, int WL = 1, bool DF = false>
constexpr DasVariant das_variant() {
  return DasVariant{G,     TL, MB, WL, DF, das_fast_kernel<true, G, TL, MB, RTS, WL, DF>,
                    das_fast_kernel<false, 16, 4, 1>, false, false};
}
// Transmit-table shapes: channels per warp G, lines per CTA WL (32 / WL
// depths), MB resident CTAs per SM.
template <int G, int WL, int MB>
constexpr DasVariant das_table_variant() {
  return DasVariant{G, WL, MB, WL, false, das_table_kernel<G, WL, MB>, das_fast_kernel<false, 16, 4, 1>, false, true};
}
template <int G, int TL, int E>
constexpr DasVariant das_staged_variant() {
  return DasVariant{G, TL, 0, 1, false, das_staged_kernel<G, TL, E>, das_fast_kernel<false, 16, 4, 1>, true, false};
}
// The channel-warp kernel: minimum-variance exports, and coherent or select
// IQ delay-and-sum, DMAS and coherence factor with the channel combine in
// shared memory; RF and incoherent launches use variant 0.
template <int G, int PW, int CQ, int WL>
constexpr DasVariant das_export_variant() {
  return DasVariant{G, PW, 0, WL, false, das_export_kernel<G, PW, CQ, WL>, das_fast_kernel<false, 16, 4, 1>,
                    false, false, 0, CQ, das_csum_kernel<G, PW, CQ, WL>};
}
// The producer-warp ring (same applicability as the staged kernel).
template <int G, int TL, int S>
constexpr DasVariant das_ring_variant() {
  return DasVariant{G, TL, 0, 1, false, das_ring_kernel<G, TL, S>, das_fast_kernel<false, 16, 4, 1>, true, false, 1};
}
const DasVariant kDasVariants[] = {
    das_variant<8, 4, 8>(),  das_variant<16, 4, 1>(), das_variant<16, 8, 2>(), das_variant<32, 4, 1>(),
    das_variant<8, 8, 4>(),  das_variant<16, 2, 8>(), das_variant<4, 4, 12>(), das_variant<8, 2, 16>(),
    das_variant<16, 4, 8, true>(), das_variant<16, 2, 16, true>(), das_staged_variant<8, 4, 1>(),
    das_variant<8, 4, 8, false, 4>(), das_variant<4, 4, 12, false, 4>(), das_variant<4, 4, 12, false, 2>(),
    das_variant<8, 2, 16, false, 2>(), das_variant<8, 8, 4, false, 4>(), das_variant<8, 8, 4, false, 8>(),
    das_variant<4, 4, 12, false, 2, true>(), das_variant<4, 4, 12, false, 4, true>(),
    das_variant<8, 4, 8, false, 4, true>(),
    das_table_variant<4, 2, 2>(),
    das_ring_variant<8, 8, 8>(),
    das_export_variant<4, 4, 4, 4>(), das_export_variant<8, 4, 4, 4>(),
};
constexpr int kNumDasVariants = static_cast<int>(sizeof(kDasVariants) / sizeof(kDasVariants[0]));

// ------------------------------------------------------------------------
// Minimum variance (reference beamformer.cpp:137-214, Cholesky :47-79).
//
// One warp per pixel. Shared memory per warp: the compacted active-channel
// samples of the pixel and its range neighbours, and the L x L covariance.
// The covariance entries are spread over the lanes, each entry summed over
// (range offset, subarray) in the reference's order. The Cholesky follows the
// reference's row-oriented recurrence; entries on one anti-diagonal i + j are
// independent and are computed in parallel, each with its inner product in
// the reference's order, so the factor is bit-identical to a serial one.
struct MvShared {
  cplx ys[2 * kMaxRangeAvg + 1][kMaxCh];  // [d + ra][active index]
  cplx R[kMaxL * kMaxL];
  cplx w[kMaxL];
  int act[kMaxCh];
  int fail;
};

__global__ void __launch_bounds__(32 * kMvWarps) mv_kernel(const BfArgs a) {
  extern __shared__ float4 mv_smem_raw[];
  MvShared* sh_all = reinterpret_cast<MvShared*>(mv_smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  MvShared& S = sh_all[warp];
  const long gw = static_cast<long>(blockIdx.x) * kMvWarps + warp;
  if (gw >= a.n_pix) return;
  const int pix = static_cast<int>(gw);
  const long frame = blockIdx.y;
  const int j = pix % a.n1;
  const float px = __ldg(a.points + 3 * pix), pz = __ldg(a.points + 3 * pix + 2);
  const float2* Y = a.y_out + frame * static_cast<long>(a.n_pix) * a.n_ch;
  const bool incoherent = a.compounding == USX_COMP_INCOHERENT;

  // Active channels of this pixel, compacted in ascending channel order.
  int n_act = 0;
  for (int c0 = 0; c0 < a.n_ch; c0 += 32) {
    const int ch = c0 + lane;
    bool act = false;
    if (ch < a.n_ch)
      act = aperture_weight(elem_x(a, ch), px, pz, a.f_number, a.rx_window, a.tukey_alpha) > 0.0f;
    const unsigned m = __ballot_sync(0xffffffffu, act);
    if (act) S.act[n_act + __popc(m & ((1u << lane) - 1u))] = ch;
    n_act += __popc(m);
  }
  __syncwarp();

  const float2* yc = Y + static_cast<long>(pix) * a.n_ch;
  auto finish = [&](cplx out) {
    if (lane != 0) return;
    if (a.cf && n_act > 0) {
      cplx coh = mk(0.f, 0.f);
      float inc = 0.0f;
      for (int q = 0; q < n_act; ++q) {
        const float2 v = yc[S.act[q]];
        coh = cadd(coh, mk(v.x, v.y));
        inc += cnorm(mk(v.x, v.y));
      }
      out = cscale(out, (inc > 0.0f) ? cnorm(coh) / (static_cast<float>(n_act) * inc) : 0.0f);
    }
    if (incoherent)
      a.acc_out[frame * a.n_pix + pix] += cnorm(out);
    else
      a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
  };
  auto das_of_center = [&]() {
    cplx acc = mk(0.f, 0.f);
    for (int q = 0; q < n_act; ++q) {
      const float2 v = yc[S.act[q]];
      acc = cadd(acc, mk(v.x, v.y));
    }
    return acc;
  };

  if (n_act == 0) {
    if (!incoherent && lane == 0) a.out[frame * a.out_stride + pix] = make_float2(0.f, 0.f);
    return;
  }
  if (n_act < 4) {
    finish(das_of_center());
    return;
  }
  int L = a.mv_subarray;
  const int hi = max(2, n_act / 2);
  if (L < 2) L = 2;
  if (L > hi) L = hi;
  const int n_sub = n_act - L + 1;
  const int ra = a.mv_range_average;

  // Stage the active samples of the valid range neighbours.
  int n_d = 0;
  for (int d = -ra; d <= ra; ++d) {
    const int jj = j + d;
    if (jj < 0 || jj >= a.n1) continue;
    const float2* yr = Y + static_cast<long>(pix + d) * a.n_ch;
    for (int q = lane; q < n_act; q += 32) {
      const float2 v = yr[S.act[q]];
      S.ys[n_d][q] = mk(v.x, v.y);
    }
    ++n_d;
  }
  __syncwarp();
  const int n_snap = n_d * n_sub;

  // Covariance, upper triangle, entry (r, c) with c >= r.
  const int n_ent = L * (L + 1) / 2;
  const float inv = 1.0f / static_cast<float>(n_snap);
  for (int e = lane; e < n_ent; e += 32) {
    // Decode packed upper-triangle index e -> (r, c).
    int r = 0, rem = e;
    while (rem >= L - r) {
      rem -= L - r;
      ++r;
    }
    const int c = r + rem;
    cplx acc = mk(0.f, 0.f);
    for (int d = 0; d < n_d; ++d)
      for (int s0 = 0; s0 < n_sub; ++s0) acc = cadd(acc, cmul(S.ys[d][s0 + r], cconj(S.ys[d][s0 + c])));
    acc = cscale(acc, inv);
    S.R[r * L + c] = acc;
    if (c != r) S.R[c * L + r] = cconj(acc);
  }
  __syncwarp();
  if (lane == 0) {
    float trace = 0.0f;
    for (int r = 0; r < L; ++r) trace += S.R[r * L + r].re;
    const float eps = fmaxf(a.mv_loading * trace / static_cast<float>(L), 1e-20f);
    for (int r = 0; r < L; ++r) S.R[r * L + r] = cadd(S.R[r * L + r], mk(eps, 0.0f));
    S.fail = 0;
  }
  __syncwarp();

  // Cholesky by anti-diagonals t = i + j of the lower triangle.
  for (int t = 0; t <= 2 * (L - 1); ++t) {
    const int j_lo = max(0, t - (L - 1));
    const int j_hi = t / 2;
    for (int jc = j_lo + lane; jc <= j_hi; jc += 32) {
      const int i = t - jc;
      cplx sum = S.R[i * L + jc];
      for (int k = 0; k < jc; ++k) sum = csub(sum, cmul(S.R[i * L + k], cconj(S.R[jc * L + k])));
      if (i == jc) {
        const float d = sum.re;
        if (!(d > 0.0f)) S.fail = 1;
        S.R[i * L + jc] = mk(sqrtf(d), 0.0f);
      } else {
        S.R[i * L + jc] = cdiv_wide(sum, S.R[jc * L + jc]);
      }
    }
    __syncwarp();
  }
  if (S.fail) {
    finish(das_of_center());
    return;
  }
  // Forward and back substitution for R w = 1 (serial, reference order).
  if (lane == 0) {
    for (int i = 0; i < L; ++i) {
      cplx sum = mk(1.0f, 0.0f);
      for (int k = 0; k < i; ++k) sum = csub(sum, cmul(S.R[i * L + k], S.w[k]));
      S.w[i] = cdiv_wide(sum, S.R[i * L + i]);
    }
    for (int i = L - 1; i >= 0; --i) {
      cplx sum = S.w[i];
      for (int k = i + 1; k < L; ++k) sum = csub(sum, cmul(cconj(S.R[k * L + i]), S.w[k]));
      S.w[i] = cdiv_wide(sum, S.R[i * L + i]);
    }
    cplx denom = mk(0.f, 0.f);
    for (int q = 0; q < L; ++q) denom = cadd(denom, S.w[q]);
    cplx out;
    if (cabsf_(denom) < 1e-30f) {
      out = das_of_center();
    } else {
      out = mk(0.f, 0.f);
      // Weighted subarray average of the centre pixel (its row in ys).
      int dc = 0;
      for (int d = -ra; d < 0; ++d)
        if (j + d >= 0) ++dc;
      for (int q = 0; q < L; ++q) {
        cplx avg = mk(0.f, 0.f);
        for (int s0 = 0; s0 < n_sub; ++s0) avg = cadd(avg, S.ys[dc][s0 + q]);
        avg = cdivr(avg, static_cast<float>(n_sub));
        out = cadd(out, cmul(cconj(S.w[q]), avg));
      }
      out = cscale(cdiv_wide(out, denom), static_cast<float>(n_act));
    }
    finish(out);
  }
}

__global__ void sqrt_acc_kernel(const float* acc, float2* out, long n_pix, long out_stride,
                                int n_frames) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n_pix * n_frames) return;
  const long f = i / n_pix, p = i - f * n_pix;
  out[f * out_stride + p] = make_float2(sqrtf(acc[i]), 0.0f);
}

}  // namespace
}  // namespace usxcu

using namespace usxcu;

struct usx_bf_plan {
  usx_ctx* ctx = nullptr;
  int device = 0;
  usx_channel_desc cd{};
  usx_beamformer_config cfg{};
  int n0 = 0, n1 = 0;
  float* d_points = nullptr;
  TxDev* d_tx = nullptr;
  int ev_begin = 0, ev_end = 0;
  int mv_mode = USX_MV_EXACT;
  int precision = USX_BF_FAST;
  int das_variant = 0;         // index into kDasVariants (the autotuner's choice)
  bool all_plane_waves = false;  // every event is a plane wave (the staged kernel's bound)
  int* d_mv_stats = nullptr;   // [0] FP64 re-solves, [1] factorisation failures, [2] learned-MV gate rejections
  // Learned minimum variance: the network (not owned) and the gate on |1^H w - 1|.
  usx_mlp* mlp = nullptr;
  float lmv_gate = 0.05f;
  int lmv_beams = -1;   // < 0: the network's weights as predicted; >= 0: subspace refinement
  int lmv_use_net = 1;  // 0: the refinement's basis without the network's direction
  float lmv_share_gate = INFINITY;  // largest share of the refinement's power reduction from the network
  float lmv_level_gate = INFINITY;  // largest tr(R) over its depth's geometric mean
  int lmv_level_lines = 0, lmv_level_depths = 0;  // the level gate's neighbourhood (half widths)
  int64_t lmv_pixels = 0;      // pixels beamformed by the learned path since the last stats read
  // Training export (minimum variance plans): features, weights, valid flags.
  float* exp_feat = nullptr;
  float* exp_w = nullptr;
  uint8_t* exp_valid = nullptr;
  // Tensor-core minimum variance: pixels in classes of similar subarray
  // length (built on first use), device pixel lists per class.
  std::vector<MvClass> mv_classes;
  int* d_class_pixels = nullptr;
  bool classes_built = false;
};

namespace {

int validate_bf_config(const usx_beamformer_config& c) {
  if (!(c.f_number > 0)) return fail(USX_ERR_INVALID, "BeamformerConfig.f_number must be > 0");
  if (c.mv_subarray < 2) return fail(USX_ERR_INVALID, "BeamformerConfig.mv_subarray must be >= 2");
  if (c.mv_diagonal_loading < 0)
    return fail(USX_ERR_INVALID, "BeamformerConfig.mv_diagonal_loading must be >= 0");
  if (c.mv_range_average < 0)
    return fail(USX_ERR_INVALID, "BeamformerConfig.mv_range_average must be >= 0");
  return USX_OK;
}

// Pixels are sorted into classes of similar subarray length from the
// aperture interval |x_e - x_p| <= z / (2 F#) (the support of every receive
// window). The count may differ by one from the kernel's window test at the
// interval's ends; a class keeps a margin of one L and two channels, and the
// kernel sends anything beyond it to the general kernel.
int build_mv_classes(usx_bf_plan* p, const float* points_host) {
  const int n_ch = p->cd.probe.n_elements;
  const long n_pix = static_cast<long>(p->n0) * p->n1;
  const float half_nm1 = 0.5f * static_cast<float>(n_ch - 1), pitch = p->cd.probe.pitch;
  const int plan_lmax = std::min(std::max(p->cfg.mv_subarray, 2), std::max(2, n_ch / 2));
  constexpr int kClasses = 4;
  std::vector<int> bucket[kClasses];
  int nmax[kClasses] = {0, 0, 0, 0};
  for (long i = 0; i < n_pix; ++i) {
    const float px = points_host[3 * i], pz = points_host[3 * i + 2];
    int n_act = 0;
    if (pz > 0.0f) {
      const double half = 0.5 * pz / std::max(p->cfg.f_number, 1e-3f);
      const double lo = std::max(0.0, std::ceil(half_nm1 + (px - half) / pitch));
      const double hi = std::min(static_cast<double>(n_ch - 1), std::floor(half_nm1 + (px + half) / pitch));
      n_act = hi >= lo ? static_cast<int>(hi - lo) + 1 : 0;
    }
    int L = std::min(std::max(p->cfg.mv_subarray, 2), std::max(2, n_act / 2));
    const int b = std::min(kClasses - 1, L / 16);
    bucket[b].push_back(static_cast<int>(i));
    nmax[b] = std::max(nmax[b], n_act);
  }
  USX_CUDA(cudaMalloc(&p->d_class_pixels, sizeof(int) * std::max<long>(1, n_pix)));
  long off = 0;
  p->mv_classes.clear();
  for (int b = 0; b < kClasses; ++b) {
    if (bucket[b].empty()) continue;
    USX_CUDA(cudaMemcpy(p->d_class_pixels + off, bucket[b].data(), sizeof(int) * bucket[b].size(),
                        cudaMemcpyHostToDevice));
    MvClass c;
    c.pixels = p->d_class_pixels + off;
    c.count = static_cast<int>(bucket[b].size());
    c.lmax = std::min(16 * (b + 1), plan_lmax);
    c.nmax = std::min(n_ch, nmax[b] + 2);
    p->mv_classes.push_back(c);
    off += static_cast<long>(bucket[b].size());
  }
  p->classes_built = true;
  return USX_OK;
}

BfArgs make_args(const usx_bf_plan* p) {
  BfArgs a;
  std::memset(&a, 0, sizeof(a));
  const usx_channel_desc& cd = p->cd;
  a.points = p->d_points;
  a.tx = p->d_tx;
  a.status = p->ctx->d_status + 12;
  a.n_ch = cd.probe.n_elements;
  a.n_smp = cd.acq.n_samples;
  a.n1 = p->n1;
  a.n_pix = p->n0 * p->n1;
  a.ev_begin = p->ev_begin;
  a.ev_end = p->ev_end;
  a.c = cd.medium.speed_of_sound;
  a.fs = cd.acq.sampling_frequency;
  a.t0 = cd.acq.t0;
  a.fdem = cd.is_iq ? cd.demodulation_frequency : 0.0f;
  a.two_pi_f = 2.0f * kPi * a.fdem;
  a.lambda = cd.medium.speed_of_sound / cd.probe.center_frequency;
  a.pitch = cd.probe.pitch;
  a.half_nm1 = 0.5f * static_cast<float>(cd.probe.n_elements - 1);
  a.f_number = p->cfg.f_number;
  a.tukey_alpha = p->cfg.tukey_alpha;
  a.rx_window = p->cfg.rx_window;
  a.combiner = p->cfg.combiner;
  a.compounding = p->cfg.compounding;
  a.tx_weighting = p->cfg.transmit_weighting;
  a.cf = p->cfg.coherence_factor;
  a.is_mv = p->cfg.combiner == USX_COMB_MV || p->cfg.combiner == USX_COMB_LEARNED_MV;
  a.mv_subarray = p->cfg.mv_subarray;
  a.mv_range_average = a.is_mv ? p->cfg.mv_range_average : 0;
  a.mv_loading = p->cfg.mv_diagonal_loading;
  a.seq_epf = 0;
  a.pass = -1;
  return a;
}


int bf_execute(usx_bf_plan* plan, int n_frames, const void* data, int64_t data_stride,
               float* frames, int64_t frame_stride, int seq_epf) {
  if (!plan || !data || !frames) return fail(USX_ERR_INVALID, "usx_cu_bf_execute: null argument");
  if (n_frames <= 0) return USX_OK;
  if (n_frames > 65535) return fail(USX_ERR_UNSUPPORTED, "beamforming more than 65535 frames per call");
  usx_ctx* ctx = plan->ctx;
  BfArgs a = make_args(plan);
  if (plan->cd.is_iq)
    a.iq = static_cast<const float2*>(data);
  else
    a.rf = static_cast<const float*>(data);
  a.data_stride = data_stride;
  a.out = reinterpret_cast<float2*>(frames);
  a.out_stride = frame_stride;
  a.seq_epf = seq_epf;
  const long n_pix = a.n_pix;
  const int ev_per_frame = seq_epf > 0 ? seq_epf : (a.ev_end - a.ev_begin);
  if (ev_per_frame <= 0) {
    // No events: the reference returns an all-zero frame.
    for (int f = 0; f < n_frames; ++f)
      USX_CUDA(cudaMemsetAsync(frames + 2 * f * frame_stride, 0, sizeof(float2) * n_pix, ctx->stream));
    return USX_OK;
  }
  const bool fast = plan->precision == USX_BF_FAST;
  const DasVariant* dvp = &kDasVariants[plan->das_variant];
  if (dvp->staged) {
    const bool ok = plan->cd.is_iq && plan->all_plane_waves && a.compounding != USX_COMP_INCOHERENT &&
                    reinterpret_cast<uintptr_t>(data) % 16 == 0 && a.n_smp >= kStageW + 2;
    if (!ok) dvp = &kDasVariants[0];
  }
  if (dvp->table) {
    const bool ok = plan->cd.is_iq && a.compounding != USX_COMP_INCOHERENT && a.n_ch <= kTableMaxCh;
    if (!ok) dvp = &kDasVariants[0];
  }
  const DasVariant& dv = *dvp;
  const bool table = fast && dv.table;
  dim3 grid_das(table  ? ceil_div(plan->n0, dv.warp_lines) * ceil_div(plan->n1, 32 / dv.warp_lines)
                : fast ? ceil_div(plan->n0, dv.tile_lines) * ceil_div(plan->n1, 32)
                       : ceil_div(n_pix, kBfThreads),
                n_frames);
  const size_t table_smem = table ? table_smem_bytes(a.n_ch) : 0;
  if (table)
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(dv.iq), table_smem)) return rc_;
  auto launch_das = [&](const BfArgs& b, const char* name) -> int {
    const bool csum = fast && dv.channel_warps > 1 && !b.is_mv && plan->cd.is_iq &&
                      !(b.compounding == USX_COMP_INCOHERENT && b.pass < 0);
    const bool cexport = fast && dv.channel_warps > 1 && b.is_mv && plan->cd.is_iq;
    // The profiling label names the kernel that runs.
    prof_begin(ctx, csum ? "das_csum_kernel" : cexport ? "das_export_kernel(mv export)" : name);
    if (csum) {
      const size_t tb = exp_table_bytes(dv.tile_lines);
      if (int rc_ = smem_limit(reinterpret_cast<const void*>(dv.sum), tb)) return rc_;
      dv.sum<<<grid_das, 32 * dv.tile_lines * dv.channel_warps, tb, ctx->stream>>>(b);
    } else if (fast && dv.channel_warps > 1 && !(b.is_mv && plan->cd.is_iq)) {
      // A channel-warp shape on an RF or incoherent launch: variant 0.
      const DasVariant& d0 = kDasVariants[0];
      const dim3 g0(ceil_div(plan->n0, d0.tile_lines) * ceil_div(plan->n1, 32), grid_das.y);
      if (plan->cd.is_iq)
        d0.iq<<<g0, 32 * d0.tile_lines, 0, ctx->stream>>>(b);
      else
        d0.rf<<<g0, 32 * d0.tile_lines, 0, ctx->stream>>>(b);
    } else if (fast && dv.channel_warps > 1) {
      const size_t tb = exp_table_bytes(dv.tile_lines);
      if (int rc_ = smem_limit(reinterpret_cast<const void*>(dv.iq), tb)) return rc_;
      dv.iq<<<grid_das, 32 * dv.tile_lines * dv.channel_warps, tb, ctx->stream>>>(b);
    } else if (table) {
      dv.iq<<<grid_das, 32 * table_warps(dv.group, b.n_ch), table_smem, ctx->stream>>>(b);
    } else if (fast) {
      if (plan->cd.is_iq)
        dv.iq<<<grid_das, 32 * (dv.tile_lines + dv.producer_warps), 0, ctx->stream>>>(b);
      else
        dv.rf<<<grid_das, 32 * dv.tile_lines, 0, ctx->stream>>>(b);
    } else {
      if (plan->cd.is_iq)
        das_kernel<true><<<grid_das, kBfThreads, 0, ctx->stream>>>(b);
      else
        das_kernel<false><<<grid_das, kBfThreads, 0, ctx->stream>>>(b);
    }
    prof_end(ctx);
    USX_CHECK_LAUNCH(name);
    return USX_OK;
  };
  if (!a.is_mv) return launch_das(a, fast ? "das_fast_kernel" : "das_kernel");
  if (a.combiner == USX_COMB_LEARNED_MV) {
    // Frames go through in chunks of at most 2^21 pixels: export the
    // compounded channel samples, features, network, gated apply, and the
    // exact tensor-core solve of the gated pixels.
    if (!plan->mlp)
      return fail(USX_ERR_INVALID, "learned minimum variance: no network attached (usx_cu_bf_plan_set_learned)");
    if (a.compounding == USX_COMP_INCOHERENT)
      return fail(USX_ERR_UNSUPPORTED, "learned minimum variance supports coherent and select compounding only");
    const int chunk = static_cast<int>(std::max<long>(1, std::min<long>(n_frames, (1L << 21) / n_pix)));
    const long rows = chunk * n_pix, padded = (rows + 127) / 128 * 128;
    const int widest = mlp_widest(plan->mlp);
    auto up = [](size_t b) { return (b + 255) / 256 * 256; };
    const size_t sz[12] = {up(sizeof(float2) * rows * a.n_ch), up(2 * padded * kLmvFeatures),
                          up(sizeof(float2) * rows * 64),       up(sizeof(float4) * rows),
                          up(2 * padded * widest),              up(2 * padded * widest),
                          up(sizeof(float) * padded * kLmvOutputs), up(sizeof(int2) * rows * kLmvGateClasses),
                          up(sizeof(int2) * rows), up(sizeof(int2) * rows),
                          plan->lmv_beams >= 0 ? up(static_cast<size_t>(lmv_subspace_record_bytes(plan->lmv_beams)) * rows)
                                               : 0,
                          up(sizeof(float) * static_cast<size_t>(chunk) * plan->n1)};
    size_t total = 256;
    for (size_t b : sz) total += b;
    void* ws = nullptr;
    if (int rc = scratch(ctx, total, &ws)) return rc;
    char* q = static_cast<char*>(ws);
    void* bufs[12];
    for (int i = 0; i < 12; ++i) {
      bufs[i] = q;
      q += sz[i];
    }
    // [0, kLmvGateClasses) gated pixels per subarray class, then FP64 re-solves, then overflow.
    int* counters = reinterpret_cast<int*>(q);
    float2* y = static_cast<float2*>(bufs[0]);
    char* feat16 = static_cast<char*>(bufs[1]);
    float2* avg = static_cast<float2*>(bufs[2]);
    float4* meta = static_cast<float4*>(bufs[3]);
    float* net = static_cast<float*>(bufs[6]);
    int2* gated = static_cast<int2*>(bufs[7]);
    int2* fb = static_cast<int2*>(bufs[8]);      // FP64 re-solves
    int2* ovf = static_cast<int2*>(bufs[9]);     // pixels past their class's aperture limit
    for (int f0 = 0; f0 < n_frames; f0 += chunk) {
      const int nf = std::min(chunk, n_frames - f0);
      const long nrows = nf * n_pix, npad = (nrows + 127) / 128 * 128;
      BfArgs b = a;
      b.y_out = y;
      if (b.iq) b.iq += f0 * data_stride;
      if (b.rf) b.rf += f0 * data_stride;
      b.out = a.out + f0 * frame_stride;
      if (seq_epf > 0) b.ev_begin += f0 * seq_epf;
      grid_das.y = nf;
      if (int rc = launch_das(b, fast ? "das_fast_kernel(mv export)" : "das_kernel(mv export)")) return rc;
      LmvLaunch l;
      l.y = y;
      l.points = b.points;
      l.n_ch = b.n_ch;
      l.n_pix = b.n_pix;
      l.n1 = b.n1;
      l.n_frames = nf;
      l.mv_subarray = b.mv_subarray;
      l.range_avg = b.mv_range_average;
      l.f_number = b.f_number;
      l.tukey_alpha = b.tukey_alpha;
      l.half_nm1 = b.half_nm1;
      l.pitch = b.pitch;
      l.rx_window = b.rx_window;
      l.cf = b.cf;
      l.feat16 = feat16;
      l.avg = avg;
      l.meta = meta;
      l.out = b.out;
      l.out_stride = b.out_stride;
      if (npad > nrows)
        USX_CUDA(cudaMemsetAsync(feat16 + 2 * nrows * kLmvFeatures, 0, 2 * (npad - nrows) * kLmvFeatures, ctx->stream));
      if (int rc = launch_lmv_features(ctx, l)) return rc;
      if (int rc = mlp_infer(plan->mlp, ctx, feat16, npad, bufs[4], bufs[5], net)) return rc;
      USX_CUDA(cudaMemsetAsync(counters, 0, (kLmvGateClasses + 2) * sizeof(int), ctx->stream));
      if (plan->lmv_beams >= 0) {
        if (int rc = launch_lmv_subspace(ctx, l, net, plan->lmv_beams, b.mv_loading, plan->lmv_gate,
                                         plan->lmv_use_net, plan->lmv_share_gate, plan->lmv_level_gate,
                                         plan->lmv_level_lines, plan->lmv_level_depths,
                                         static_cast<float*>(bufs[11]), counters,
                                         gated, static_cast<int>(nrows), plan->d_mv_stats + 2,
                                         static_cast<float*>(bufs[10])))
          return rc;
      } else if (int rc = launch_lmv_apply(ctx, net, avg, meta, b.out, b.out_stride, b.n_pix, nf, plan->lmv_gate,
                                           counters, gated, static_cast<int>(nrows), plan->d_mv_stats + 2)) {
        return rc;
      }
      // The exact solve of the gated pixels, one launch per subarray class so
      // that shared memory is sized for the class; pixels past a class's
      // aperture limit go to the CTA kernel.
      const int plan_lmax = std::min(std::max(b.mv_subarray, 2), std::max(2, b.n_ch / 2));
      for (int c = 0; c < kLmvGateClasses; ++c) {
        const int lmax = std::min(kLmvClassWidth * (c + 1), plan_lmax);
        if (c > 0 && kLmvClassWidth * c >= plan_lmax) break;
        MvTcExtra ex;
        // The plan's FP32 mode also serves its gated pixels.
        ex.cov_engine = plan->mv_mode == USX_MV_FP32 ? 2 : 0;
        ex.list = gated + static_cast<long>(c) * nrows;
        ex.list_count = counters + c;
        ex.list_cap = static_cast<int>(nrows);
        ex.list_lmax = lmax;
        // Below the plan's clamp L = n_act / 2, so n_act <= 2 L + 1; the clamped
        // class can hold every aperture.
        ex.list_nmax = lmax >= plan_lmax ? b.n_ch : std::min(b.n_ch, 2 * lmax + 2);
        ex.overflow_count = counters + kLmvGateClasses + 1;
        ex.overflow = ovf;
        ex.overflow_cap = static_cast<int>(nrows);
        if (int rc = launch_mv_tc(ctx, y, b.points, b.out, b.out_stride, nullptr, b.n_ch, b.n_pix, b.n1, nf,
                                  b.mv_subarray, b.mv_range_average, b.mv_loading, b.f_number, b.tukey_alpha,
                                  b.rx_window, b.half_nm1, b.pitch, b.cf, 0, plan->d_mv_stats,
                                  counters + kLmvGateClasses, fb, static_cast<int>(nrows), ex))
          return rc;
      }
    }
    plan->lmv_pixels += static_cast<int64_t>(n_frames) * n_pix;
    return USX_OK;
  }
  // Minimum variance: per pass, export compounded channel samples, then solve.
  const size_t y_bytes = static_cast<size_t>(n_frames) * n_pix * a.n_ch * sizeof(float2);
  const size_t acc_bytes = static_cast<size_t>(n_frames) * n_pix * sizeof(float);
  const size_t fb_bytes = static_cast<size_t>(n_frames) * n_pix * sizeof(int2);
  auto up = [](size_t b) { return (b + 255) / 256 * 256; };
  void* ws = nullptr;
  if (int rc = scratch(ctx, up(y_bytes) + up(acc_bytes) + 2 * up(fb_bytes) + 256, &ws)) return rc;
  char* wsb = static_cast<char*>(ws);
  a.y_out = reinterpret_cast<float2*>(wsb);
  a.acc_out = reinterpret_cast<float*>(wsb + up(y_bytes));
  int2* fb_list = reinterpret_cast<int2*>(wsb + up(y_bytes) + up(acc_bytes));
  int2* ov_list = reinterpret_cast<int2*>(wsb + up(y_bytes) + up(acc_bytes) + up(fb_bytes));
  int* fb_count = reinterpret_cast<int*>(wsb + up(y_bytes) + up(acc_bytes) + 2 * up(fb_bytes));  // [0] FP64, [1] overflow
  const bool tensor = (plan->mv_mode == USX_MV_TENSOR || plan->mv_mode == USX_MV_TENSOR_MMA ||
                       plan->mv_mode == USX_MV_FP32) &&
                      mv_tc_supported(a.n_ch, a.mv_subarray, a.mv_range_average);
  const bool incoherent = a.compounding == USX_COMP_INCOHERENT;
  const size_t smem = sizeof(MvShared) * kMvWarps;
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(mv_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  const dim3 grid_mv(ceil_div(n_pix, kMvWarps), n_frames);
  if (incoherent) USX_CUDA(cudaMemsetAsync(a.acc_out, 0, acc_bytes, ctx->stream));
  const int n_pass = incoherent ? ev_per_frame : 1;
  for (int pass = 0; pass < n_pass; ++pass) {
    BfArgs b = a;
    b.pass = incoherent ? pass : -1;
    if (int rc = launch_das(b, fast ? "das_fast_kernel(mv export)" : "das_kernel(mv export)")) return rc;
    if (tensor) {
      MvTcExtra ex;
      ex.cov_engine = plan->mv_mode == USX_MV_TENSOR_MMA ? 0 : plan->mv_mode == USX_MV_FP32 ? 2 : 1;
      if (plan->exp_feat) {
        // Training pairs: features of every pixel and its Capon weights.
        LmvLaunch l;
        l.y = b.y_out;
        l.points = b.points;
        l.n_ch = b.n_ch;
        l.n_pix = b.n_pix;
        l.n1 = b.n1;
        l.n_frames = n_frames;
        l.mv_subarray = b.mv_subarray;
        l.range_avg = b.mv_range_average;
        l.f_number = b.f_number;
        l.tukey_alpha = b.tukey_alpha;
        l.half_nm1 = b.half_nm1;
        l.pitch = b.pitch;
        l.rx_window = b.rx_window;
        l.cf = b.cf;
        l.feat32 = plan->exp_feat;
        if (int rc = launch_lmv_features(ctx, l)) return rc;
        ex.w_export = plan->exp_w;
        ex.w_valid = plan->exp_valid;
      }
      ex.classes = plan->mv_classes.data();
      ex.n_classes = static_cast<int>(plan->mv_classes.size());
      ex.overflow_count = fb_count + 1;
      ex.overflow = ov_list;
      ex.overflow_cap = static_cast<int>(n_frames * n_pix);
      USX_CUDA(cudaMemsetAsync(fb_count, 0, sizeof(int), ctx->stream));
      if (int rc = launch_mv_tc(ctx, b.y_out, b.points, b.out, b.out_stride, b.acc_out, b.n_ch, b.n_pix, b.n1,
                                n_frames, b.mv_subarray, b.mv_range_average, b.mv_loading, b.f_number,
                                b.tukey_alpha, b.rx_window, b.half_nm1, b.pitch, b.cf, incoherent ? 1 : 0,
                                plan->d_mv_stats, fb_count, fb_list, static_cast<int>(n_frames * n_pix), ex))
        return rc;
    } else {
      prof_begin(ctx, "mv_kernel");
      mv_kernel<<<grid_mv, 32 * kMvWarps, smem, ctx->stream>>>(b);
      prof_end(ctx);
      USX_CHECK_LAUNCH("mv_kernel");
    }
  }
  if (incoherent) {
    const long n = n_pix * n_frames;
    sqrt_acc_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(a.acc_out, a.out, n_pix, frame_stride,
                                                              n_frames);
    USX_CHECK_LAUNCH("sqrt_acc_kernel");
  }
  return USX_OK;
}

}  // namespace

extern "C" {

int usx_cu_bf_plan_create(usx_ctx* ctx, const usx_channel_desc* cd, const usx_grid_desc* grid,
                          const float* points_host, const usx_beamformer_config* cfg,
                          int event_begin, int event_end, usx_bf_plan** out) {
  if (!ctx || !cd || !grid || !points_host || !cfg || !out)
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_create: null argument");
  if (int rc = validate_channel(*cd)) return rc;
  if (int rc = validate_bf_config(*cfg)) return rc;
  if (grid->n_axis0 <= 0 || grid->n_axis1 <= 0)
    return fail(USX_ERR_INVALID, "ScanGrid dimensions must be > 0");
  if (cfg->combiner != USX_COMB_DAS && cfg->combiner != USX_COMB_DMAS && cfg->combiner != USX_COMB_MV &&
      cfg->combiner != USX_COMB_LEARNED_MV)
    return fail(USX_ERR_UNSUPPORTED, "usx_cu_bf_plan_create: unknown combiner");
  if (cfg->combiner == USX_COMB_LEARNED_MV &&
      !mv_tc_supported(cd->probe.n_elements, cfg->mv_subarray, cfg->mv_range_average))
    return fail(USX_ERR_UNSUPPORTED,
                "learned minimum variance supports <= 128 channels, subarrays <= 64 and range averaging <= +/-4");
  if (cfg->combiner == USX_COMB_MV || cfg->combiner == USX_COMB_LEARNED_MV) {
    if (cd->probe.n_elements > kMaxCh)
      return fail(USX_ERR_UNSUPPORTED, "minimum variance supports at most 256 channels");
    if (std::min(cfg->mv_subarray, std::max(2, cd->probe.n_elements / 2)) > kMaxL)
      return fail(USX_ERR_UNSUPPORTED, "minimum variance supports subarrays up to 64");
    if (cfg->mv_range_average > kMaxRangeAvg)
      return fail(USX_ERR_UNSUPPORTED, "minimum variance supports range averaging up to +/-4");
  }
  const long n_pix = static_cast<long>(grid->n_axis0) * grid->n_axis1;
  if (n_pix > 0x7fffffffL / 2) return fail(USX_ERR_UNSUPPORTED, "grid too large");
  const int n_ev = cd->n_events;
  if (event_end < 0) event_end = n_ev;
  event_begin = std::min(std::max(event_begin, 0), n_ev);
  event_end = std::min(std::max(event_end, event_begin), n_ev);

  usx_bf_plan* p = new usx_bf_plan();
  p->ctx = ctx;
  p->device = ctx->device;
  p->cd = *cd;
  p->cd.transmits = nullptr;
  p->cfg = *cfg;
  p->n0 = grid->n_axis0;
  p->n1 = grid->n_axis1;
  p->ev_begin = event_begin;
  p->ev_end = event_end;
  std::vector<TxDev> txs(static_cast<size_t>(n_ev));
  for (int e = 0; e < n_ev; ++e) txs[static_cast<size_t>(e)] = make_txdev(cd->probe, cd->transmits[e]);
  p->all_plane_waves = n_ev > 0;
  for (int e = 0; e < n_ev; ++e) p->all_plane_waves = p->all_plane_waves && txs[static_cast<size_t>(e)].type == USX_TX_PLANE_WAVE;
  cudaError_t e1 = cudaMalloc(&p->d_points, sizeof(float) * 3 * n_pix);
  cudaError_t e2 = cudaMalloc(&p->d_tx, sizeof(TxDev) * std::max(1, n_ev));
  cudaError_t e3 = cudaMalloc(&p->d_mv_stats, sizeof(int) * 4);
  if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
    cudaFree(p->d_points);
    cudaFree(p->d_tx);
    cudaFree(p->d_mv_stats);
    delete p;
    return fail(USX_ERR_NOMEM, "usx_cu_bf_plan_create: device allocation failed");
  }
  cudaMemset(p->d_mv_stats, 0, sizeof(int) * 4);
  cudaMemcpy(p->d_points, points_host, sizeof(float) * 3 * n_pix, cudaMemcpyHostToDevice);
  if (cfg->combiner == USX_COMB_MV && mv_tc_supported(cd->probe.n_elements, cfg->mv_subarray, cfg->mv_range_average)) {
    if (int rc = build_mv_classes(p, points_host)) {
      usx_cu_bf_plan_destroy(p);
      return rc;
    }
  }
  cudaMemcpy(p->d_tx, txs.data(), sizeof(TxDev) * n_ev, cudaMemcpyHostToDevice);
  *out = p;
  return USX_OK;
}

int usx_cu_bf_plan_destroy(usx_bf_plan* plan) {
  if (!plan) return USX_OK;
  // The context may already be gone: synchronise the device, not its stream.
  cudaSetDevice(plan->device);
  cudaDeviceSynchronize();
  cudaFree(plan->d_points);
  cudaFree(plan->d_tx);
  cudaFree(plan->d_mv_stats);
  cudaFree(plan->d_class_pixels);
  delete plan;
  return USX_OK;
}

int usx_cu_bf_plan_workspace(const usx_bf_plan* plan, size_t* bytes) {
  if (!plan || !bytes) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_workspace: null argument");
  const size_t n_pix = static_cast<size_t>(plan->n0) * plan->n1;
  *bytes = 0;
  if (plan->cfg.combiner == USX_COMB_MV || plan->cfg.combiner == USX_COMB_LEARNED_MV)
    *bytes = n_pix * plan->cd.probe.n_elements * sizeof(float2) + n_pix * sizeof(float);
  return USX_OK;
}

int usx_cu_bf_execute_batch(usx_bf_plan* plan, int n_frames, const void* data,
                            int64_t data_stride, float* frames, int64_t frame_stride) {
  return bf_execute(plan, n_frames, data, data_stride, frames, frame_stride, 0);
}

int usx_cu_bf_execute_sequence(usx_bf_plan* plan, int events_per_frame, int n_frames,
                               const void* data, float* frames, int64_t frame_stride) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_execute_sequence: null plan");
  if (events_per_frame <= 0)
    return fail(USX_ERR_INVALID, "beamform_sequence: events_per_frame must be > 0");
  if (plan->ev_begin + static_cast<long>(events_per_frame) * n_frames > plan->ev_end)
    return fail(USX_ERR_INVALID, "beamform_sequence: frames exceed the plan's events");
  return bf_execute(plan, n_frames, data, 0, frames, frame_stride, events_per_frame);
}

int usx_cu_bf_plan_set_mv_mode(usx_bf_plan* plan, int mode) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_mv_mode: null plan");
  if (mode != USX_MV_EXACT && mode != USX_MV_TENSOR && mode != USX_MV_TENSOR_MMA && mode != USX_MV_FP32)
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_mv_mode: unknown mode");
  if (mode != USX_MV_EXACT &&
      !mv_tc_supported(plan->cd.probe.n_elements, plan->cfg.mv_subarray, plan->cfg.mv_range_average))
    return fail(USX_ERR_UNSUPPORTED, "tensor-core minimum variance supports <= 128 channels, L <= 64, range +/-4");
  plan->mv_mode = mode;
  return USX_OK;
}

int usx_cu_bf_variant_count(void) { return kNumDasVariants; }

int usx_cu_bf_variant_info(int index, int* channel_group, int* tile_lines, int* min_blocks, int* warp_lines) {
  if (index < 0 || index >= kNumDasVariants) return fail(USX_ERR_INVALID, "usx_cu_bf_variant_info: no such variant");
  if (channel_group) *channel_group = kDasVariants[index].group;
  if (tile_lines) *tile_lines = kDasVariants[index].tile_lines;
  if (min_blocks) *min_blocks = kDasVariants[index].min_blocks;
  if (warp_lines) *warp_lines = kDasVariants[index].warp_lines;
  return USX_OK;
}

int usx_cu_bf_variant_order(int index, int* deep_first) {
  if (index < 0 || index >= kNumDasVariants) return fail(USX_ERR_INVALID, "usx_cu_bf_variant_order: no such variant");
  if (deep_first) *deep_first = kDasVariants[index].deep_first ? 1 : 0;
  return USX_OK;
}

int usx_cu_bf_variant_kind(int index, int* kind) {
  if (index < 0 || index >= kNumDasVariants) return fail(USX_ERR_INVALID, "usx_cu_bf_variant_kind: no such variant");
  if (kind)
    *kind = kDasVariants[index].table            ? 2
            : kDasVariants[index].producer_warps ? 3
            : kDasVariants[index].channel_warps > 1 ? 4
            : kDasVariants[index].staged         ? 1
                                                 : 0;
  return USX_OK;
}

int usx_cu_bf_plan_set_variant(usx_bf_plan* plan, int index) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_variant: null plan");
  if (index < 0 || index >= kNumDasVariants) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_variant: no such variant");
  plan->das_variant = index;
  return USX_OK;
}

int usx_cu_bf_plan_get_variant(const usx_bf_plan* plan, int* index) {
  if (!plan || !index) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_get_variant: null argument");
  *index = plan->das_variant;
  return USX_OK;
}

int usx_cu_bf_plan_autotune(usx_bf_plan* plan, const void* data, float* frame, int repeats, float* ms_out) {
  if (!plan || !data || !frame) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_autotune: null argument");
  if (plan->precision != USX_BF_FAST) return USX_OK;  // the exact kernel has one shape
  usx_ctx* ctx = plan->ctx;
  const int reps = std::max(1, repeats);
  cudaEvent_t e0, e1;
  USX_CUDA(cudaEventCreate(&e0));
  USX_CUDA(cudaEventCreate(&e1));
  int best = plan->das_variant;
  float best_ms = 0.0f;
  int rc = USX_OK;
  const bool saved_prof = ctx->profiling;
  ctx->profiling = false;
  for (int v = 0; v < kNumDasVariants && rc == USX_OK; ++v) {
    plan->das_variant = v;
    rc = bf_execute(plan, 1, data, 0, frame, 0, 0);  // warm-up (first-use set-up, caches)
    if (rc != USX_OK) break;
    if (cudaEventRecord(e0, ctx->stream) != cudaSuccess) rc = fail(USX_ERR_CUDA, "autotune: event record");
    for (int r = 0; r < reps && rc == USX_OK; ++r) rc = bf_execute(plan, 1, data, 0, frame, 0, 0);
    if (rc != USX_OK) break;
    float ms = 0.0f;
    if (cudaEventRecord(e1, ctx->stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
        cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      rc = fail(USX_ERR_CUDA, "autotune: event timing");
      break;
    }
    ms /= static_cast<float>(reps);
    if (ms_out) ms_out[v] = ms;
    if (v == 0 || ms < best_ms) {
      best_ms = ms;
      best = v;
    }
  }
  ctx->profiling = saved_prof;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  plan->das_variant = best;
  if (rc != USX_OK) return rc;
  // Leave the caller's frame holding the chosen variant's result (all
  // variants agree bit for bit, so this is the same frame).
  return bf_execute(plan, 1, data, 0, frame, 0, 0);
}

int usx_cu_bf_plan_set_precision(usx_bf_plan* plan, int precision) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_precision: null plan");
  if (precision != USX_BF_FAST && precision != USX_BF_EXACT)
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_precision: unknown precision");
  plan->precision = precision;
  return USX_OK;
}

int usx_cu_bf_plan_mv_stats(usx_bf_plan* plan, int64_t* fp64_resolves, int64_t* factorization_failures) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_mv_stats: null plan");
  int h[2] = {0, 0};
  USX_CUDA(cudaMemcpyAsync(h, plan->d_mv_stats, sizeof(h), cudaMemcpyDeviceToHost, plan->ctx->stream));
  USX_CUDA(cudaStreamSynchronize(plan->ctx->stream));
  USX_CUDA(cudaMemsetAsync(plan->d_mv_stats, 0, sizeof(h), plan->ctx->stream));
  if (fp64_resolves) *fp64_resolves = h[0];
  if (factorization_failures) *factorization_failures = h[1];
  return USX_OK;
}

int usx_cu_bf_plan_set_learned(usx_bf_plan* plan, usx_mlp* mlp, float gate) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned: null plan");
  if (plan->cfg.combiner != USX_COMB_LEARNED_MV)
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned: the plan's combiner is not LEARNED_MV");
  if (mlp && !mlp_is_lmv(mlp))
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned: the network must map 256 features to 128 outputs");
  if (!(gate >= 0.0f)) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned: gate must be >= 0");
  plan->mlp = mlp;
  plan->lmv_gate = gate;
  return USX_OK;
}

int usx_cu_bf_plan_set_learned_refine(usx_bf_plan* plan, int n_beams) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_refine: null plan");
  if (n_beams > 6 || (n_beams >= 0 && n_beams % 2 != 0))
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_refine: n_beams must be negative, 0, 2, 4 or 6");
  plan->lmv_beams = n_beams < 0 ? -1 : n_beams;
  return USX_OK;
}

int usx_cu_bf_plan_set_learned_subspace(usx_bf_plan* plan, int use_network, float max_network_share) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_subspace: null plan");
  if (!(max_network_share >= 0.0f))
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_subspace: max_network_share must be >= 0");
  plan->lmv_use_net = use_network ? 1 : 0;
  plan->lmv_share_gate = max_network_share;
  return USX_OK;
}

int usx_cu_bf_plan_set_learned_level_gate(usx_bf_plan* plan, float max_level_ratio) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_level_gate: null plan");
  if (!(max_level_ratio >= 1.0f))
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_level_gate: max_level_ratio must be >= 1");
  plan->lmv_level_gate = max_level_ratio;
  return USX_OK;
}

int usx_cu_bf_plan_set_learned_level_window(usx_bf_plan* plan, int half_lines, int half_depths) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_level_window: null plan");
  if (half_lines < 0 || half_depths < 0 || half_lines > 16 || half_depths > 16)
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_learned_level_window: half widths must be in [0, 16]");
  plan->lmv_level_lines = half_lines;
  plan->lmv_level_depths = half_depths;
  return USX_OK;
}

int usx_cu_bf_plan_set_training_export(usx_bf_plan* plan, float* features, float* weights, uint8_t* valid) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_training_export: null plan");
  const bool any = features || weights || valid;
  if (any && !(features && weights && valid))
    return fail(USX_ERR_INVALID, "usx_cu_bf_plan_set_training_export: give all three buffers or none");
  if (any && (plan->cfg.combiner != USX_COMB_MV || plan->mv_mode == USX_MV_EXACT ||
              plan->cfg.compounding == USX_COMP_INCOHERENT))
    return fail(USX_ERR_INVALID,
                "usx_cu_bf_plan_set_training_export: needs a coherent minimum-variance plan in USX_MV_TENSOR mode");
  plan->exp_feat = features;
  plan->exp_w = weights;
  plan->exp_valid = valid;
  return USX_OK;
}

int usx_cu_bf_plan_learned_stats(usx_bf_plan* plan, int64_t* gated, int64_t* pixels) {
  if (!plan) return fail(USX_ERR_INVALID, "usx_cu_bf_plan_learned_stats: null plan");
  int h = 0;
  USX_CUDA(cudaMemcpyAsync(&h, plan->d_mv_stats + 2, sizeof(int), cudaMemcpyDeviceToHost, plan->ctx->stream));
  USX_CUDA(cudaStreamSynchronize(plan->ctx->stream));
  USX_CUDA(cudaMemsetAsync(plan->d_mv_stats + 2, 0, sizeof(int), plan->ctx->stream));
  if (gated) *gated = h;
  if (pixels) *pixels = plan->lmv_pixels;
  plan->lmv_pixels = 0;
  return USX_OK;
}

int usx_cu_bf_execute(usx_bf_plan* plan, const void* data, float* frame) {
  return usx_cu_bf_execute_batch(plan, 1, data, 0, frame, 0);
}

int usx_cu_bf_execute_queue(usx_ctx* ctx, int n, usx_bf_plan* const* plans, const void* const* data,
                            float* const* frames) {
  if (!ctx || (n > 0 && (!plans || !data || !frames)))
    return fail(USX_ERR_INVALID, "usx_cu_bf_execute_queue: null argument");
  if (n <= 0) return USX_OK;
  bool iq = false;
  for (int i = 0; i < n; ++i) {
    const usx_bf_plan* p = plans[i];
    if (!p || !data[i] || !frames[i]) return fail(USX_ERR_INVALID, "usx_cu_bf_execute_queue: null entry");
    if (p->ctx != ctx) return fail(USX_ERR_INVALID, "usx_cu_bf_execute_queue: a plan of another context");
    if (p->cfg.combiner == USX_COMB_MV || p->cfg.combiner == USX_COMB_LEARNED_MV)
      return fail(USX_ERR_UNSUPPORTED, "usx_cu_bf_execute_queue: DAS, DMAS and coherence-factor plans only");
    if (p->precision != USX_BF_FAST)
      return fail(USX_ERR_UNSUPPORTED, "usx_cu_bf_execute_queue: plans in the reference's operation order run alone");
    if (p->cfg.compounding == USX_COMP_INCOHERENT)
      return fail(USX_ERR_UNSUPPORTED, "usx_cu_bf_execute_queue: incoherent compounding runs alone");
    if (i == 0) iq = p->cd.is_iq;
    if (p->cd.is_iq != iq) return fail(USX_ERR_INVALID, "usx_cu_bf_execute_queue: mixed IQ and RF plans");
  }
  unsigned* next = reinterpret_cast<unsigned*>(ctx->d_status + 15);
  for (int i0 = 0; i0 < n; i0 += kQueueMax) {
    const int m = std::min(kQueueMax, n - i0);
    DasQueueArgs q;
    std::memset(&q, 0, sizeof(q));
    q.n = 0;
    q.first[0] = 0;
    for (int k = 0; k < m; ++k) {
      const usx_bf_plan* p = plans[i0 + k];
      BfArgs a = make_args(p);
      if (iq)
        a.iq = static_cast<const float2*>(data[i0 + k]);
      else
        a.rf = static_cast<const float*>(data[i0 + k]);
      a.out = reinterpret_cast<float2*>(frames[i0 + k]);
      a.out_stride = 0;
      a.data_stride = 0;
      if (a.ev_end <= a.ev_begin) {  // no events: the reference's all-zero frame
        USX_CUDA(cudaMemsetAsync(frames[i0 + k], 0, sizeof(float2) * a.n_pix, ctx->stream));
        continue;
      }
      const int tiles = ceil_div(p->n0, 4) * ceil_div(p->n1, 32);
      q.args[q.n] = a;
      q.tiles[q.n] = tiles;
      q.first[q.n + 1] = q.first[q.n] + tiles;
      ++q.n;
    }
    if (q.n == 0) continue;
    q.next = next;
    USX_CUDA(cudaMemsetAsync(next, 0, sizeof(unsigned), ctx->stream));
    // IQ: das_csum_kernel's body (4 pixel warps x 4 channel warps, the
    // transmit table, the in-order channel combine; the autotuner's usual
    // choice); RF: das_fast_kernel's RF shape.
    const void* kern = iq ? reinterpret_cast<const void*>(das_csum_queue_kernel)
                          : reinterpret_cast<const void*>(das_queue_kernel<false, 16, 4, 1>);
    const int threads = iq ? 512 : 32 * 4;
    const size_t tb = iq ? exp_table_bytes(4) : 0;
    if (iq)
      if (int rc = smem_limit(kern, tb)) return rc;
    int per_sm = 0;
    if (int rc = occupancy(kern, threads, tb, &per_sm)) return rc;
    const unsigned grid = static_cast<unsigned>(std::max(1, per_sm) * ctx->sm_count);
    prof_begin(ctx, iq ? "das_csum_queue_kernel" : "das_queue_kernel");
    if (iq)
      das_csum_queue_kernel<<<grid, threads, tb, ctx->stream>>>(q);
    else
      das_queue_kernel<false, 16, 4, 1><<<grid, threads, 0, ctx->stream>>>(q);
    prof_end(ctx);
    USX_CHECK_LAUNCH("das_queue_kernel");
  }
  return USX_OK;
}

int usx_cu_beamform(usx_ctx* ctx, const usx_channel_desc* cd, const void* data,
                    const usx_grid_desc* grid, const float* points_host,
                    const usx_beamformer_config* cfg, int event_begin, int event_end,
                    float* frame) {
  usx_bf_plan* plan = nullptr;
  if (int rc = usx_cu_bf_plan_create(ctx, cd, grid, points_host, cfg, event_begin, event_end, &plan))
    return rc;
  const int rc = usx_cu_bf_execute(plan, data, frame);
  usx_cu_bf_plan_destroy(plan);
  return rc;
}

}  // extern "C"
