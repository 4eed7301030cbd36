// learned.cu — learned minimum variance: a small MLP predicts each pixel's
// normalised Capon weights, plain minimum variance is the per-pixel fallback.
// No reference counterpart; the method it imitates is the reference's minimum
// variance (core/src/beamformer.cpp:137-214): same active aperture, same
// subarray length L = clamp(mv_subarray, 2, max(2, n_act / 2)), same
// n_sub = n_act - L + 1 subarray average, same DAS output when n_act < 4.
//
// Per pixel (one warp), from the compounded per-channel samples y_d of the
// range rows d in the smoothing window:
//   * the diagonal sums of the smoothed covariance, without forming it:
//       rho[m] = sum_i R[i+m][i] * K = sum_d sum_t c(t, m) y_d[t+m] conj(y_d[t]),
//     c(t, m) = #{ s < n_sub : 0 <= t - s < L - m } (a trapezoid), O(n_act L)
//     per row instead of the covariance's O(K L^2);
//   * the subarray-averaged snapshot a_i = mean_s y_0[s + i], i < L.
// Features (256 floats, scale- and phase-free like the Capon weights):
//   f[2m], f[2m+1]   m = 1..63: r[m] / r[0], r[m] = rho[m] / (L - m), zero for m >= L
//   f[0], f[1]       L / 64, n_act / 128
//   f[128 + 2i], +1  a_i conj(u) / rms(a), u the phase of sum_i a_i, zero for i >= L
// The network's 128 outputs are L w_i / sum(w), i < 64 (interleaved re, im).
// The apply step forms w~ = out / L over i < L and gates on the distortionless
// residual |1^H w~ - 1| (the steering vector is all ones after focusing):
// above the gate the pixel goes on a work list that the tensor-core minimum
// variance solves exactly; below it the output is
//   n_act * sum_i conj(w~_i) a_i / conj(sum_i w~_i)   (unit gain on the look direction).
#include <cuda_bf16.h>

#include <algorithm>
#include <type_traits>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kLmvWarps = 8;      // pixels per CTA, one warp each
constexpr int kLmvMaxL = 64;
constexpr int kLmvFeat = kLmvFeatures;
constexpr int kLmvOut = kLmvOutputs;

struct LmvArgs {
  const float2* y;        // [frame][pix][n_ch] compounded channel samples
  const float* points;
  int n_ch, n_pix, n1;
  long n_rows;            // frames * n_pix
  int mv_subarray, range_avg, n_dmax;
  float f_number, tukey_alpha, half_nm1, pitch;
  int rx_window, cf;
  __nv_bfloat16* feat16;  // [row][256] (inference) or null
  float* feat32;          // [row][256] (training export) or null
  float2* avg;            // [row][64] subarray-averaged snapshot (inference) or null
  float4* meta;           // [row] (L, n_act, coherence factor, first active channel) (inference) or null
  float2* out;            // frames, written here for n_act < 4 (inference) or null
  long out_stride;
};

// kStride: the shared-memory row stride when it is known at compile time
// (n_ch <= 128: 128), else 0 (n_ch); kND: the full smoothing window's row
// count that gets an unrolled lag loop (5 for range averaging 2), else 0.
// Five CTAs per SM (48 registers) measured faster than the four that 59
// registers allow. Staging the rows with the range rows in an inner loop
// (no integer division in the index) measured the same (2.60 ms per frame).
template <int kStride, int kND>
__global__ void __launch_bounds__(32 * kLmvWarps, 5) lmv_features_kernel(const LmvArgs a) {
  extern __shared__ float2 lmv_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int rs = kStride ? kStride : a.n_ch;
  float2* rows = lmv_smem + static_cast<size_t>(warp) * a.n_dmax * rs;
  int* act = reinterpret_cast<int*>(lmv_smem + static_cast<size_t>(kLmvWarps) * a.n_dmax * rs) + warp * a.n_ch;

  for (long row = static_cast<long>(blockIdx.x) * kLmvWarps + warp; row < a.n_rows;
       row += static_cast<long>(gridDim.x) * kLmvWarps) {
    const long frame = row / a.n_pix;
    const int pix = static_cast<int>(row - frame * a.n_pix);
    const int j = pix % a.n1;
    const float px = __ldg(a.points + 3 * pix), pz = __ldg(a.points + 3 * pix + 2);
    const float2* Y = a.y + frame * static_cast<long>(a.n_pix) * a.n_ch;
    __syncwarp();
    int n_act = 0;
    for (int c0 = 0; c0 < a.n_ch; c0 += 32) {
      const int ch = c0 + lane;
      bool on = false;
      if (ch < a.n_ch)
        on = aperture_weight((static_cast<float>(ch) - a.half_nm1) * a.pitch, px, pz, a.f_number, a.rx_window,
                             a.tukey_alpha) > 0.0f;
      const unsigned m = __ballot_sync(0xffffffffu, on);
      if (on) act[n_act + __popc(m & ((1u << lane) - 1u))] = ch;
      n_act += __popc(m);
    }
    __syncwarp();

    int L = a.mv_subarray;
    const int hi = max(2, n_act / 2);
    if (L < 2) L = 2;
    if (L > hi) L = hi;
    const int n_sub = n_act - L + 1;
    int dlo = -a.range_avg, dhi = a.range_avg;
    while (j + dlo < 0) ++dlo;
    while (j + dhi >= a.n1) --dhi;
    const int n_d = dhi - dlo + 1, dc = -dlo;

    if (n_act >= 4) {
      for (int k = lane; k < n_d * n_act; k += 32) {
        const int d = k / n_act, q = k - d * n_act;
        rows[d * rs + q] = Y[static_cast<long>(pix + dlo + d) * a.n_ch + act[q]];
      }
    } else {
      for (int q = lane; q < n_act; q += 32) rows[dc * rs + q] = Y[static_cast<long>(pix) * a.n_ch + act[q]];
    }
    __syncwarp();

    // Coherence factor terms over the active aperture of the centre row.
    float cre = 0.f, cim = 0.f, inc = 0.f;
    for (int q = lane; q < n_act; q += 32) {
      const float2 v = rows[dc * rs + q];
      cre += v.x;
      cim += v.y;
      inc = fmaf(v.x, v.x, fmaf(v.y, v.y, inc));
    }
    for (int o = 16; o > 0; o >>= 1) {
      cre += __shfl_xor_sync(0xffffffffu, cre, o);
      cim += __shfl_xor_sync(0xffffffffu, cim, o);
      inc += __shfl_xor_sync(0xffffffffu, inc, o);
    }
    const float cf_factor =
        (a.cf && n_act > 0) ? ((inc > 0.f) ? (cre * cre + cim * cim) / (static_cast<float>(n_act) * inc) : 0.f) : 1.f;

    if (n_act < 4) {
      // The reference's rule: fewer than four active channels give the DAS sum.
      if (lane == 0) {
        if (a.out) a.out[frame * a.out_stride + pix] = make_float2(cre * cf_factor, cim * cf_factor);
        if (a.meta) a.meta[row] = make_float4(0.f, static_cast<float>(n_act), cf_factor, 0.f);
      }
      for (int f = lane; f < kLmvFeat; f += 32) {
        if (a.feat16) a.feat16[row * kLmvFeat + f] = __float2bfloat16_rn(0.f);
        if (a.feat32) a.feat32[row * kLmvFeat + f] = 0.f;
      }
      if (a.avg)
        for (int i = lane; i < kLmvMaxL; i += 32) a.avg[row * kLmvMaxL + i] = make_float2(0.f, 0.f);
      continue;
    }

    // Diagonal sums rho[m] for the lags m1 = lane and m2 = 63 - lane, in one
    // loop of (n_act - m1) + (n_act - m2) steps: lag m has n_act - m terms, so
    // when L > 32 every lane runs about the same count (as two loops the
    // warp would run lane 0's n_act steps, then lane 31's n_act - 32).
    float rre[2] = {0.f, 0.f}, rim[2] = {0.f, 0.f};
    {
      const int m1 = lane, m2 = 63 - lane;
      const int len1 = m1 < L ? n_act - m1 : 0;
      const int len = len1 + (m2 < L ? n_act - m2 : 0);   // len1 == 0 implies len == 0
      auto lags = [&](auto nd_c) {
        // ND > 0: the full window with a compile-time row count (and, with
        // kStride, immediate row offsets); 0: n_d rows at run time.
        constexpr int ND = decltype(nd_c)::value;
        const int nd = ND > 0 ? ND : n_d;
        int m = m1, t = 0;
        float are = 0.f, aim = 0.f;
        for (int it = 0; it < len; ++it, ++t) {
          if (it == len1) {   // on to the second lag
            rre[0] = are;
            rim[0] = aim;
            are = 0.f;
            aim = 0.f;
            m = m2;
            t = 0;
          }
          // The trapezoid weight depends on t only: sum the range rows first.
          const float w = static_cast<float>(min(t, n_sub - 1) - max(0, t - (L - m - 1)) + 1);
          const float2* pp = rows + m;
          float sre = 0.f, sim = 0.f;
#pragma unroll 5
          for (int d = 0; d < nd; ++d) {
            const float2 pv = pp[d * rs + t], q = rows[d * rs + t];
            sre = fmaf(pv.x, q.x, fmaf(pv.y, q.y, sre));
            sim = fmaf(pv.y, q.x, fmaf(-pv.x, q.y, sim));
          }
          are = fmaf(w, sre, are);
          aim = fmaf(w, sim, aim);
        }
        if (len > len1) {
          rre[1] = are;
          rim[1] = aim;
        } else if (len > 0) {
          rre[0] = are;
          rim[0] = aim;
        }
      };
      if (kND > 0 && n_d == kND)
        lags(std::integral_constant<int, kND>{});
      else
        lags(std::integral_constant<int, 0>{});
      if (m1 < L) {
        rre[0] /= static_cast<float>(L - m1);
        rim[0] /= static_cast<float>(L - m1);
      }
      if (m2 < L) {
        rre[1] /= static_cast<float>(L - m2);
        rim[1] /= static_cast<float>(L - m2);
      }
    }
    // Lag 32 + lane from lane 31 - lane, for the feature writes below.
    rre[1] = __shfl_sync(0xffffffffu, rre[1], 31 - lane);
    rim[1] = __shfl_sync(0xffffffffu, rim[1], 31 - lane);
    const float r0 = __shfl_sync(0xffffffffu, rre[0], 0);
    const float inv_r0 = r0 > 0.f ? 1.0f / r0 : 0.f;

    // Subarray-averaged snapshot of the centre row.
    float2 av[2];
    float sre = 0.f, sim = 0.f, e2 = 0.f;
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int i = lane + 32 * s2;
      float xr = 0.f, xi = 0.f;
      if (i < L) {
        const float2* yr = rows + dc * rs + i;
        for (int s = 0; s < n_sub; ++s) {
          xr += yr[s].x;
          xi += yr[s].y;
        }
        xr /= static_cast<float>(n_sub);
        xi /= static_cast<float>(n_sub);
      }
      av[s2] = make_float2(xr, xi);
      sre += xr;
      sim += xi;
      e2 = fmaf(xr, xr, fmaf(xi, xi, e2));
    }
    for (int o = 16; o > 0; o >>= 1) {
      sre += __shfl_xor_sync(0xffffffffu, sre, o);
      sim += __shfl_xor_sync(0xffffffffu, sim, o);
      e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    }
    const float smag = sqrtf(sre * sre + sim * sim);
    const float ure = smag > 0.f ? sre / smag : 1.f, uim = smag > 0.f ? sim / smag : 0.f;
    const float inv_rms = e2 > 0.f ? rsqrtf(e2 / static_cast<float>(L)) : 0.f;

    // Features: lane writes pairs (2m, 2m+1) for m = lane, lane+32 and
    // (128 + 2i, 129 + 2i) for i = lane, lane + 32.
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int m = lane + 32 * s2;
      float2 fr = make_float2(rre[s2] * inv_r0, rim[s2] * inv_r0);
      if (m >= L) fr = make_float2(0.f, 0.f);
      if (m == 0) fr = make_float2(static_cast<float>(L) / 64.0f, static_cast<float>(n_act) / 128.0f);
      const float2 v = av[s2];
      // a conj(u) / rms
      const float2 fa = make_float2(fmaf(v.x, ure, v.y * uim) * inv_rms, fmaf(v.y, ure, -v.x * uim) * inv_rms);
      if (a.feat16) {
        __nv_bfloat162* f2 = reinterpret_cast<__nv_bfloat162*>(a.feat16 + row * kLmvFeat);
        f2[m] = __floats2bfloat162_rn(fr.x, fr.y);
        f2[64 + m] = __floats2bfloat162_rn(fa.x, fa.y);
      }
      if (a.feat32) {
        float2* f2 = reinterpret_cast<float2*>(a.feat32 + row * kLmvFeat);
        f2[m] = fr;
        f2[64 + m] = fa;
      }
      if (a.avg) a.avg[row * kLmvMaxL + m] = v;
    }
    if (lane == 0 && a.meta)
      a.meta[row] = make_float4(static_cast<float>(L), static_cast<float>(n_act), cf_factor, static_cast<float>(act[0]));
  }
}

// A gated pixel joins the exact solver's work list of its subarray class.
__device__ __forceinline__ void push_gated(int* counts, int2* lists, int cap, int L, int pix, long frame) {
  const int c = min(kLmvGateClasses - 1, max(0, (L - 1) / kLmvClassWidth));
  const int slot = atomicAdd(counts + c, 1);
  if (slot < cap) lists[static_cast<long>(c) * cap + slot] = make_int2(pix, static_cast<int>(frame));
}

struct ApplyArgs {
  const float* net;       // [row][128] network outputs (FP32)
  const float2* avg;      // [row][64]
  const float4* meta;     // [row]
  float2* out;
  long out_stride;
  int n_pix;
  long n_rows;
  float gate;
  int* gated_count;       // pixels sent to the exact solver, per subarray class
  int2* gated;            // their (pixel, frame): kLmvGateClasses lists of gated_cap
  int gated_cap;
  int* stats;             // running count of gated pixels (plan statistics)
};

__global__ void __launch_bounds__(256) lmv_apply_kernel(const ApplyArgs a) {
  const int lane = threadIdx.x & 31;
  const long n_warps = static_cast<long>(gridDim.x) * (blockDim.x >> 5);
  for (long row = static_cast<long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); row < a.n_rows;
       row += n_warps) {
    const float4 meta = a.meta[row];
    const int L = static_cast<int>(meta.x);
    if (L == 0) continue;  // n_act < 4: written by the feature pass
    // Lane holds weights 2 lane, 2 lane + 1 (one float4 of the output row).
    const float4 o = reinterpret_cast<const float4*>(a.net + row * kLmvOut)[lane];
    const float4 v = reinterpret_cast<const float4*>(a.avg + row * kLmvMaxL)[lane];
    const float inv_l = 1.0f / static_cast<float>(L);
    float dre = 0.f, dim = 0.f, nre = 0.f, nim = 0.f;
    const int i0 = 2 * lane;
    if (i0 < L) {
      const float wr = o.x * inv_l, wi = o.y * inv_l;
      dre += wr;
      dim += wi;
      nre = fmaf(wr, v.x, fmaf(wi, v.y, nre));   // conj(w) a
      nim = fmaf(wr, v.y, fmaf(-wi, v.x, nim));
    }
    if (i0 + 1 < L) {
      const float wr = o.z * inv_l, wi = o.w * inv_l;
      dre += wr;
      dim += wi;
      nre = fmaf(wr, v.z, fmaf(wi, v.w, nre));
      nim = fmaf(wr, v.w, fmaf(-wi, v.z, nim));
    }
    for (int s = 16; s > 0; s >>= 1) {
      dre += __shfl_xor_sync(0xffffffffu, dre, s);
      dim += __shfl_xor_sync(0xffffffffu, dim, s);
      nre += __shfl_xor_sync(0xffffffffu, nre, s);
      nim += __shfl_xor_sync(0xffffffffu, nim, s);
    }
    if (lane != 0) continue;
    const long frame = row / a.n_pix;
    const int pix = static_cast<int>(row - frame * a.n_pix);
    const float res = sqrtf((dre - 1.f) * (dre - 1.f) + dim * dim);
    if (!(res <= a.gate)) {
      push_gated(a.gated_count, a.gated, a.gated_cap, L, pix, frame);
      if (a.stats) atomicAdd(a.stats, 1);
      continue;
    }
    // n_act * num / conj(den), num = sum conj(w) a, den = sum w.
    const float den2 = dre * dre + dim * dim;
    const float scale = meta.y * meta.z / den2;
    a.out[frame * a.out_stride + pix] =
        make_float2((nre * dre - nim * dim) * scale, (nim * dre + nre * dim) * scale);
  }
}

// Learned-subspace refinement (an alternative to lmv_apply_kernel).
//
// The network's weights w~ are a guess of the Capon direction R^-1 1. Instead
// of using them as they are, the pixel solves the Capon problem exactly
// within the subspace spanned by the DFT beams u_b[i] = e^{j 2 pi b i / L} / sqrt(L),
// b = 0, +1, -1, ..., +3, -3 (n_beams + 1 of them; b = 0 is the look direction) and w~
// (its part orthogonal to the beams, dropped when negligible):
//   minimise w^H R~ w subject to 1^H w = 1, w = Q c,
//   (Q^H R Q + eps I) c = Q^H 1,   eps = max(delta tr(R) / L, 1e-20),
// with R the spatially smoothed, range-averaged covariance of the reference's
// minimum variance (beamformer.cpp:158-187) applied through its snapshots
// y_s = y_d[s0 .. s0 + L), never formed. The beams are orthonormal, so their
// snapshot projections are window sums of e^{-j w t} y_d[t], i.e. differences
// of one prefix sum per beam and range row (O(1) per snapshot); only w~
// costs L multiply-adds per snapshot. If w~ is the Capon direction the result
// is the exact minimum variance; in every case it is distortionless, and its
// output power is at most that of DAS (w = 1/L) and of w~. The gate on the
// network's distortionless residual |1^H w~ / L - 1| comes first; gated
// pixels go to the exact solver.
constexpr int kSubMaxBeams = 7;            // b = 0, +1, -1, +2, -2, +3, -3
constexpr int kSubWarps = 4;
constexpr int kSubMaxN = 128;              // active channels

struct SubArgs {
  const float2* y;        // [frame][pix][n_ch]
  const float* points;
  const float* net;       // [row][128]
  const float2* avg;      // [row][64] subarray-averaged snapshot of the centre row
  const float4* meta;     // [row] (L, n_act, cf, first active channel)
  float2* out;
  long out_stride;
  int n_ch, n_pix, n1, n_dmax;
  long n_rows;
  int range_avg, n_beams;
  float f_number, tukey_alpha, half_nm1, pitch, loading, gate;
  int rx_window;
  int use_net;            // 0: the beams alone (the network's direction left out)
  float share_gate;       // largest share of the power reduction the network's direction may carry
  float log_level_gate;   // ln of the largest tr(R) over its depth's level (+inf: off)
  float* level;           // [frame][n1]: mean over lines of ln tr(R) (the depth's level)
  int level_lines, level_depths;  // the level gate's neighbourhood: +/- lines, +/- depths
  int* gated_count;
  int2* gated;
  int gated_cap;
  int* stats;
  float* rec;             // [row][lmv_rec_floats(NB)] stage-1 records
};

// Floats per pixel record between the two stages: the Gram matrix (upper
// triangle, re/im), the projections of the subarray average, w_q^H 1, eps,
// the snapshot count, the basis size, flags, L, valid, tr(R).
__host__ __device__ constexpr int lmv_rec_floats(int nb) {
  return ((nb + 1) * (nb + 2) + 2 * (nb + 1) + 9 + 3) / 4 * 4;
}

// The beams' prefix sums are stored skewed, t at t + t / 16: conflict-free
// both for the runs of four the scan writes (t = 4 lane + c) and for the
// consecutive t the snapshot passes read. Three range rows (linear, zero past
// n_act): the next two stream in (cp.async) while the current one is used.
constexpr int kSubPre = kSubMaxN + 1 + kSubMaxN / 16;
constexpr int kSubRing = 32;   // snapshot projections left over from full passes

__device__ __forceinline__ int skw(int t) { return t + (t >> 4); }

template <int NB>
struct SubWarpSmem {
  float2 pre[NB][kSubPre];                  // prefix sums of one row, per beam (skewed)
  float2 tw1[kSubMaxN];                     // e^{-j 2 pi t / L}; beam b's twiddle is its b-th power
  float4 qq[kLmvMaxL];                      // the network's direction q, orthogonalised: (q.x, q.x, q.y, q.y), 0 past L
  float2 ring[NB + 1][kSubRing];            // z vectors of snapshots past each row's full passes
  float2 rows[3][kSubMaxN];
};

// e^{-j 2 pi b t / L} for b = 0, 1, -1, 2, -2, 3, -3 (k = 0..6) from
// t1 = e^{-j 2 pi t / L}: the |b|-th power, conjugated for negative b.
__device__ __forceinline__ float2 beam_twiddle(float2 t1, int k) {
  if (k == 0) return make_float2(1.f, 0.f);
  float2 t = t1;
  if (k >= 3) t = make_float2(t1.x * t1.x - t1.y * t1.y, 2.f * t1.x * t1.y);
  if (k >= 5) t = make_float2(t.x * t1.x - t.y * t1.y, t.x * t1.y + t.y * t1.x);
  return (k & 1) ? t : make_float2(t.x, -t.y);
}
template <int NB>
__host__ __device__ constexpr size_t sub_warp_bytes() {
  return (sizeof(SubWarpSmem<NB>) + 15) / 16 * 16;
}

__device__ __forceinline__ void cp_async8(void* smem, const void* g, int src_bytes) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
               "l"(g), "r"(src_bytes)
               : "memory");
}

__device__ __forceinline__ float2 warp_sum2(float2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

// Stage 1 of the refinement, one warp per pixel: the gate, the basis, the
// snapshot projections and the Gram matrix G = sum_s z_s z_s^H (z = Q^H y_s),
// written with the projections of the subarray average and of 1 onto the
// basis as one record per pixel (stage 2 solves it, one thread per pixel).
// The range rows are processed one at a time while the next streams in: the
// beams' prefix sums, then passes of 32 snapshots (each lane one snapshot:
// beam projections from the prefix sums, the network direction's by a
// sliding dot product, its Gram update). The snapshots past the last full
// pass (n_sub mod 32, often one) take the network direction's projection
// from the whole warp and wait in a ring until 32 have gathered. NB, the
// number of beams (1, 3, 5 or 7), is a template parameter so that every loop
// over the basis is unrolled to its size.
// Three CTAs per SM (168 registers, 12 warps) measured faster than four with
// the spills a 128-register cap forces, and than 14 warps in two-warp CTAs
// at 144 registers (7.0 against 6.3 ms per frame).
template <int NB>
__global__ void __launch_bounds__(32 * kSubWarps, 3) lmv_subspace_gram_kernel(const SubArgs a) {
  extern __shared__ float4 sub_smem_raw[];
  constexpr int K1 = NB + 1;
  constexpr int kG = K1 * (K1 + 1);  // upper triangle of G, (re, im)
  constexpr int kTail = kG + 2 * K1; // record: [G][Q^H abar][w_q^H 1, eps, K, nb, has_w, L, valid, tr R]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  SubWarpSmem<NB>& sm = *reinterpret_cast<SubWarpSmem<NB>*>(reinterpret_cast<char*>(sub_smem_raw) +
                                                           warp * sub_warp_bytes<NB>());
  const long stride = static_cast<long>(gridDim.x) * kSubWarps;

  // The next pixel's metadata and network output are fetched while the
  // current one is processed.
  long row = static_cast<long>(blockIdx.x) * kSubWarps + warp;
  float4 meta_n = make_float4(0.f, 0.f, 0.f, 0.f), o_n = meta_n;
  if (row < a.n_rows) {
    meta_n = a.meta[row];
    o_n = reinterpret_cast<const float4*>(a.net + row * kLmvOut)[lane];
  }
  for (; row < a.n_rows; row += stride) {
    const float4 meta = meta_n, o = o_n;
    if (row + stride < a.n_rows) {
      meta_n = a.meta[row + stride];
      o_n = reinterpret_cast<const float4*>(a.net + (row + stride) * kLmvOut)[lane];
    }
    float* rec = a.rec + row * lmv_rec_floats(NB);
    const int L = static_cast<int>(meta.x);
    if (L == 0) {  // n_act < 4: written by the feature pass
      if (lane == 0) rec[kTail + 7] = 0.f;
      continue;
    }
    const long frame = row / a.n_pix;
    const int pix = static_cast<int>(row - frame * a.n_pix);
    // The first nb of b = 0, 1, -1, 2, -2, 3, -3 are distinct modulo L when
    // nb <= L; with nb = L they span every length-L vector (the exact solve).
    const int nb = min(NB, L);

    // Active aperture (|x_e - x_p| < z / (2 F#): one contiguous run, from the
    // feature pass) and the range rows of the smoothing window; the first row
    // starts streaming now.
    const int j = pix % a.n1;
    const float2* Y = a.y + frame * static_cast<long>(a.n_pix) * a.n_ch;
    const int n_act = min(static_cast<int>(meta.y), kSubMaxN), first = static_cast<int>(meta.w);
    const int n_sub = n_act - L + 1;
    int dlo = -a.range_avg, dhi = a.range_avg;
    while (j + dlo < 0) ++dlo;
    while (j + dhi >= a.n1) --dhi;
    const int n_d = dhi - dlo + 1;
    auto issue_row = [&](int d) {
      float2* dst = sm.rows[d % 3];
      const float2* src = Y + static_cast<long>(pix + dlo + d) * a.n_ch + first;
#pragma unroll
      for (int c = 0; c < kSubMaxN / 32; ++c) {
        const int t = c * 32 + lane;
        const bool in = t < n_act;
        cp_async8(dst + t, in ? src + t : src, in ? 8 : 0);   // zero-fills past n_act
      }
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    };
    issue_row(0);
    if (n_d > 1) issue_row(1);
    const float4 av4 = reinterpret_cast<const float4*>(a.avg + row * kLmvMaxL)[lane];

    // The network's weights (lane holds i = 2 lane, 2 lane + 1) and the gate.
    const float inv_l = 1.0f / static_cast<float>(L);
    float2 w0 = make_float2(0.f, 0.f), w1 = make_float2(0.f, 0.f);
    if (2 * lane < L) w0 = make_float2(o.x * inv_l, o.y * inv_l);
    if (2 * lane + 1 < L) w1 = make_float2(o.z * inv_l, o.w * inv_l);
    const float2 sw = warp_sum2(make_float2(w0.x + w1.x, w0.y + w1.y));
    const float res = sqrtf((sw.x - 1.f) * (sw.x - 1.f) + sw.y * sw.y);
    if (!(res <= a.gate)) {
      asm volatile("cp.async.wait_all;\n" ::: "memory");
      if (lane == 0) {
        push_gated(a.gated_count, a.gated, a.gated_cap, L, pix, frame);
        if (a.stats) atomicAdd(a.stats, 1);
        rec[kTail + 7] = 0.f;
      }
      __syncwarp();
      continue;
    }
    // Twiddles e^{-j 2 pi t / L}, t < 128, argument reduced to one turn.
    // (Read up to t < 64 when the aperture fits 64 channels, else t < 128.)
    const int n_tw = n_act <= 64 ? 64 : kSubMaxN;
    for (int t = lane; t < n_tw; t += 32) {
      float sn, cs;
      sincospif(2.0f * static_cast<float>(t % L) * inv_l, &sn, &cs);
      sm.tw1[t] = make_float2(cs, -sn);
    }
    const float rs = rsqrtf(static_cast<float>(L));
    __syncwarp();
    // w~ minus its projections on the beams: c_b = u_b^H w~ (u_b = conj(tw_b) / sqrt(L)).
    float2 wv[2];
    {
      const int i0 = 2 * lane;
      wv[0] = w0;
      wv[1] = w1;
      // (wv is zero past L; beams past nb alias earlier ones and are left out.)
      float2 cb[NB];
      float2 t1h[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) t1h[h] = sm.tw1[i0 + h];
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        float2 d = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < 2; ++h) {  // conj(u_b[i]) w~_i = tw_b[i] w~_i / sqrt(L)
          const float2 t = beam_twiddle(t1h[h], k);
          d.x += t.x * wv[h].x - t.y * wv[h].y;
          d.y += t.x * wv[h].y + t.y * wv[h].x;
        }
        cb[k] = d;
      }
      float n0 = w0.x * w0.x + w0.y * w0.y + w1.x * w1.x + w1.y * w1.y;
      // The beam reductions and the norm interleaved, level by level.
#pragma unroll
      for (int o2 = 16; o2 > 0; o2 >>= 1) {
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          cb[k].x += __shfl_xor_sync(0xffffffffu, cb[k].x, o2);
          cb[k].y += __shfl_xor_sync(0xffffffffu, cb[k].y, o2);
        }
        n0 += __shfl_xor_sync(0xffffffffu, n0, o2);
      }
      // c_b / L: both u_b factors' 1 / sqrt(L); zero for the aliases.
#pragma unroll
      for (int k = 0; k < NB; ++k)
        cb[k] = k < nb ? make_float2(cb[k].x * inv_l, cb[k].y * inv_l) : make_float2(0.f, 0.f);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float mi = i0 + h < L ? 1.f : 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          const float2 t = beam_twiddle(t1h[h], k);  // u_b[i] = conj(t) / sqrt(L)
          wv[h].x -= mi * (cb[k].x * t.x + cb[k].y * t.y);
          wv[h].y -= mi * (cb[k].y * t.x - cb[k].x * t.y);
        }
      }
      float n1 = wv[0].x * wv[0].x + wv[0].y * wv[0].y + wv[1].x * wv[1].x + wv[1].y * wv[1].y;
      for (int o2 = 16; o2 > 0; o2 >>= 1) n1 += __shfl_xor_sync(0xffffffffu, n1, o2);
      const float sc = (a.use_net && n0 > 0.f && n1 > 1e-4f * n0) ? rsqrtf(n1) : 0.f;
      wv[0] = make_float2(wv[0].x * sc, wv[0].y * sc);
      wv[1] = make_float2(wv[1].x * sc, wv[1].y * sc);
      sm.qq[i0] = make_float4(wv[0].x, wv[0].x, wv[0].y, wv[0].y);   // kLmvMaxL = 64: lanes cover every i
      sm.qq[i0 + 1] = make_float4(wv[1].x, wv[1].x, wv[1].y, wv[1].y);
    }
    const bool has_w =
        __any_sync(0xffffffffu, wv[0].x != 0.f || wv[0].y != 0.f || wv[1].x != 0.f || wv[1].y != 0.f);

    float g[kG];
#pragma unroll
    for (int e = 0; e < kG; ++e) g[e] = 0.f;
    auto gram_add = [&](const float2 (&z)[K1]) {
      int e = 0;
#pragma unroll
      for (int r = 0; r < K1; ++r)
#pragma unroll
        for (int c = r; c < K1; ++c, e += 2) {
          g[e] = fmaf(z[r].x, z[c].x, fmaf(z[r].y, z[c].y, g[e]));      // z_r conj(z_c)
          if (r != c)  // the diagonal is real
            g[e + 1] = fmaf(z[r].y, z[c].x, fmaf(-z[r].x, z[c].y, g[e + 1]));
        }
    };
    float tr = 0.f;
    int ring_n = 0;
    for (int d = 0; d < n_d; ++d) {
      // Row d + 2 starts streaming; row d is the oldest copy in flight.
      if (d + 2 < n_d) {
        issue_row(d + 2);
        asm volatile("cp.async.wait_group 2;\n" ::: "memory");
      } else if (d + 1 < n_d) {
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");
      } else {
        asm volatile("cp.async.wait_group 0;\n" ::: "memory");
      }
      __syncwarp();
      const float2* yr = sm.rows[d % 3];

      // Trace of the covariance (times K): every sample weighted by the
      // number of subarrays that contain it.
      for (int t = lane; t < n_act; t += 32) {
        const float2 yv = yr[t];
        const int c = min(t, n_sub - 1) - max(0, t - L + 1) + 1;
        tr = fmaf(static_cast<float>(c), fmaf(yv.x, yv.x, yv.y * yv.y), tr);
      }

      // The beams' prefix sums P_b[t + 1] = sum_{t' <= t} tw_b[t'] y[t']: lane
      // l sums its run of C samples t = C l .. C l + C - 1 (C = 1, 2 or 4 for
      // apertures of at most 32, 64 or 128 channels; the row is zero past
      // n_act), then a warp scan of the run totals, beam by beam.
      auto scan_row = [&](auto run_len) {
        constexpr int C = decltype(run_len)::value;
        float2 yv[C], t1v[C];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          yv[c] = yr[C * lane + c];
          t1v[c] = sm.tw1[C * lane + c];
        }
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          float2 run = make_float2(0.f, 0.f), loc[C];
#pragma unroll
          for (int c = 0; c < C; ++c) {
            const float2 tw = beam_twiddle(t1v[c], k);
            run.x = fmaf(tw.x, yv[c].x, fmaf(-tw.y, yv[c].y, run.x));
            run.y = fmaf(tw.x, yv[c].y, fmaf(tw.y, yv[c].x, run.y));
            loc[c] = run;
          }
          float2 inc = run;
#pragma unroll
          for (int o2 = 1; o2 < 32; o2 <<= 1) {
            const float ux = __shfl_up_sync(0xffffffffu, inc.x, o2), uy = __shfl_up_sync(0xffffffffu, inc.y, o2);
            const float take = lane >= o2 ? 1.f : 0.f;
            inc.x = fmaf(take, ux, inc.x);
            inc.y = fmaf(take, uy, inc.y);
          }
          const float2 ex = make_float2(inc.x - run.x, inc.y - run.y);
#pragma unroll
          for (int c = 0; c < C; ++c) sm.pre[k][skw(C * lane + c + 1)] = make_float2(ex.x + loc[c].x, ex.y + loc[c].y);
        }
      };
      if (n_act <= 32)
        scan_row(std::integral_constant<int, 1>{});
      else if (n_act <= 64)
        scan_row(std::integral_constant<int, 2>{});
      else
        scan_row(std::integral_constant<int, 4>{});
      if (lane == 0)
#pragma unroll
        for (int k = 0; k < NB; ++k) sm.pre[k][0] = make_float2(0.f, 0.f);
      __syncwarp();

      // Beam projections of snapshot s without their 1 / sqrt(L) (applied to
      // G at the end): conj(tw_b[s]) (P_b[s + L] - P_b[s]).
      auto zbeams = [&](int s, float2 (&z)[K1]) {
        const float2 t1 = sm.tw1[s];
        const int hi_i = skw(s + L), lo_i = skw(s);
#pragma unroll
        for (int k = 0; k < NB; ++k) {
          const float2 hi = sm.pre[k][hi_i], lo = sm.pre[k][lo_i];
          const float2 df = make_float2(hi.x - lo.x, hi.y - lo.y);
          const float2 t = beam_twiddle(t1, k);
          z[k] = make_float2(fmaf(t.x, df.x, t.y * df.y), fmaf(t.x, df.y, -t.y * df.x));
        }
      };
      // w_q^H y_s by one lane: with q = (x, y), (x, x) * y and (y, y) * y
      // accumulate in FP32 pairs and conj(q) y = (A.x + B.y, A.y - B.x).
      auto zdir = [&](int s) {
        float2 A = make_float2(0.f, 0.f), B = A;
        const float2* ys = yr + s;
#pragma unroll 4
        for (int i = 0; i < L; ++i) {
          const float4 q = sm.qq[i];
          const float2 yv = ys[i];
          A = __ffma2_rn(make_float2(q.x, q.y), yv, A);
          B = __ffma2_rn(make_float2(q.z, q.w), yv, B);
        }
        return make_float2(A.x + B.y, A.y - B.x);
      };
      const int n_full = n_sub & ~31;
      for (int s0 = 0; s0 < n_full; s0 += 32) {
        float2 z[K1];
        zbeams(s0 + lane, z);
        z[NB] = has_w ? zdir(s0 + lane) : make_float2(0.f, 0.f);
        gram_add(z);
      }
      const int rem = n_sub - n_full;
      if (rem > 0) {
        float2 z[K1];
        const int s = n_full + min(lane, rem - 1);
        zbeams(s, z);
        z[NB] = make_float2(0.f, 0.f);
        if (has_w) {
          if (rem <= 4) {
            // A few snapshots: each one's w_q^H y_s by the whole warp.
            for (int r = 0; r < rem; ++r) {
              float2 acc = make_float2(0.f, 0.f);
              for (int i = lane; i < L; i += 32) {
                const float4 q = sm.qq[i];
                const float2 yv = yr[n_full + r + i];
                acc.x = fmaf(q.x, yv.x, fmaf(q.z, yv.y, acc.x));
                acc.y = fmaf(q.x, yv.y, fmaf(-q.z, yv.x, acc.y));
              }
              acc = warp_sum2(acc);
              if (lane == r) z[NB] = acc;
            }
          } else if (lane < rem) {
            z[NB] = zdir(s);
          }
        }
        if (ring_n + rem >= 32) {
          // One full pass: the ring's entries, then this row's first leftovers.
          const int take = 32 - ring_n;
          float2 zp[K1];
          const int src = lane - ring_n;   // this row's leftover in lanes ring_n ..
#pragma unroll
          for (int k = 0; k < K1; ++k) {
            const float v_x = __shfl_sync(0xffffffffu, z[k].x, src & 31), v_y = __shfl_sync(0xffffffffu, z[k].y, src & 31);
            zp[k] = lane < ring_n ? sm.ring[k][lane] : make_float2(v_x, v_y);
          }
          gram_add(zp);
          __syncwarp();
          // The rest of this row's leftovers start the ring again.
#pragma unroll
          for (int k = 0; k < K1; ++k) {
            const float v_x = __shfl_sync(0xffffffffu, z[k].x, (lane + take) & 31),
                        v_y = __shfl_sync(0xffffffffu, z[k].y, (lane + take) & 31);
            if (lane < rem - take) sm.ring[k][lane] = make_float2(v_x, v_y);
          }
          ring_n = rem - take;
        } else {
          if (lane < rem)
#pragma unroll
            for (int k = 0; k < K1; ++k) sm.ring[k][ring_n + lane] = z[k];
          ring_n += rem;
        }
      }
      __syncwarp();
    }
    if (ring_n > 0) {
      float2 z[K1];
#pragma unroll
      for (int k = 0; k < K1; ++k) z[k] = lane < ring_n ? sm.ring[k][lane] : make_float2(0.f, 0.f);
      gram_add(z);
    }
    for (int o2 = 16; o2 > 0; o2 >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o2);
    const float K = static_cast<float>(n_d * n_sub);

    // G, reduced across the warp by a reduce-scatter: after five halvings each
    // lane holds kPad / 32 finished entries, written straight to the record.
    // The projections of the subarray average and of 1 onto the basis ride
    // in the padding of the same reduce-scatter (the record keeps them right
    // after G).
    constexpr int kPad = (kG + 31) / 32 * 32;
    constexpr int kRed = kG + 2 * K1 + 2;
    static_assert(kRed <= kPad, "the projections fit the reduce-scatter's padding");
    float v[kPad];
    {
      // The beams' 1 / sqrt(L) per factor; entries of beams past nb are
      // replaced by the identity in stage 2.
      int e = 0;
#pragma unroll
      for (int r = 0; r < K1; ++r)
#pragma unroll
        for (int c = r; c < K1; ++c, e += 2) {
          const float f = (r < NB ? rs : 1.f) * (c < NB ? rs : 1.f);
          v[e] = g[e] * f;
          v[e + 1] = g[e + 1] * f;
        }
#pragma unroll
      for (int k = 0; k < K1; ++k) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          const int i = 2 * lane + h;
          const float mi = i < L ? 1.f : 0.f;   // the average is defined for i < L
          const float ax = (h ? av4.z : av4.x) * mi, ay = (h ? av4.w : av4.y) * mi;
          float2 q;   // basis vector k at i (beams past nb are unused by stage 2)
          if (k < NB) {
            const float2 t = beam_twiddle(sm.tw1[i], k);
            q = make_float2(t.x * rs, -t.y * rs);
          } else {
            q = wv[h];
          }
          acc.x += q.x * ax + q.y * ay;   // conj(q) abar
          acc.y += q.x * ay - q.y * ax;
        }
        v[kG + 2 * k] = acc.x;
        v[kG + 2 * k + 1] = acc.y;
      }
      float2 bw = make_float2(0.f, 0.f);   // w_q^H 1
      if (2 * lane < L) bw = make_float2(wv[0].x, -wv[0].y);
      if (2 * lane + 1 < L) bw = make_float2(bw.x + wv[1].x, bw.y - wv[1].y);
      v[kG + 2 * K1] = bw.x;
      v[kG + 2 * K1 + 1] = bw.y;
#pragma unroll
      for (int e2 = kRed; e2 < kPad; ++e2) v[e2] = 0.f;
    }
    int base = 0;
#pragma unroll
    for (int lvl = 0; lvl < 5; ++lvl) {
      const int m = 16 >> lvl;
      const int half = kPad >> (lvl + 1);
      const bool up = (lane & m) != 0;
#pragma unroll
      for (int i = 0; i < kPad / 2; ++i) {
        if (i >= half) break;
        const float send = up ? v[i] : v[i + half];
        const float keep = up ? v[i + half] : v[i];
        v[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
      }
      if (up) base += half;
    }
#pragma unroll
    for (int i = 0; i < kPad / 32; ++i)
      if (base + i < kRed) rec[base + i] = v[i];
    if (lane == 0) {
      float* tail = rec + kG;
      tail[2 * K1 + 2] = fmaxf(a.loading * (tr / K) * inv_l, 1e-20f);   // eps
      tail[2 * K1 + 3] = K;
      tail[2 * K1 + 4] = static_cast<float>(nb);
      tail[2 * K1 + 5] = has_w ? 1.f : 0.f;
      tail[2 * K1 + 6] = static_cast<float>(L);
      tail[2 * K1 + 7] = 1.f;   // record valid
      tail[2 * K1 + 8] = tr / K;
    }
    __syncwarp();
  }
}

// The level of each depth: the mean over lateral lines of ln tr(R) of the
// pixels with a record (the geometric mean of their covariance traces), one
// thread per (frame, depth). A strong point target raises tr(R) far above its
// depth's level in the pixels around it, where the subspace solve cannot form
// the deep nulls of the exact minimum variance; the level gate sends those
// pixels to the exact solver.
// One 128-thread block per (depth, frame): the threads stride over the
// lines, then a fixed tree (warp shuffles, then the four warps in order).
template <int NB>
__global__ void __launch_bounds__(128) lmv_level_kernel(const SubArgs a) {
  constexpr int K1 = NB + 1;
  constexpr int kG = K1 * (K1 + 1);
  __shared__ float s_sum[4];
  __shared__ int s_n[4];
  const int j = blockIdx.x;
  const long frame = blockIdx.y;
  const int n0 = a.n_pix / a.n1;
  float sum = 0.f;
  int n = 0;
  for (int i = threadIdx.x; i < n0; i += blockDim.x) {
    const float* tail = a.rec + (frame * a.n_pix + static_cast<long>(i) * a.n1 + j) * lmv_rec_floats(NB) + kG;
    if (tail[2 * K1 + 7] > 0.f && tail[2 * K1 + 8] > 0.f) {
      sum += logf(tail[2 * K1 + 8]);
      ++n;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum += __shfl_xor_sync(0xffffffffu, sum, o);
    n += __shfl_xor_sync(0xffffffffu, n, o);
  }
  if ((threadIdx.x & 31) == 0) {
    s_sum[threadIdx.x >> 5] = sum;
    s_n[threadIdx.x >> 5] = n;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    const float t = ((s_sum[0] + s_sum[1]) + s_sum[2]) + s_sum[3];
    const int c = s_n[0] + s_n[1] + s_n[2] + s_n[3];
    a.level[frame * a.n1 + j] = c > 0 ? t / static_cast<float>(c) : 0.f;
  }
}

// Stage 2, one thread per pixel: (G / K + eps I) c = Q^H 1, then the output
// n_act * cf * sum conj(c_k) (q_k^H abar) / sum c_k (1^H q_k). Pixels whose
// small factorisation fails go to the exact solver.
template <int NB>
__global__ void lmv_subspace_solve_kernel(const SubArgs a) {
  constexpr int K1 = NB + 1;
  constexpr int kG = K1 * (K1 + 1);
  const long row = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (row >= a.n_rows) return;
  const float* rec = a.rec + row * lmv_rec_floats(NB);
  const float* tail = rec + kG;
  if (!(tail[2 * K1 + 7] > 0.f)) return;  // gated, or n_act < 4
  const float eps = tail[2 * K1 + 2], Kf = tail[2 * K1 + 3];
  if (a.level && a.log_level_gate < INFINITY) {
    // Any pixel of the neighbourhood (the pixel itself by default) whose
    // tr(R) is above its depth's level by the gate sends this one to the
    // exact solver: with a neighbourhood, the flanks of a strong target's
    // response go with its peak.
    const long frame = row / a.n_pix;
    const int pix = static_cast<int>(row - frame * a.n_pix);
    const int n0 = a.n_pix / a.n1, line = pix / a.n1, depth = pix - line * a.n1;
    bool hot = false;
    for (int dl = -a.level_lines; dl <= a.level_lines && !hot; ++dl) {
      const int ln = line + dl;
      if (ln < 0 || ln >= n0) continue;
      for (int dd = -a.level_depths; dd <= a.level_depths; ++dd) {
        const int dp = depth + dd;
        if (dp < 0 || dp >= a.n1) continue;
        const float* nt = a.rec + (frame * a.n_pix + static_cast<long>(ln) * a.n1 + dp) * lmv_rec_floats(NB) + kG;
        const float tr = nt[2 * K1 + 8];
        if (nt[2 * K1 + 7] > 0.f && tr > 0.f && logf(tr) - a.level[frame * a.n1 + dp] > a.log_level_gate) {
          hot = true;
          break;
        }
      }
    }
    if (hot) {
      push_gated(a.gated_count, a.gated, a.gated_cap, static_cast<int>(tail[2 * K1 + 6]), pix, frame);
      if (a.stats) atomicAdd(a.stats, 1);
      return;
    }
  }
  const int nb = static_cast<int>(tail[2 * K1 + 4]);
  const bool has_w = tail[2 * K1 + 5] > 0.f;
  const int L = static_cast<int>(tail[2 * K1 + 6]);
  bool keep[K1];
#pragma unroll
  for (int k = 0; k < NB; ++k) keep[k] = k < nb;
  keep[NB] = has_w;
  float2 A[K1][K1];
  {
    int e = 0;
    const float ik = 1.0f / Kf;
#pragma unroll
    for (int r = 0; r < K1; ++r)
#pragma unroll
      for (int c = r; c < K1; ++c, e += 2) {
        float2 x = make_float2(rec[e] * ik, rec[e + 1] * ik);
        if (r == c) x = make_float2(x.x + eps, 0.f);
        if (!(keep[r] && keep[c])) x = (r == c) ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
        A[r][c] = x;
        A[c][r] = make_float2(x.x, -x.y);
      }
  }
  bool ok = true;
#pragma unroll
  for (int c = 0; c < K1; ++c) {
    float dsum = A[c][c].x;
#pragma unroll
    for (int k = 0; k < c; ++k) dsum -= A[c][k].x * A[c][k].x + A[c][k].y * A[c][k].y;
    ok = ok && dsum > 0.f;
    const float lc = sqrtf(fmaxf(dsum, 1e-30f));
    A[c][c] = make_float2(lc, 0.f);
    const float il = 1.0f / lc;
#pragma unroll
    for (int r = c + 1; r < K1; ++r) {
      float2 sv = A[r][c];
#pragma unroll
      for (int k = 0; k < c; ++k) {  // s -= L[r][k] conj(L[c][k])
        sv.x -= A[r][k].x * A[c][k].x + A[r][k].y * A[c][k].y;
        sv.y -= A[r][k].y * A[c][k].x - A[r][k].x * A[c][k].y;
      }
      A[r][c] = make_float2(sv.x * il, sv.y * il);
    }
  }
  // Right-hand side Q^H 1: sqrt(L) for the look direction, 0 for the other
  // beams, w_q^H 1 for the network's direction.
  float2 cv[K1];
#pragma unroll
  for (int r = 0; r < K1; ++r) {
    float2 sv = make_float2(0.f, 0.f);
    if (r == 0) sv = make_float2(sqrtf(static_cast<float>(L)), 0.f);
    if (r == NB && has_w) sv = make_float2(tail[2 * K1], tail[2 * K1 + 1]);
#pragma unroll
    for (int k = 0; k < r; ++k) {
      sv.x -= A[r][k].x * cv[k].x - A[r][k].y * cv[k].y;
      sv.y -= A[r][k].x * cv[k].y + A[r][k].y * cv[k].x;
    }
    cv[r] = make_float2(sv.x / A[r][r].x, sv.y / A[r][r].x);
  }
  // The gate on the network's share: with y = L^-1 Q^H 1, the subspace's
  // Capon output power is 1 / |y|^2, and that of the beams alone is
  // 1 / |y_beams|^2 (the leading block of the factor is the beams' factor),
  // so |y_w|^2 / |y|^2 is the fraction of the output power the network's
  // direction removed. Where that fraction is large the optimum lies well
  // outside the beams' span and the subspace solve may still miss it: the
  // pixel goes to the exact solver.
  bool share_ok = true;
  if (has_w) {
    float tot = 0.f;
#pragma unroll
    for (int k = 0; k < K1; ++k) tot += cv[k].x * cv[k].x + cv[k].y * cv[k].y;
    const float net = cv[NB].x * cv[NB].x + cv[NB].y * cv[NB].y;
    share_ok = !(net > a.share_gate * tot);
  }
#pragma unroll
  for (int r = K1 - 1; r >= 0; --r) {
    float2 sv = cv[r];
#pragma unroll
    for (int k = r + 1; k < K1; ++k) {  // s -= conj(L[k][r]) c_k
      sv.x -= A[k][r].x * cv[k].x + A[k][r].y * cv[k].y;
      sv.y -= A[k][r].x * cv[k].y - A[k][r].y * cv[k].x;
    }
    cv[r] = make_float2(sv.x / A[r][r].x, sv.y / A[r][r].x);
  }
  // num = sum_k conj(c_k) a_k, den = sum_k c_k conj(b_k) with b = Q^H 1.
  float2 num = make_float2(0.f, 0.f), den = make_float2(0.f, 0.f);
#pragma unroll
  for (int k = 0; k < K1; ++k) {
    if (!keep[k]) continue;
    const float2 ak = make_float2(tail[2 * k], tail[2 * k + 1]);
    num.x += cv[k].x * ak.x + cv[k].y * ak.y;
    num.y += cv[k].x * ak.y - cv[k].y * ak.x;
    float2 bk = make_float2(0.f, 0.f);
    if (k == 0) bk = make_float2(sqrtf(static_cast<float>(L)), 0.f);
    if (k == NB) bk = make_float2(tail[2 * K1], tail[2 * K1 + 1]);
    den.x += cv[k].x * bk.x + cv[k].y * bk.y;
    den.y += cv[k].y * bk.x - cv[k].x * bk.y;
  }
  const long frame = row / a.n_pix;
  const int pix = static_cast<int>(row - frame * a.n_pix);
  const float dn = den.x * den.x + den.y * den.y;
  if (!ok || !(dn > 1e-30f) || !share_ok) {
    push_gated(a.gated_count, a.gated, a.gated_cap, L, pix, frame);
    if (a.stats) atomicAdd(a.stats, 1);
    return;
  }
  const float4 meta = a.meta[row];
  const float scale = meta.y * meta.z / dn;   // n_act * cf * num / den
  a.out[frame * a.out_stride + pix] =
      make_float2((num.x * den.x + num.y * den.y) * scale, (num.y * den.x - num.x * den.y) * scale);
}

}  // namespace

int lmv_features_smem(int n_ch, int range_avg) {
  const int n_dmax = 2 * range_avg + 1;
  const int rs = n_ch <= 128 ? 128 : n_ch;
  return static_cast<int>(sizeof(float2) * kLmvWarps * n_dmax * rs + sizeof(int) * kLmvWarps * n_ch);
}

int launch_lmv_features(usx_ctx* ctx, const LmvLaunch& l) {
  LmvArgs a;
  a.y = l.y;
  a.points = l.points;
  a.n_ch = l.n_ch;
  a.n_pix = l.n_pix;
  a.n1 = l.n1;
  a.n_rows = static_cast<long>(l.n_frames) * l.n_pix;
  a.mv_subarray = l.mv_subarray;
  a.range_avg = l.range_avg;
  a.n_dmax = 2 * l.range_avg + 1;
  a.f_number = l.f_number;
  a.tukey_alpha = l.tukey_alpha;
  a.half_nm1 = l.half_nm1;
  a.pitch = l.pitch;
  a.rx_window = l.rx_window;
  a.cf = l.cf;
  a.feat16 = static_cast<__nv_bfloat16*>(l.feat16);
  a.feat32 = l.feat32;
  a.avg = l.avg;
  a.meta = l.meta;
  a.out = l.out;
  a.out_stride = l.out_stride;
  const int smem = lmv_features_smem(l.n_ch, l.range_avg);
  auto go = [&](auto kernel) -> int {
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(kernel), static_cast<size_t>(smem))) return rc_;
    int per_sm = 0;
    if (int rc_ = occupancy(reinterpret_cast<const void*>(kernel), 32 * kLmvWarps, static_cast<size_t>(smem), &per_sm))
      return rc_;
    const long want = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count * 8;
    const long need = (a.n_rows + kLmvWarps - 1) / kLmvWarps;
    prof_begin(ctx, "lmv_features_kernel");
    kernel<<<static_cast<unsigned>(std::max(1L, std::min(want, need))), 32 * kLmvWarps, smem, ctx->stream>>>(a);
    prof_end(ctx);
    USX_CHECK_LAUNCH("lmv_features_kernel");
    return USX_OK;
  };
  if (l.n_ch <= 128) return l.range_avg == 2 ? go(lmv_features_kernel<128, 5>) : go(lmv_features_kernel<128, 0>);
  return go(lmv_features_kernel<0, 0>);
}

int launch_lmv_apply(usx_ctx* ctx, const float* net, const float2* avg, const float4* meta, float2* out,
                     long out_stride, int n_pix, int n_frames, float gate, int* gated_count, int2* gated,
                     int gated_cap, int* stats) {
  ApplyArgs a;
  a.net = net;
  a.avg = avg;
  a.meta = meta;
  a.out = out;
  a.out_stride = out_stride;
  a.n_pix = n_pix;
  a.n_rows = static_cast<long>(n_frames) * n_pix;
  a.gate = gate;
  a.gated_count = gated_count;
  a.gated = gated;
  a.gated_cap = gated_cap;
  a.stats = stats;
  const long need = (a.n_rows + 7) / 8;
  const long want = static_cast<long>(ctx->sm_count) * 8 * 4;
  prof_begin(ctx, "lmv_apply_kernel");
  lmv_apply_kernel<<<static_cast<unsigned>(std::max(1L, std::min(want, need))), 256, 0, ctx->stream>>>(a);
  prof_end(ctx);
  USX_CHECK_LAUNCH("lmv_apply_kernel");
  return USX_OK;
}


int launch_lmv_subspace(usx_ctx* ctx, const LmvLaunch& l, const float* net, int n_beams, float loading,
                        float gate, int use_net, float share_gate, float level_gate, int level_lines,
                        int level_depths, float* level,
                        int* gated_count, int2* gated, int gated_cap, int* stats, float* rec) {
  SubArgs a;
  a.y = l.y;
  a.points = l.points;
  a.net = net;
  a.avg = l.avg;
  a.meta = l.meta;
  a.out = l.out;
  a.out_stride = l.out_stride;
  a.n_ch = l.n_ch;
  a.n_pix = l.n_pix;
  a.n1 = l.n1;
  a.n_dmax = 2 * l.range_avg + 1;
  a.n_rows = static_cast<long>(l.n_frames) * l.n_pix;
  a.range_avg = l.range_avg;
  a.n_beams = n_beams;
  a.f_number = l.f_number;
  a.tukey_alpha = l.tukey_alpha;
  a.half_nm1 = l.half_nm1;
  a.pitch = l.pitch;
  a.loading = loading;
  a.gate = gate;
  a.use_net = use_net;
  a.share_gate = share_gate;
  a.log_level_gate = level_gate < INFINITY ? logf(std::max(level_gate, 1e-30f)) : INFINITY;
  a.level = level_gate < INFINITY ? level : nullptr;
  a.level_lines = std::max(0, level_lines);
  a.level_depths = std::max(0, level_depths);
  a.rx_window = l.rx_window;
  a.gated_count = gated_count;
  a.gated = gated;
  a.gated_cap = gated_cap;
  a.stats = stats;
  a.rec = rec;
  if (l.n_ch > kSubMaxN || a.n_dmax > 9)
    return fail(USX_ERR_UNSUPPORTED, "learned-subspace refinement supports <= 128 channels, range average <= 4");
  auto go = [&](auto gram, auto solve, auto level_k, size_t per_warp) -> int {
    const int smem = static_cast<int>(per_warp * kSubWarps);
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(gram), static_cast<size_t>(smem))) return rc_;
    int per_sm = 0;
    if (int rc_ = occupancy(reinterpret_cast<const void*>(gram), 32 * kSubWarps, static_cast<size_t>(smem), &per_sm))
      return rc_;
    const long want = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count * 8;
    const long need = (a.n_rows + kSubWarps - 1) / kSubWarps;
    prof_begin(ctx, "lmv_subspace_gram_kernel");
    gram<<<static_cast<unsigned>(std::max(1L, std::min(want, need))), 32 * kSubWarps, smem, ctx->stream>>>(a);
    prof_end(ctx);
    USX_CHECK_LAUNCH("lmv_subspace_gram_kernel");
    if (a.level) {
      prof_begin(ctx, "lmv_level_kernel");
      level_k<<<dim3(static_cast<unsigned>(a.n1), static_cast<unsigned>(l.n_frames)), 128, 0, ctx->stream>>>(a);
      prof_end(ctx);
      USX_CHECK_LAUNCH("lmv_level_kernel");
    }
    prof_begin(ctx, "lmv_subspace_solve_kernel");
    solve<<<static_cast<unsigned>(ceil_div(a.n_rows, 128)), 128, 0, ctx->stream>>>(a);
    prof_end(ctx);
    USX_CHECK_LAUNCH("lmv_subspace_solve_kernel");
    return USX_OK;
  };
  switch (std::min(kSubMaxBeams, 1 + n_beams)) {
    case 1: return go(lmv_subspace_gram_kernel<1>, lmv_subspace_solve_kernel<1>, lmv_level_kernel<1>, sub_warp_bytes<1>());
    case 3: return go(lmv_subspace_gram_kernel<3>, lmv_subspace_solve_kernel<3>, lmv_level_kernel<3>, sub_warp_bytes<3>());
    case 5: return go(lmv_subspace_gram_kernel<5>, lmv_subspace_solve_kernel<5>, lmv_level_kernel<5>, sub_warp_bytes<5>());
    default: return go(lmv_subspace_gram_kernel<7>, lmv_subspace_solve_kernel<7>, lmv_level_kernel<7>, sub_warp_bytes<7>());
  }
}

int lmv_subspace_record_bytes(int n_beams) {
  return static_cast<int>(sizeof(float)) * lmv_rec_floats(std::min(kSubMaxBeams, 1 + std::max(0, n_beams)));
}

}  // namespace usxcu
