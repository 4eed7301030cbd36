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
  float4* meta;           // [row] (L, n_act, coherence factor, 0) (inference) or null
  float2* out;            // frames, written here for n_act < 4 (inference) or null
  long out_stride;
};

__global__ void __launch_bounds__(32 * kLmvWarps) lmv_features_kernel(const LmvArgs a) {
  extern __shared__ float2 lmv_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2* rows = lmv_smem + static_cast<size_t>(warp) * a.n_dmax * a.n_ch;
  int* act = reinterpret_cast<int*>(lmv_smem + static_cast<size_t>(kLmvWarps) * a.n_dmax * a.n_ch) + warp * a.n_ch;

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
        rows[d * a.n_ch + q] = Y[static_cast<long>(pix + dlo + d) * a.n_ch + act[q]];
      }
    } else {
      for (int q = lane; q < n_act; q += 32) rows[dc * a.n_ch + q] = Y[static_cast<long>(pix) * a.n_ch + act[q]];
    }
    __syncwarp();

    // Coherence factor terms over the active aperture of the centre row.
    float cre = 0.f, cim = 0.f, inc = 0.f;
    for (int q = lane; q < n_act; q += 32) {
      const float2 v = rows[dc * a.n_ch + q];
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

    // Diagonal sums rho[m] for m = lane, lane + 32.
    float rre[2] = {0.f, 0.f}, rim[2] = {0.f, 0.f};
#pragma unroll
    for (int s2 = 0; s2 < 2; ++s2) {
      const int m = lane + 32 * s2;
      if (m >= L) continue;
      const int lm1 = L - m - 1;
      for (int d = 0; d < n_d; ++d) {
        const float2* yr = rows + d * a.n_ch;
        float are = 0.f, aim = 0.f;
        for (int t = 0; t < n_act - m; ++t) {
          const int c = min(t, n_sub - 1) - max(0, t - lm1) + 1;
          const float2 p = yr[t + m], q = yr[t];
          const float w = static_cast<float>(c);
          are = fmaf(w, fmaf(p.x, q.x, p.y * q.y), are);
          aim = fmaf(w, fmaf(p.y, q.x, -p.x * q.y), aim);
        }
        rre[s2] += are;
        rim[s2] += aim;
      }
      rre[s2] /= static_cast<float>(L - m);
      rim[s2] /= static_cast<float>(L - m);
    }
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
        const float2* yr = rows + dc * a.n_ch + i;
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
      a.meta[row] = make_float4(static_cast<float>(L), static_cast<float>(n_act), cf_factor, 0.f);
  }
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
  int* gated_count;       // pixels sent to the exact solver
  int2* gated;            // their (pixel, frame)
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
      const int slot = atomicAdd(a.gated_count, 1);
      if (slot < a.gated_cap) a.gated[slot] = make_int2(pix, static_cast<int>(frame));
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

}  // namespace

int lmv_features_smem(int n_ch, int range_avg) {
  const int n_dmax = 2 * range_avg + 1;
  return static_cast<int>(sizeof(float2) * kLmvWarps * n_dmax * n_ch + sizeof(int) * kLmvWarps * n_ch);
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
  USX_CUDA(cudaFuncSetAttribute(lmv_features_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  int per_sm = 0;
  USX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lmv_features_kernel, 32 * kLmvWarps, smem));
  const long want = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count * 8;
  const long need = (a.n_rows + kLmvWarps - 1) / kLmvWarps;
  prof_begin(ctx, "lmv_features_kernel");
  lmv_features_kernel<<<static_cast<unsigned>(std::max(1L, std::min(want, need))), 32 * kLmvWarps, smem,
                        ctx->stream>>>(a);
  prof_end(ctx);
  USX_CHECK_LAUNCH("lmv_features_kernel");
  return USX_OK;
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

}  // namespace usxcu
