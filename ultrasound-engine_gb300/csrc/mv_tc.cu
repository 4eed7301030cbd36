// mv_tc.cu — minimum variance with the covariance on the tensor cores
// (reference beamformer.cpp:137-214 is the algorithm; this is the fast
// formulation, selected with USX_MV_TENSOR).
//
// Per pixel, with the active channels a_0 < ... < a_{n-1}, subarray length L,
// n_sub = n - L + 1 subarrays and n_d valid range offsets, the spatially
// smoothed covariance is R = X X^H / K with the K = n_d * n_sub snapshot
// columns x_(d,s)[i] = y_d[s + i] (Hankel in (s, i)). Stacking real and
// imaginary parts as interleaved rows of a 2L x K real matrix A, G = A A^T
// holds every product R needs:
//     R[a][b] = (G[2a][2b] + G[2a+1][2b+1]) + i (G[2a+1][2b] - G[2a][2b+1]).
// G is computed with mma.sync m16n8k16 (BF16 operands, FP32 accumulation),
// upper block-triangle only; A is never materialised: each fragment element is
// fetched from a per-pixel shared staging of the snapshots (scaled by a power
// of two so the scale is exact) in pairs laid out so that any two consecutive
// snapshot entries are one aligned 32-bit load.
//
// The Capon solve then runs in FP32 on the BF16 covariance R~ (+ diagonal
// loading from the exact FP32 trace), followed by one step of iterative
// refinement against the exact FP32 covariance, applied as R w = X (X^H w)/K
// directly from the FP32 snapshots (O(K L), no second covariance):
//     w0 = R~^-1 1,  r = 1 - (R + eps I) w0,  w = w0 + R~^-1 r.
// If the refined residual |1 - (R + eps I) w| / sqrt(L) still exceeds 1e-3,
// the pixel is re-solved in FP64 (covariance and Cholesky) on the GPU.
// Fallback rules are the reference's: n_active < 4 or a failed factorisation
// or |sum w| < 1e-30 give the DAS sum.
#include <cuda_bf16.h>

#include <algorithm>

#include "tc5.cuh"
#include "usx_internal.cuh"

namespace usxcu {

namespace {

constexpr int kTcWarps = 4;
constexpr int kTcMaxL = 64;
constexpr int kTcMaxCh = 128;
constexpr float kRefineGate = 1e-3f;

struct MvTcLayout {
  int n_ch, n_dmax, lmax;
  int words;          // 32-bit words per (part, parity, d) staging row
  size_t off_act, off_yf, off_yb, off_r, off_w, off_t, bytes;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~static_cast<size_t>(15); }

__host__ __device__ inline MvTcLayout mv_tc_layout(int n_ch, int n_dmax, int lmax) {
  MvTcLayout l;
  l.n_ch = n_ch;
  l.n_dmax = n_dmax;
  l.lmax = lmax;
  l.words = n_ch / 2 + 10;  // pairs up to index n_ch + 16 (masked subarray starts)
  size_t o = 0;
  l.off_act = o;  o = align16(o + sizeof(int) * n_ch);
  l.off_yf = o;   o = align16(o + sizeof(float2) * n_dmax * n_ch);
  l.off_yb = o;
  o = align16(o + (sizeof(uint32_t) * 4 * n_dmax * l.words > sizeof(float2) * n_dmax * n_ch
                       ? sizeof(uint32_t) * 4 * n_dmax * l.words
                       : sizeof(float2) * n_dmax * n_ch));  // bf16 pairs, then t_k
  l.off_r = o;    o = align16(o + sizeof(float2) * (lmax * (lmax + 1) / 2));
  l.off_w = o;    o = align16(o + sizeof(float2) * 2 * lmax);
  l.off_t = l.off_yb;
  l.bytes = o;
  return l;
}

__device__ __forceinline__ int tri(int i, int j) { return i * (i + 1) / 2 + j; }  // lower, i >= j

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat16 l = __float2bfloat16_rn(lo), h = __float2bfloat16_rn(hi);
  return static_cast<uint32_t>(__bfloat16_as_ushort(l)) | (static_cast<uint32_t>(__bfloat16_as_ushort(h)) << 16);
}

// Pair (v[q], v[q+1]) of part p (0 re, 1 im) of staged row d, as one word.
__device__ __forceinline__ uint32_t pair_at(const uint32_t* yb, int words, int n_dmax, int p, int d, int q) {
  const int par = q & 1;
  return yb[((p * 2 + par) * n_dmax + d) * words + (q >> 1)];
}

// Zero the halves of a pair whose subarray start s (for the low half) or s+1
// (for the high half) is past the last subarray.
__device__ __forceinline__ uint32_t mask_pair(uint32_t w, int s, int n_sub) {
  if (s + 1 < n_sub) return w;
  if (s < n_sub) return w & 0x0000ffffu;
  return 0u;
}

struct MvTcArgs {
  const float2* y;        // [frame][pix][n_ch] compounded channel samples
  const float* points;
  float2* out;
  long out_stride;
  float* acc_out;
  int n_ch, n_pix, n1;
  int mv_subarray, range_avg;
  float loading, f_number, tukey_alpha, half_nm1, pitch;
  int rx_window, cf, incoherent;
  int n_dmax, lmax;
  int* stats;             // [0] FP64 fallbacks, [1] factorisation failures
  int* fallback_count;    // pixels whose refined residual failed
  int2* fallback;         // (pixel, frame) of each, up to fallback_cap
  int fallback_cap;
  const int2* list;       // optional (pixel, frame) work list instead of all pixels
  const int* list_count;
  int list_cap;
  float* w_export;        // optional [frame * n_pix + pix][2 * kTcMaxL]: L w / sum(w)
  uint8_t* w_valid;       // [frame * n_pix + pix]: 1 where w_export holds a solve
};

// Training export of a solved pixel: L * w_i / sum(w) for i < L, zero beyond;
// lane-parallel over i = lane, lane + 32.
__device__ __forceinline__ void export_weights(const MvTcArgs& a, long row, int lane, int L, const float2 (&w)[2],
                                               float dre, float dim) {
  if (!a.w_export) return;
  const float den = dre * dre + dim * dim;
  float2* dst = reinterpret_cast<float2*>(a.w_export) + row * kTcMaxL;
#pragma unroll
  for (int s2 = 0; s2 < 2; ++s2) {
    const int i = lane + 32 * s2;
    float2 v = make_float2(0.f, 0.f);
    if (i < L && den > 0.f) {
      // w / d = w conj(d) / |d|^2
      v.x = (w[s2].x * dre + w[s2].y * dim) / den * static_cast<float>(L);
      v.y = (w[s2].y * dre - w[s2].x * dim) / den * static_cast<float>(L);
    }
    dst[i] = v;
  }
  if (lane == 0) a.w_valid[row] = den > 0.f ? 1 : 0;
}

// Marks a pixel with no Capon solve in the training export.
__device__ __forceinline__ void export_invalid(const MvTcArgs& a, long row, int tid) {
  if (!a.w_export) return;
  float2* dst = reinterpret_cast<float2*>(a.w_export) + row * kTcMaxL;
  for (int i = tid; i < kTcMaxL; i += 32) dst[i] = make_float2(0.f, 0.f);
  if (tid == 0) a.w_valid[row] = 0;
}

// One CTA (kTcWarps warps) per pixel; a grid-stride loop over pixels keeps
// the shared layout resident.
__global__ void __launch_bounds__(32 * kTcWarps) mv_tc_kernel(const MvTcArgs a) {
  extern __shared__ float4 tc_smem_raw[];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const MvTcLayout lay = mv_tc_layout(a.n_ch, a.n_dmax, a.lmax);
  char* base = reinterpret_cast<char*>(tc_smem_raw);
  int* act = reinterpret_cast<int*>(base + lay.off_act);
  float2* yf = reinterpret_cast<float2*>(base + lay.off_yf);
  uint32_t* yb = reinterpret_cast<uint32_t*>(base + lay.off_yb);
  float2* tk = reinterpret_cast<float2*>(base + lay.off_yb);   // aliases yb after the covariance
  float2* Rl = reinterpret_cast<float2*>(base + lay.off_r);
  float2* wv = reinterpret_cast<float2*>(base + lay.off_w);     // [0,L): w, [L,2L): r / partial sums
  __shared__ int s_misc[8];
  __shared__ float s_red[kTcWarps][4];

  const long n_items = a.list ? static_cast<long>(min(*a.list_count, a.list_cap)) : static_cast<long>(a.n_pix);
  for (long item = blockIdx.x; item < n_items; item += gridDim.x) {
    int pix;
    long frame;
    if (a.list) {
      const int2 pf = a.list[item];
      pix = pf.x;
      frame = pf.y;
    } else {
      pix = static_cast<int>(item);
      frame = blockIdx.y;
    }
    const long row = frame * a.n_pix + pix;
    const int j = pix % a.n1;
    const float px = __ldg(a.points + 3 * pix), pz = __ldg(a.points + 3 * pix + 2);
    const float2* Y = a.y + frame * static_cast<long>(a.n_pix) * a.n_ch;
    const float2* yc = Y + static_cast<long>(pix) * a.n_ch;
    __syncthreads();  // the previous pixel is done with the shared layout

    // Active channels (warp 0, ascending).
    if (warp == 0) {
      int n = 0;
      for (int c0 = 0; c0 < a.n_ch; c0 += 32) {
        const int ch = c0 + lane;
        bool on = false;
        if (ch < a.n_ch)
          on = aperture_weight((static_cast<float>(ch) - a.half_nm1) * a.pitch, px, pz, a.f_number, a.rx_window,
                               a.tukey_alpha) > 0.0f;
        const unsigned m = __ballot_sync(0xffffffffu, on);
        if (on) act[n + __popc(m & ((1u << lane) - 1u))] = ch;
        n += __popc(m);
      }
      if (lane == 0) s_misc[0] = n;
    }
    __syncthreads();
    const int n_act = s_misc[0];

    auto finish = [&](cplx out) {  // thread 0 only
      if (a.cf && n_act > 0) {
        cplx coh = mk(0.f, 0.f);
        float inc = 0.0f;
        for (int q = 0; q < n_act; ++q) {
          const float2 v = yc[act[q]];
          coh = cadd(coh, mk(v.x, v.y));
          inc += cnorm(mk(v.x, v.y));
        }
        out = cscale(out, (inc > 0.0f) ? cnorm(coh) / (static_cast<float>(n_act) * inc) : 0.0f);
      }
      if (a.incoherent)
        a.acc_out[frame * a.n_pix + pix] += cnorm(out);
      else
        a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
    };
    auto center_das = [&]() {
      cplx acc = mk(0.f, 0.f);
      for (int q = 0; q < n_act; ++q) {
        const float2 v = yc[act[q]];
        acc = cadd(acc, mk(v.x, v.y));
      }
      return acc;
    };
    if (n_act < 4) {
      if (warp == 0) export_invalid(a, row, tid);
      if (n_act == 0) {
        if (tid == 0 && !a.incoherent) a.out[frame * a.out_stride + pix] = make_float2(0.f, 0.f);
      } else if (tid == 0) {
        finish(center_das());
      }
      continue;
    }
    int L = a.mv_subarray;
    const int hi = max(2, n_act / 2);
    if (L < 2) L = 2;
    if (L > hi) L = hi;
    const int n_sub = n_act - L + 1;
    int dlo = -a.range_avg, dhi = a.range_avg;
    while (j + dlo < 0) ++dlo;
    while (j + dhi >= a.n1) --dhi;
    const int n_d = dhi - dlo + 1, dc = -dlo;
    const int K = n_d * n_sub;

    // Stage the FP32 snapshots, then find the largest magnitude.
    float amax = 0.0f;
    for (int k = tid; k < n_d * n_act; k += blockDim.x) {
      const int d = k / n_act, q = k - d * n_act;
      const float2 v = Y[static_cast<long>(pix + dlo + d) * a.n_ch + act[q]];
      yf[d * a.n_ch + q] = v;
      amax = fmaxf(amax, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    if (lane == 0) s_red[warp][0] = amax;
    __syncthreads();
    amax = fmaxf(fmaxf(s_red[0][0], s_red[1][0]), fmaxf(s_red[2][0], s_red[3][0]));
    if (!(amax > 0.0f)) {
      if (warp == 0) export_invalid(a, row, tid);
      if (tid == 0) finish(mk(0.f, 0.f));
      continue;
    }
    // Power-of-two scale: exact, brings the largest magnitude to [0.5, 1).
    int e2;
    frexpf(amax, &e2);
    const float sc = ldexpf(1.0f, -e2), inv_sc = ldexpf(1.0f, e2);
    for (int k = tid; k < n_d * n_act; k += blockDim.x) {
      const int d = k / n_act, q = k - d * n_act;
      const float2 v = yf[d * a.n_ch + q];
      yf[d * a.n_ch + q] = make_float2(v.x * sc, v.y * sc);
    }
    __syncthreads();
    // BF16 pair staging: word (p, par, d, w) = (v[2w+par], v[2w+par+1]) of part p.
    for (int k = tid; k < 4 * n_d * lay.words; k += blockDim.x) {
      const int w = k % lay.words;
      const int d = (k / lay.words) % n_d;
      const int pp = k / (lay.words * n_d);
      const int p = pp >> 1, par = pp & 1;
      const int q0 = 2 * w + par, q1 = q0 + 1;
      const float2 v0 = q0 < n_act ? yf[d * a.n_ch + q0] : make_float2(0.f, 0.f);
      const float2 v1 = q1 < n_act ? yf[d * a.n_ch + q1] : make_float2(0.f, 0.f);
      yb[(pp * a.n_dmax + d) * lay.words + w] = pack_bf16(p ? v0.y : v0.x, p ? v1.y : v1.x);
    }
    __syncthreads();

    // ---- G = A A^T on the tensor cores, upper block-triangle ----------------
    // Task = (row strip mt, chunk of up to 8 column tiles), spread over warps.
    const int g = lane >> 2, t4 = lane & 3;
    const int two_l = 2 * L;
    const int MT = (two_l + 15) / 16, NT = (two_l + 7) / 8;
    const int n_kstep = (n_sub + 15) / 16;
    const float inv_k = 1.0f / static_cast<float>(K);
    int task = 0;
    for (int mt = 0; mt < MT; ++mt) {
      for (int nt0 = 2 * mt; nt0 < NT; nt0 += 8, ++task) {
        if (task % kTcWarps != warp) continue;
        float acc[8][4];
#pragma unroll
        for (int x = 0; x < 8; ++x) acc[x][0] = acc[x][1] = acc[x][2] = acc[x][3] = 0.f;
        const int r0 = mt * 16 + g, r1 = r0 + 8;
        for (int d = 0; d < n_d; ++d) {
          for (int ks = 0; ks < n_kstep; ++ks) {
            const int s_lo = ks * 16 + 2 * t4, s_hi = s_lo + 8;
            uint32_t af[4];
            af[0] = r0 < two_l ? mask_pair(pair_at(yb, lay.words, a.n_dmax, r0 & 1, d, s_lo + (r0 >> 1)), s_lo, n_sub) : 0u;
            af[1] = r1 < two_l ? mask_pair(pair_at(yb, lay.words, a.n_dmax, r1 & 1, d, s_lo + (r1 >> 1)), s_lo, n_sub) : 0u;
            af[2] = r0 < two_l ? mask_pair(pair_at(yb, lay.words, a.n_dmax, r0 & 1, d, s_hi + (r0 >> 1)), s_hi, n_sub) : 0u;
            af[3] = r1 < two_l ? mask_pair(pair_at(yb, lay.words, a.n_dmax, r1 & 1, d, s_hi + (r1 >> 1)), s_hi, n_sub) : 0u;
#pragma unroll
            for (int x = 0; x < 8; ++x) {
              const int nt = nt0 + x;
              if (nt < NT) {
                const int c = nt * 8 + g;
                uint32_t b0 = 0u, b1 = 0u;
                if (c < two_l) {
                  b0 = mask_pair(pair_at(yb, lay.words, a.n_dmax, c & 1, d, s_lo + (c >> 1)), s_lo, n_sub);
                  b1 = mask_pair(pair_at(yb, lay.words, a.n_dmax, c & 1, d, s_hi + (c >> 1)), s_hi, n_sub);
                }
                mma16816(acc[x], af, b0, b1);
              }
            }
          }
        }
#pragma unroll
        for (int x = 0; x < 8; ++x) {
          const int nt = nt0 + x;
          if (nt >= NT) continue;
          const float o0 = __shfl_xor_sync(0xffffffffu, acc[x][0], 4);
          const float o1 = __shfl_xor_sync(0xffffffffu, acc[x][1], 4);
          const float o2 = __shfl_xor_sync(0xffffffffu, acc[x][2], 4);
          const float o3 = __shfl_xor_sync(0xffffffffu, acc[x][3], 4);
          if ((g & 1) == 0) {
            const int bcol = (nt * 8 + 2 * t4) >> 1;
            const int ar0 = r0 >> 1, ar1 = r1 >> 1;
            if (bcol < L && ar0 < L && bcol >= ar0)
              Rl[tri(bcol, ar0)] = make_float2((acc[x][0] + o1) * inv_k, -(o0 - acc[x][1]) * inv_k);
            if (bcol < L && ar1 < L && bcol >= ar1)
              Rl[tri(bcol, ar1)] = make_float2((acc[x][2] + o3) * inv_k, -(o2 - acc[x][3]) * inv_k);
          }
        }
      }
    }
    __syncthreads();  // covariance complete; yb is free (tk aliases it)

    // ---- exact trace and diagonal loading -----------------------------------
    float tr = 0.0f;
    for (int k = tid; k < K; k += blockDim.x) {
      const int d = k / n_sub, s = k - d * n_sub;
      const float2* x = yf + d * a.n_ch + s;
      for (int i = 0; i < L; ++i) tr = fmaf(x[i].x, x[i].x, fmaf(x[i].y, x[i].y, tr));
    }
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    if (lane == 0) s_red[warp][1] = tr;
    __syncthreads();
    tr = (s_red[0][1] + s_red[1][1] + s_red[2][1] + s_red[3][1]) * inv_k;
    const float eps = fmaxf(a.loading * tr / static_cast<float>(L), 1e-20f);
    for (int i = tid; i < L; i += blockDim.x) Rl[tri(i, i)].x += eps;
    __syncthreads();

    // ---- Cholesky of R~, right-looking; two threads per trailing row ------
    bool ok = true;
    for (int c = 0; c < L; ++c) {
      const float dgl = Rl[tri(c, c)].x;
      if (!(dgl > 0.0f)) {
        ok = false;
        break;
      }
      const float ljj = sqrtf(dgl), inv = 1.0f / ljj;
      __syncthreads();  // everyone has read the pivot
      if (tid == 0) Rl[tri(c, c)] = make_float2(ljj, 0.0f);
      for (int i = c + 1 + tid; i < L; i += blockDim.x) {
        const float2 v = Rl[tri(i, c)];
        Rl[tri(i, c)] = make_float2(v.x * inv, v.y * inv);
      }
      __syncthreads();
      for (int t = tid; t < 2 * (L - c - 1); t += blockDim.x) {
        const int i = c + 1 + (t >> 1);
        const float2 lic = Rl[tri(i, c)];
        const int row = i * (i + 1) / 2;
        for (int k = c + 1 + (t & 1); k <= i; k += 2) {
          const float2 lkc = Rl[k * (k + 1) / 2 + c];
          float2 v = Rl[row + k];
          v.x -= fmaf(lic.x, lkc.x, lic.y * lkc.y);
          v.y -= fmaf(lic.y, lkc.x, -lic.x * lkc.y);
          Rl[row + k] = v;
        }
      }
      __syncthreads();
    }
    if (!ok) {
      if (warp == 0) export_invalid(a, row, tid);
      if (tid == 0) {
        if (a.stats) atomicAdd(a.stats + 1, 1);
        finish(center_das());
      }
      continue;
    }

    // Triangular solves with the factor (warp 0), vector in registers.
    auto solve = [&](float2 (&v)[2]) {
      for (int c = 0; c < L; ++c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const float ljj = Rl[tri(c, c)].x;
          v[sl] = make_float2(v[sl].x / ljj, v[sl].y / ljj);
        }
        const float vx = __shfl_sync(0xffffffffu, sl ? v[1].x : v[0].x, own);
        const float vy = __shfl_sync(0xffffffffu, sl ? v[1].y : v[0].y, own);
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i > c && i < L) {
            const float2 l = Rl[tri(i, c)];
            v[s2].x -= fmaf(l.x, vx, -l.y * vy);
            v[s2].y -= fmaf(l.x, vy, l.y * vx);
          }
        }
      }
      for (int c = L - 1; c >= 0; --c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const float ljj = Rl[tri(c, c)].x;
          v[sl] = make_float2(v[sl].x / ljj, v[sl].y / ljj);
        }
        const float vx = __shfl_sync(0xffffffffu, sl ? v[1].x : v[0].x, own);
        const float vy = __shfl_sync(0xffffffffu, sl ? v[1].y : v[0].y, own);
        const int row = c * (c + 1) / 2;
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i < c) {
            const float2 l = Rl[row + i];
            v[s2].x -= fmaf(l.x, vx, l.y * vy);
            v[s2].y -= fmaf(l.x, vy, -l.y * vx);
          }
        }
      }
    };

    // r = 1 - (R + eps I) w for the w in wv[0, L), R = X X^H / K applied from
    // the FP32 snapshots as X (X^H w) / K; written to wv[L, 2L).
    auto residual = [&]() {
      for (int k = tid; k < K; k += blockDim.x) {  // t_k = x_k^H w
        const int d = k / n_sub, s = k - d * n_sub;
        const float2* x = yf + d * a.n_ch + s;
        float tre = 0.f, tim = 0.f;
        for (int i = 0; i < L; ++i) {
          const float2 xi = x[i], wi = wv[i];
          tre = fmaf(xi.x, wi.x, fmaf(xi.y, wi.y, tre));
          tim = fmaf(xi.x, wi.y, fmaf(-xi.y, wi.x, tim));
        }
        tk[k] = make_float2(tre, tim);
      }
      __syncthreads();
      {  // (R w)[i]: two threads per i split the snapshots
        const int i = tid >> 1, half = tid & 1;
        float are = 0.f, aim = 0.f;
        if (i < L) {
          for (int d = 0; d < n_d; ++d) {
            const float2* xr = yf + d * a.n_ch + i;
            const float2* tr_ = tk + d * n_sub;
            for (int s = half; s < n_sub; s += 2) {
              const float2 x = xr[s], t = tr_[s];
              are = fmaf(x.x, t.x, fmaf(-x.y, t.y, are));
              aim = fmaf(x.x, t.y, fmaf(x.y, t.x, aim));
            }
          }
        }
        are += __shfl_xor_sync(0xffffffffu, are, 1);
        aim += __shfl_xor_sync(0xffffffffu, aim, 1);
        if (i < L && half == 0) {
          const float2 wi = wv[i];
          wv[L + i] = make_float2(1.0f - fmaf(are, inv_k, eps * wi.x), -fmaf(aim, inv_k, eps * wi.y));
        }
      }
      __syncthreads();
    };

    float2 w[2];
    if (warp == 0) {
      w[0] = lane < L ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
      w[1] = lane + 32 < L ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
      solve(w);
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2)
        if (lane + 32 * s2 < L) wv[lane + 32 * s2] = w[s2];
    }
    __syncthreads();
    residual();
    // One refinement step: w = w0 + R~^-1 r.
    if (warp == 0) {
      float2 r[2];
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int i = lane + 32 * s2;
        r[s2] = i < L ? wv[L + i] : make_float2(0.f, 0.f);
      }
      solve(r);
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        w[s2].x += r[s2].x;
        w[s2].y += r[s2].y;
        if (lane + 32 * s2 < L) wv[lane + 32 * s2] = w[s2];
      }
    }
    __syncthreads();
    residual();
    if (warp == 0) {
      // The refined residual |1 - (R + eps I) w| / sqrt(L) gates the FP64 re-solve.
      float rn = 0.f;
#pragma unroll
      for (int s2 = 0; s2 < 2; ++s2) {
        const int i = lane + 32 * s2;
        if (i < L) {
          const float2 r = wv[L + i];
          rn = fmaf(r.x, r.x, fmaf(r.y, r.y, rn));
        }
      }
      for (int o = 16; o > 0; o >>= 1) rn += __shfl_xor_sync(0xffffffffu, rn, o);
      if (!(sqrtf(rn / static_cast<float>(L)) <= kRefineGate)) {
        if (lane == 0) {
          const int slot = atomicAdd(a.fallback_count, 1);
          if (slot < a.fallback_cap) a.fallback[slot] = make_int2(pix, static_cast<int>(frame));
          if (a.stats) atomicAdd(a.stats, 1);
        }
      } else {
        // out = sum conj(w_i) avg_i / sum w * n_act, avg from the centre row.
        float dre = 0.f, dim = 0.f, ore = 0.f, oim = 0.f;
#pragma unroll
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i < L) {
            dre += w[s2].x;
            dim += w[s2].y;
            float are = 0.f, aim = 0.f;
            for (int s = 0; s < n_sub; ++s) {
              const float2 v = yf[dc * a.n_ch + s + i];
              are += v.x;
              aim += v.y;
            }
            are = are * inv_sc / static_cast<float>(n_sub);
            aim = aim * inv_sc / static_cast<float>(n_sub);
            ore += w[s2].x * are + w[s2].y * aim;
            oim += w[s2].x * aim - w[s2].y * are;
          }
        }
        for (int o = 16; o > 0; o >>= 1) {
          dre += __shfl_xor_sync(0xffffffffu, dre, o);
          dim += __shfl_xor_sync(0xffffffffu, dim, o);
          ore += __shfl_xor_sync(0xffffffffu, ore, o);
          oim += __shfl_xor_sync(0xffffffffu, oim, o);
        }
        if (hypotf(dre, dim) < 1e-30f)
          export_invalid(a, row, lane);
        else
          export_weights(a, row, lane, L, w, dre, dim);
        if (lane == 0) {
          cplx out;
          if (hypotf(dre, dim) < 1e-30f)
            out = center_das();
          else
            out = cscale(cdiv_wide(mk(ore, oim), mk(dre, dim)), static_cast<float>(n_act));
          finish(out);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Warp-per-pixel minimum variance: every warp of the CTA solves its own
// pixels end to end (no CTA barriers), with shared memory sized for a class of
// pixels (largest L and active aperture of the class), so that short
// subarrays, the common case, pack many warps per SM.
//
// Per pixel: the active channels of the range rows in the smoothing window
// are staged once in FP32 (yf); R~ comes from the tcgen05 stage (r_pre), or
// from G = A A^T on mma.sync over BF16 pairs (yb, scaled by a power of two),
// or in FP32 from yf by the lag recurrence (cov_recur); the exact trace comes
// from the FP32 rows with each channel's subarray multiplicity; the Cholesky
// is blocked (chol_blocked); with a BF16 covariance the solves are followed
// by the refinement step and the refined-residual gate of mv_tc_kernel, with
// the FP32 one by nothing (one solve, as the reference).

constexpr int kWarpMvWarps = 4;

struct MvWarpLayout {
  int words;
  size_t off_act, off_yf, off_yb, off_r, off_w, off_p, bytes;  // per warp
};

// recur: the covariance by lags from the FP32 rows (no BF16 staging, no
// refinement, so no t_k either).
__host__ __device__ inline MvWarpLayout mv_warp_layout(int nmax, int n_dmax, int lmax, bool recur = false) {
  MvWarpLayout l;
  l.words = nmax / 2 + 10;
  size_t o = 0;
  l.off_act = o; o = align16(o + sizeof(int) * nmax);
  l.off_yf = o;  o = align16(o + sizeof(float2) * n_dmax * nmax);
  l.off_yb = o;  o = recur ? o : align16(o + sizeof(uint32_t) * 4 * n_dmax * l.words);  // also t_k after the covariance
  l.off_r = o;   o = align16(o + sizeof(float2) * (lmax * (lmax + 1) / 2));
  if (recur && n_dmax * nmax >= 4 * lmax) {
    // FP32: no refinement buffer, and the rows are dead once the covariance,
    // the trace and the centre row's average are formed, so the Cholesky's
    // panel takes their place.
    l.off_w = o;
    l.off_p = l.off_yf;
  } else {
    l.off_w = o;   o = recur ? o : align16(o + sizeof(float2) * 2 * lmax);  // refinement (BF16 only)
    l.off_p = o;   o = align16(o + sizeof(float2) * 4 * lmax);   // the Cholesky's panel, transposed
  }
  l.bytes = o;
  return l;
}

// Cholesky of the packed lower triangle Rl (L <= 64) by one warp, blocked
// right-looking: each block of four columns is factored as a panel (columns
// in turn, lanes over rows), copied transposed into P[k][0..3], and the
// trailing triangle takes one rank-4 update, R[i][k] -= sum_c l_ic conj(l_kc),
// with lanes over rows: lane l walks row k0 + l and, when the trailing part
// has more than 32 rows, row L - 1 - l, so that every lane updates about
// n + 1 entries (n trailing rows). Against one trailing row per step with
// lanes over columns, a quarter of the passes over the triangle and no lane
// idles on short rows. False on a non-positive pivot.
template <int kSlots>
__device__ bool chol_blocked(float2* Rl, float2* P, int L, int lane) {
  for (int c0 = 0; c0 < L; c0 += 4) {
    const int nb = min(4, L - c0);
    for (int c = c0; c < c0 + nb; ++c) {
      const float dgl = Rl[tri(c, c)].x;
      if (!(dgl > 0.0f)) return false;
      const float ljj = sqrtf(dgl), inv = 1.0f / ljj;
      for (int i = c + 1 + lane; i < L; i += 32) {
        const float2 v = Rl[tri(i, c)];
        Rl[tri(i, c)] = make_float2(v.x * inv, v.y * inv);
      }
      __syncwarp();
      if (lane == 0) Rl[tri(c, c)] = make_float2(ljj, 0.0f);
      for (int cc = c + 1; cc < c0 + nb; ++cc) {
        const float2 lk = Rl[tri(cc, c)];
        for (int i = cc + lane; i < L; i += 32) {
          const float2 li = Rl[tri(i, c)];
          float2 v = Rl[tri(i, cc)];
          v.x = fmaf(-li.x, lk.x, fmaf(-li.y, lk.y, v.x));
          v.y = fmaf(-li.y, lk.x, fmaf(li.x, lk.y, v.y));
          Rl[tri(i, cc)] = v;
        }
      }
      __syncwarp();
    }
    const int k0 = c0 + nb;
    if (k0 >= L) break;
    for (int k = k0 + lane; k < L; k += 32)
#pragma unroll
      for (int j = 0; j < 4; ++j) P[4 * k + j] = Rl[tri(k, c0 + j)];
    __syncwarp();
    const int n = L - k0;
#pragma unroll 1
    for (int h = 0; h < kSlots; ++h) {
      const int i = h == 0 ? k0 + lane : L - 1 - lane;
      if (h == 0 ? lane >= n : lane > n - 33) continue;
      const float4* pi = reinterpret_cast<const float4*>(P + 4 * i);
      const float4 ia = pi[0], ib = pi[1];
      float2* row = Rl + tri(i, 0);
      for (int k = k0; k <= i; ++k) {
        const float4* pk = reinterpret_cast<const float4*>(P + 4 * k);
        const float4 ka = pk[0], kb = pk[1];
        float2 v = row[k];
        v.x = fmaf(-ia.x, ka.x, fmaf(-ia.y, ka.y, v.x));
        v.y = fmaf(-ia.y, ka.x, fmaf(ia.x, ka.y, v.y));
        v.x = fmaf(-ia.z, ka.z, fmaf(-ia.w, ka.w, v.x));
        v.y = fmaf(-ia.w, ka.z, fmaf(ia.z, ka.w, v.y));
        v.x = fmaf(-ib.x, kb.x, fmaf(-ib.y, kb.y, v.x));
        v.y = fmaf(-ib.y, kb.x, fmaf(ib.x, kb.y, v.y));
        v.x = fmaf(-ib.z, kb.z, fmaf(-ib.w, kb.w, v.x));
        v.y = fmaf(-ib.w, kb.z, fmaf(ib.z, kb.w, v.y));
        row[k] = v;
      }
    }
    __syncwarp();
  }
  return true;
}

struct MvWarpArgs {
  MvTcArgs base;          // geometry, outputs, FP64 list, export
  int lmax, nmax;         // class limits (shared-memory sizing)
  const int* pix_list;    // class mode: pixels of the class, every frame
  int n_list, n_frames;
  const int2* pair_list;  // pair mode: (pixel, frame) with a device count
  const int* pair_count;
  int pair_cap;
  int* overflow_count;    // pixels beyond the class limits (solved by mv_tc_kernel)
  int2* overflow;
  int overflow_cap;
  // Class mode in chunks: items [item_begin, item_end) (item_end 0: all), and
  // their covariances R~ from mv_cov_tc5_kernel ([item - item_begin][r_stride],
  // packed lower triangle), or null to form them here on mma.sync.
  long item_begin, item_end;
  const float2* r_pre;
  const uint8_t* r_flag;  // [item - item_begin]: 1 where r_pre holds the pixel's R~
  int r_stride;
  // 1: R~ in FP32 from the rows by the lag recurrence and one FP32 solve (no
  // refinement, no FP64 re-solve: the reference's precision).
  int cov_recur;
};

template <int kSlots, bool kRecur>
__global__ void __launch_bounds__(32 * kWarpMvWarps) mv_warp_kernel(const MvWarpArgs wa) {
  extern __shared__ float4 mvw_smem_raw[];
  const MvTcArgs& a = wa.base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const MvWarpLayout lay = mv_warp_layout(wa.nmax, a.n_dmax, wa.lmax, kRecur);
  char* base = reinterpret_cast<char*>(mvw_smem_raw) + warp * lay.bytes;
  int* act = reinterpret_cast<int*>(base + lay.off_act);
  float2* yf = reinterpret_cast<float2*>(base + lay.off_yf);
  uint32_t* yb = reinterpret_cast<uint32_t*>(base + lay.off_yb);
  float2* tk = reinterpret_cast<float2*>(base + lay.off_yb);
  float2* Rl = reinterpret_cast<float2*>(base + lay.off_r);
  float2* wv = reinterpret_cast<float2*>(base + lay.off_w);
  const int nmax = wa.nmax;

  const long n_items = wa.pair_list ? static_cast<long>(min(*wa.pair_count, wa.pair_cap))
                                    : (wa.item_end > 0 ? wa.item_end : static_cast<long>(wa.n_list) * wa.n_frames);
  for (long item = (wa.pair_list ? 0 : wa.item_begin) + static_cast<long>(blockIdx.x) * kWarpMvWarps + warp;
       item < n_items; item += static_cast<long>(gridDim.x) * kWarpMvWarps) {
    int pix;
    long frame;
    if (wa.pair_list) {
      const int2 pf = wa.pair_list[item];
      pix = pf.x;
      frame = pf.y;
    } else {
      frame = item / wa.n_list;
      pix = wa.pix_list[item - frame * wa.n_list];
    }
    const long row = frame * a.n_pix + pix;
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
      if (on && n_act + __popc(m & ((1u << lane) - 1u)) < nmax) act[n_act + __popc(m & ((1u << lane) - 1u))] = ch;
      n_act += __popc(m);
    }
    __syncwarp();
    auto finish = [&](cplx out, float cre, float cim, float inc) {  // lane 0
      if (a.cf && n_act > 0) {
        const float coh = cre * cre + cim * cim;
        out = cscale(out, (inc > 0.0f) ? coh / (static_cast<float>(n_act) * inc) : 0.0f);
      }
      if (a.incoherent)
        a.acc_out[frame * a.n_pix + pix] += cnorm(out);
      else
        a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
    };
    int L = a.mv_subarray;
    const int hi = max(2, n_act / 2);
    if (L < 2) L = 2;
    if (L > hi) L = hi;
    if (n_act > nmax || L > wa.lmax) {
      if (lane == 0 && wa.overflow_count) {
        const int slot = atomicAdd(wa.overflow_count, 1);
        if (slot < wa.overflow_cap) wa.overflow[slot] = make_int2(pix, static_cast<int>(frame));
      }
      continue;
    }
    const float2* yc = Y + static_cast<long>(pix) * a.n_ch;
    if (n_act < 4) {
      export_invalid(a, row, lane);
      if (lane == 0) {
        // The reference's rule: the DAS sum, channels in ascending order.
        cplx acc = mk(0.f, 0.f);
        float inc = 0.0f;
        for (int q = 0; q < n_act; ++q) {
          const float2 v = yc[act[q]];
          acc = cadd(acc, mk(v.x, v.y));
          inc += cnorm(mk(v.x, v.y));
        }
        if (n_act == 0) {
          if (!a.incoherent) a.out[frame * a.out_stride + pix] = make_float2(0.f, 0.f);
        } else {
          finish(acc, acc.re, acc.im, inc);
        }
      }
      continue;
    }
    const int n_sub = n_act - L + 1;
    int dlo = -a.range_avg, dhi = a.range_avg;
    while (j + dlo < 0) ++dlo;
    while (j + dhi >= a.n1) --dhi;
    const int n_d = dhi - dlo + 1, dc = -dlo;
    const int K = n_d * n_sub;

    // FP32 rows of the active channels, largest magnitude.
    float amax = 0.0f;
    for (int k = lane; k < n_d * n_act; k += 32) {
      const int d = k / n_act, q = k - d * n_act;
      const float2 v = Y[static_cast<long>(pix + dlo + d) * a.n_ch + act[q]];
      yf[d * nmax + q] = v;
      amax = fmaxf(amax, fmaxf(fabsf(v.x), fabsf(v.y)));
    }
    for (int o = 16; o > 0; o >>= 1) amax = fmaxf(amax, __shfl_xor_sync(0xffffffffu, amax, o));
    __syncwarp();
    // Coherence-factor terms and the DAS sum of the centre row (ascending in
    // lanes, then a fixed tree).
    float cre = 0.f, cim = 0.f, inc = 0.f;
    if (a.cf) {
      for (int q = lane; q < n_act; q += 32) {
        const float2 v = yf[dc * nmax + q];
        cre += v.x;
        cim += v.y;
        inc += v.x * v.x + v.y * v.y;
      }
      for (int o = 16; o > 0; o >>= 1) {
        cre += __shfl_xor_sync(0xffffffffu, cre, o);
        cim += __shfl_xor_sync(0xffffffffu, cim, o);
        inc += __shfl_xor_sync(0xffffffffu, inc, o);
      }
    }
    if (!(amax > 0.0f)) {
      export_invalid(a, row, lane);
      if (lane == 0) finish(mk(0.f, 0.f), cre, cim, inc);
      continue;
    }
    int e2;
    frexpf(amax, &e2);
    const float sc = ldexpf(1.0f, -e2), sc2 = ldexpf(1.0f, -2 * e2);
    const float inv_k = 1.0f / static_cast<float>(K);
    if constexpr (kRecur) {
      // R~[i][k] = sum_d sum_{s < n_sub} x_d[s + i] conj(x_d[s + k]) by
      // diagonals (lag m = i - k): the first entry of a diagonal in full,
      // then R~[i + 1][k + 1] = R~[i][k] - x[i] conj(x[k]) + x[n_sub + i]
      // conj(x[n_sub + k]) summed over the rows, 2 n_d products per entry
      // instead of K. Lane l takes m = l and, for L > 32, m = 63 - l (every
      // lane then walks about L entries).
      const float f = sc2 * inv_k;
#pragma unroll 1
      for (int h = 0; h < kSlots; ++h) {
        const int m = h == 0 ? lane : 63 - lane;
        if (m >= L || (h == 1 && m < 32)) continue;
        // Four independent partial sums (snapshot parity x real/imaginary)
        // keep the FMA chains short.
        float re0 = 0.f, im0 = 0.f, re1 = 0.f, im1 = 0.f;
        for (int d = 0; d < n_d; ++d) {
          const float2* x = yf + d * nmax;
          int s = 0;
          for (; s + 1 < n_sub; s += 2) {
            const float2 p = x[s + m], q = x[s], pb = x[s + 1 + m], qb = x[s + 1];
            re0 = fmaf(p.x, q.x, fmaf(p.y, q.y, re0));
            im0 = fmaf(p.y, q.x, fmaf(-p.x, q.y, im0));
            re1 = fmaf(pb.x, qb.x, fmaf(pb.y, qb.y, re1));
            im1 = fmaf(pb.y, qb.x, fmaf(-pb.x, qb.y, im1));
          }
          if (s < n_sub) {
            const float2 p = x[s + m], q = x[s];
            re0 = fmaf(p.x, q.x, fmaf(p.y, q.y, re0));
            im0 = fmaf(p.y, q.x, fmaf(-p.x, q.y, im0));
          }
        }
        float re = re0 + re1, im = im0 + im1;
        Rl[tri(m, 0)] = make_float2(re * f, im * f);
        for (int j = 1; j + m < L; ++j) {
          // The step's row sums (entering minus leaving product), rows in
          // two interleaved partial sums.
          float ar = 0.f, ai = 0.f, br = 0.f, bi = 0.f;
          const float2* x = yf;
          int d = 0;
          for (; d + 1 < n_d; d += 2, x += 2 * nmax) {
            const float2 p1 = x[n_sub + m + j - 1], q1 = x[n_sub + j - 1];
            const float2 p0 = x[m + j - 1], q0 = x[j - 1];
            const float2* y = x + nmax;
            const float2 r1 = y[n_sub + m + j - 1], s1 = y[n_sub + j - 1];
            const float2 r0 = y[m + j - 1], s0 = y[j - 1];
            ar += fmaf(p1.x, q1.x, p1.y * q1.y) - fmaf(p0.x, q0.x, p0.y * q0.y);
            ai += fmaf(p1.y, q1.x, -p1.x * q1.y) - fmaf(p0.y, q0.x, -p0.x * q0.y);
            br += fmaf(r1.x, s1.x, r1.y * s1.y) - fmaf(r0.x, s0.x, r0.y * s0.y);
            bi += fmaf(r1.y, s1.x, -r1.x * s1.y) - fmaf(r0.y, s0.x, -r0.x * s0.y);
          }
          if (d < n_d) {
            const float2 p1 = x[n_sub + m + j - 1], q1 = x[n_sub + j - 1];
            const float2 p0 = x[m + j - 1], q0 = x[j - 1];
            ar += fmaf(p1.x, q1.x, p1.y * q1.y) - fmaf(p0.x, q0.x, p0.y * q0.y);
            ai += fmaf(p1.y, q1.x, -p1.x * q1.y) - fmaf(p0.y, q0.x, -p0.x * q0.y);
          }
          re += ar + br;
          im += ai + bi;
          Rl[tri(m + j, j)] = make_float2(re * f, im * f);
        }
      }
      __syncwarp();
    } else {
    if (wa.r_pre && wa.r_flag[item - wa.item_begin]) {
      // R~ from the tensor-core stage (same scale, same packing).
      const float2* src = wa.r_pre + (item - wa.item_begin) * wa.r_stride;
      for (int e = lane; e < L * (L + 1) / 2; e += 32) Rl[e] = src[e];
      __syncwarp();
    } else {
    // BF16 pairs: word (p, par, d, w) = (v[2w+par], v[2w+par+1]) of part p, scaled.
    const int words = lay.words;
    for (int k = lane; k < 4 * n_d * words; k += 32) {
      const int w = k % words;
      const int rest = k / words;
      const int d = rest % n_d, pp = rest / n_d;
      const int p = pp >> 1, par = pp & 1;
      const int q0 = 2 * w + par, q1 = q0 + 1;
      const float2 v0 = q0 < n_act ? yf[d * nmax + q0] : make_float2(0.f, 0.f);
      const float2 v1 = q1 < n_act ? yf[d * nmax + q1] : make_float2(0.f, 0.f);
      yb[(pp * a.n_dmax + d) * words + w] = pack_bf16((p ? v0.y : v0.x) * sc, (p ? v1.y : v1.x) * sc);
    }
    __syncwarp();

    // ---- R~ = A A^T / K on the tensor cores (upper block-triangle) --------
    const int g = lane >> 2, t4 = lane & 3;
    const int two_l = 2 * L;
    const int MT = (two_l + 15) / 16, NT = (two_l + 7) / 8;
    const int n_kstep = (n_sub + 15) / 16;
    for (int mt = 0; mt < MT; ++mt) {
      for (int nt0 = 2 * mt; nt0 < NT; nt0 += 8) {
        float acc[8][4];
#pragma unroll
        for (int x = 0; x < 8; ++x) acc[x][0] = acc[x][1] = acc[x][2] = acc[x][3] = 0.f;
        const int r0 = mt * 16 + g, r1 = r0 + 8;
        for (int d = 0; d < n_d; ++d) {
          for (int ks = 0; ks < n_kstep; ++ks) {
            const int s_lo = ks * 16 + 2 * t4, s_hi = s_lo + 8;
            uint32_t af[4];
            af[0] = r0 < two_l ? mask_pair(pair_at(yb, words, a.n_dmax, r0 & 1, d, s_lo + (r0 >> 1)), s_lo, n_sub) : 0u;
            af[1] = r1 < two_l ? mask_pair(pair_at(yb, words, a.n_dmax, r1 & 1, d, s_lo + (r1 >> 1)), s_lo, n_sub) : 0u;
            af[2] = r0 < two_l ? mask_pair(pair_at(yb, words, a.n_dmax, r0 & 1, d, s_hi + (r0 >> 1)), s_hi, n_sub) : 0u;
            af[3] = r1 < two_l ? mask_pair(pair_at(yb, words, a.n_dmax, r1 & 1, d, s_hi + (r1 >> 1)), s_hi, n_sub) : 0u;
#pragma unroll
            for (int x = 0; x < 8; ++x) {
              const int nt = nt0 + x;
              if (nt < NT) {
                const int c = nt * 8 + g;
                uint32_t b0 = 0u, b1 = 0u;
                if (c < two_l) {
                  b0 = mask_pair(pair_at(yb, words, a.n_dmax, c & 1, d, s_lo + (c >> 1)), s_lo, n_sub);
                  b1 = mask_pair(pair_at(yb, words, a.n_dmax, c & 1, d, s_hi + (c >> 1)), s_hi, n_sub);
                }
                mma16816(acc[x], af, b0, b1);
              }
            }
          }
        }
#pragma unroll
        for (int x = 0; x < 8; ++x) {
          const int nt = nt0 + x;
          if (nt >= NT) continue;
          const float o0 = __shfl_xor_sync(0xffffffffu, acc[x][0], 4);
          const float o1 = __shfl_xor_sync(0xffffffffu, acc[x][1], 4);
          const float o2 = __shfl_xor_sync(0xffffffffu, acc[x][2], 4);
          const float o3 = __shfl_xor_sync(0xffffffffu, acc[x][3], 4);
          if ((g & 1) == 0) {
            const int bcol = (nt * 8 + 2 * t4) >> 1;
            const int ar0 = r0 >> 1, ar1 = r1 >> 1;
            if (bcol < L && ar0 < L && bcol >= ar0)
              Rl[tri(bcol, ar0)] = make_float2((acc[x][0] + o1) * inv_k, -(o0 - acc[x][1]) * inv_k);
            if (bcol < L && ar1 < L && bcol >= ar1)
              Rl[tri(bcol, ar1)] = make_float2((acc[x][2] + o3) * inv_k, -(o2 - acc[x][3]) * inv_k);
          }
        }
      }
    }
    __syncwarp();
    }  // covariance on mma.sync
    }  // BF16 covariances

    // ---- exact trace: channel t of a row appears in c(t) subarrays -------
    float tr = 0.0f;
    for (int k = lane; k < n_d * n_act; k += 32) {
      const int d = k / n_act, t = k - d * n_act;
      const int c = min(t, n_sub - 1) - max(0, t - L + 1) + 1;
      const float2 v = yf[d * nmax + t];
      tr = fmaf(static_cast<float>(c), fmaf(v.x, v.x, v.y * v.y), tr);
    }
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    tr *= sc2 * inv_k;
    const float eps = fmaxf(a.loading * tr / static_cast<float>(L), 1e-20f);
    for (int i = lane; i < L; i += 32) Rl[tri(i, i)].x += eps;
    __syncwarp();

    // ---- Cholesky (blocked, rank-4 trailing updates) ---------------------
    // The centre row's subarray average, before the Cholesky may reuse the
    // rows' space (FP32 instance).
    float avg_re[kSlots], avg_im[kSlots];
    {
      const float inv_nsub = 1.0f / static_cast<float>(n_sub);
#pragma unroll
      for (int s2 = 0; s2 < kSlots; ++s2) {
        const int i = lane + 32 * s2;
        float are = 0.f, aim = 0.f;
        if (i < L) {
          const float2* yr = yf + dc * nmax + i;
          for (int s = 0; s < n_sub; ++s) {
            are += yr[s].x;
            aim += yr[s].y;
          }
          are *= inv_nsub;
          aim *= inv_nsub;
        }
        avg_re[s2] = are;
        avg_im[s2] = aim;
      }
    }
    __syncwarp();
    const bool ok = chol_blocked<kSlots>(Rl, reinterpret_cast<float2*>(base + lay.off_p), L, lane);
    if (!ok) {
      export_invalid(a, row, lane);
      if (lane == 0) {
        if (a.stats) atomicAdd(a.stats + 1, 1);
        cplx acc = mk(0.f, 0.f);
        for (int q = 0; q < n_act; ++q) acc = cadd(acc, mk(yc[act[q]].x, yc[act[q]].y));
        finish(acc, cre, cim, inc);
      }
      continue;
    }

    auto solve = [&](float2 (&v)[kSlots]) {
      for (int c = 0; c < L; ++c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const float ljj = Rl[tri(c, c)].x;
          v[kSlots == 1 ? 0 : sl] = make_float2(v[kSlots == 1 ? 0 : sl].x / ljj, v[kSlots == 1 ? 0 : sl].y / ljj);
        }
        const float vx = __shfl_sync(0xffffffffu, (kSlots > 1 && sl) ? v[kSlots - 1].x : v[0].x, own);
        const float vy = __shfl_sync(0xffffffffu, (kSlots > 1 && sl) ? v[kSlots - 1].y : v[0].y, own);
#pragma unroll
        for (int s2 = 0; s2 < kSlots; ++s2) {
          const int i = lane + 32 * s2;
          if (i > c && i < L) {
            const float2 l = Rl[tri(i, c)];
            v[s2].x -= fmaf(l.x, vx, -l.y * vy);
            v[s2].y -= fmaf(l.x, vy, l.y * vx);
          }
        }
      }
      for (int c = L - 1; c >= 0; --c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const float ljj = Rl[tri(c, c)].x;
          v[kSlots == 1 ? 0 : sl] = make_float2(v[kSlots == 1 ? 0 : sl].x / ljj, v[kSlots == 1 ? 0 : sl].y / ljj);
        }
        const float vx = __shfl_sync(0xffffffffu, (kSlots > 1 && sl) ? v[kSlots - 1].x : v[0].x, own);
        const float vy = __shfl_sync(0xffffffffu, (kSlots > 1 && sl) ? v[kSlots - 1].y : v[0].y, own);
        const int rowc = c * (c + 1) / 2;
#pragma unroll
        for (int s2 = 0; s2 < kSlots; ++s2) {
          const int i = lane + 32 * s2;
          if (i < c) {
            const float2 l = Rl[rowc + i];
            v[s2].x -= fmaf(l.x, vx, l.y * vy);
            v[s2].y -= fmaf(l.x, vy, -l.y * vx);
          }
        }
      }
    };
    // r = 1 - (R + eps I) w (scaled domain) for w in wv[0, L); into wv[L, 2L).
    auto residual = [&]() {
      for (int k = lane; k < K; k += 32) {  // t_k = x_k^H w
        const int d = k / n_sub, s = k - d * n_sub;
        const float2* x = yf + d * nmax + s;
        float tre = 0.f, tim = 0.f;
        for (int i = 0; i < L; ++i) {
          const float2 xi = x[i], wi = wv[i];
          tre = fmaf(xi.x, wi.x, fmaf(xi.y, wi.y, tre));
          tim = fmaf(xi.x, wi.y, fmaf(-xi.y, wi.x, tim));
        }
        tk[k] = make_float2(tre, tim);
      }
      __syncwarp();
#pragma unroll
      for (int s2 = 0; s2 < kSlots; ++s2) {
        const int i = lane + 32 * s2;
        if (i < L) {
          float are = 0.f, aim = 0.f;
          for (int d = 0; d < n_d; ++d) {
            const float2* xr = yf + d * nmax + i;
            const float2* tr_ = tk + d * n_sub;
            for (int s = 0; s < n_sub; ++s) {
              const float2 x = xr[s], t = tr_[s];
              are = fmaf(x.x, t.x, fmaf(-x.y, t.y, are));
              aim = fmaf(x.x, t.y, fmaf(x.y, t.x, aim));
            }
          }
          const float2 wi = wv[i];
          const float f = sc2 * inv_k;
          wv[L + i] = make_float2(1.0f - fmaf(are, f, eps * wi.x), -fmaf(aim, f, eps * wi.y));
        }
      }
      __syncwarp();
    };

    float2 w[kSlots];
    w[0] = lane < L ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
    if (kSlots > 1) w[kSlots - 1] = lane + 32 < L ? make_float2(1.f, 0.f) : make_float2(0.f, 0.f);
    solve(w);
    if constexpr (!kRecur) {
#pragma unroll
    for (int s2 = 0; s2 < kSlots; ++s2)
      if (lane + 32 * s2 < L) wv[lane + 32 * s2] = w[s2];
    __syncwarp();
    residual();
    {
      float2 r[kSlots];
#pragma unroll
      for (int s2 = 0; s2 < kSlots; ++s2) {
        const int i = lane + 32 * s2;
        r[s2] = i < L ? wv[L + i] : make_float2(0.f, 0.f);
      }
      solve(r);
#pragma unroll
      for (int s2 = 0; s2 < kSlots; ++s2) {
        w[s2].x += r[s2].x;
        w[s2].y += r[s2].y;
      }
      __syncwarp();
#pragma unroll
      for (int s2 = 0; s2 < kSlots; ++s2)
        if (lane + 32 * s2 < L) wv[lane + 32 * s2] = w[s2];
      __syncwarp();
    }
    residual();
    float rn = 0.f;
#pragma unroll
    for (int s2 = 0; s2 < kSlots; ++s2) {
      const int i = lane + 32 * s2;
      if (i < L) {
        const float2 r = wv[L + i];
        rn = fmaf(r.x, r.x, fmaf(r.y, r.y, rn));
      }
    }
    for (int o = 16; o > 0; o >>= 1) rn += __shfl_xor_sync(0xffffffffu, rn, o);
    if (!(sqrtf(rn / static_cast<float>(L)) <= kRefineGate)) {
      if (lane == 0) {
        const int slot = atomicAdd(a.fallback_count, 1);
        if (slot < a.fallback_cap) a.fallback[slot] = make_int2(pix, static_cast<int>(frame));
        if (a.stats) atomicAdd(a.stats, 1);
      }
      continue;
    }
    }  // refinement
    // out = n_act * sum conj(w_i) avg_i / sum w, avg from the centre row.
    float dre = 0.f, dim = 0.f, ore = 0.f, oim = 0.f;
#pragma unroll
    for (int s2 = 0; s2 < kSlots; ++s2) {
      const int i = lane + 32 * s2;
      if (i < L) {
        dre += w[s2].x;
        dim += w[s2].y;
        const float are = avg_re[s2], aim = avg_im[s2];
        ore += w[s2].x * are + w[s2].y * aim;
        oim += w[s2].x * aim - w[s2].y * are;
      }
    }
    for (int o = 16; o > 0; o >>= 1) {
      dre += __shfl_xor_sync(0xffffffffu, dre, o);
      dim += __shfl_xor_sync(0xffffffffu, dim, o);
      ore += __shfl_xor_sync(0xffffffffu, ore, o);
      oim += __shfl_xor_sync(0xffffffffu, oim, o);
    }
    if (hypotf(dre, dim) < 1e-30f)
      export_invalid(a, row, lane);
    else
      {
        const float2 w2[2] = {w[0], kSlots > 1 ? w[kSlots - 1] : make_float2(0.f, 0.f)};
        export_weights(a, row, lane, L, w2, dre, dim);
      }
    if (lane == 0) {
      cplx out;
      if (hypotf(dre, dim) < 1e-30f) {
        out = mk(0.f, 0.f);
        for (int q = 0; q < n_act; ++q) out = cadd(out, mk(yc[act[q]].x, yc[act[q]].y));
      } else {
        out = cscale(cdiv_wide(mk(ore, oim), mk(dre, dim)), static_cast<float>(n_act));
      }
      finish(out, cre, cim, inc);
    }
  }
}

// ---------------------------------------------------------------------------
// The covariance stage on the fifth-generation tensor cores
// (mv_cov_tc5_kernel<P>): every pixel of a class gets its spatially smoothed
// covariance as one batched Hermitian rank-K update, G = A A^T, where A is the
// real 2L x K form of the pixel's snapshot matrix (rows 2i and 2i + 1: real
// and imaginary part of subarray element i; column k = d * S8 + s: snapshot s
// of range row d, S8 = n_sub rounded up to 8, zero past n_sub), in BF16
// scaled by the power of two of mv_warp_kernel, accumulated in FP32 in tensor
// memory. P pixels share one M = N = 128 tile (pixel q's rows at
// q * 128 / P; the blocks that mix two pixels are never read). One thread
// issues the tile's K / 16 tcgen05.mma (M = N = 128, K = 16) with the same
// shared-memory operand as A and B and commits them to an mbarrier (bounded
// wait); the four warps then read their TMEM lanes back and write
//   R~[a][b] = (G[2a][2b] + G[2a+1][2b+1] + i (G[2a+1][2b] - G[2a][2b+1])) / K
// in the packed lower triangle mv_warp_kernel uses (tri(b, a) = conj R~[a][b]).
// The solve kernel reads it back (r_pre) for the trace, Cholesky, solves and
// refinement. A is built from the pixel's staged FP32 rows: for a column
// chunk (8 snapshots) and 8 consecutive elements, one thread slides a 15-sample
// window (the Hankel structure: element i + 1 at snapshot s is element i at
// s + 1) and writes 16-byte chunks in the 128-byte-swizzled K-major layout.

constexpr int kCovThreads = 256;   // eight warps: two per TMEM lane quarter in the epilogue

struct MvCovArgs {
  MvTcArgs base;
  const int* pix_list;
  int n_list, n_frames;
  long item_begin, item_end;
  int lmax, nmax, kcap;     // class limits; K capacity (multiple of 64)
  float2* r_out;            // [item - item_begin][r_stride]
  uint8_t* r_flag;          // [item - item_begin]: 1 where r_out holds the pixel's R~
  int r_stride;
  int* status;              // set on an mbarrier timeout
};

struct CovItem {
  int state;                // 0 none, 1 covariance here, 2 staged but amax unknown yet
  int L, n_act, n_sub, n_d, dlo, pix, s8, kq;
  long frame;
  unsigned amax_bits;
  float sc, inv_k;
};

__host__ __device__ inline int cov_ystride(int nmax) { return nmax + 16; }

// One buffer of per-tile pixel data (two are kept: the next tile's fills
// while this tile's MMAs run).
// Byte offsets within one buffer: staged rows, active channels, items (16-byte aligned).
__host__ __device__ inline size_t cov_act_off(int P, int n_dmax, int nmax) {
  return sizeof(float2) * static_cast<size_t>(P) * n_dmax * cov_ystride(nmax);
}
__host__ __device__ inline size_t cov_item_off(int P, int n_dmax, int nmax) {
  return align16(cov_act_off(P, n_dmax, nmax) + sizeof(int) * P * nmax);
}
__host__ __device__ inline size_t cov_buf_bytes(int P, int n_dmax, int nmax) {
  return align16(cov_item_off(P, n_dmax, nmax) + sizeof(CovItem) * P);
}

__host__ __device__ inline size_t cov_smem_bytes(int P, int n_dmax, int nmax, int kcap) {
  return 1024 + static_cast<size_t>(kcap) * 256 + 2 * cov_buf_bytes(P, n_dmax, nmax) + 64;
}

template <int P>
struct CovBuf {
  float2* yst;   // [P][n_dmax][ystride]
  int* act;      // [P][nmax]
  CovItem* it;   // [P]
};

template <int P>
__device__ __forceinline__ CovBuf<P> cov_buf(char* base, const MvCovArgs& c) {
  CovBuf<P> b;
  b.yst = reinterpret_cast<float2*>(base);
  b.act = reinterpret_cast<int*>(base + cov_act_off(P, c.base.n_dmax, c.nmax));
  b.it = reinterpret_cast<CovItem*>(base + cov_item_off(P, c.base.n_dmax, c.nmax));
  return b;
}

// Pixel data of tile `tile` into buffer b: the aperture and subarray (warp q
// for pixel q), then the range rows staged by all threads, then the scale.
// Ends with a CTA barrier.
template <int P>
__device__ void cov_fill(const MvCovArgs& c, const CovBuf<P>& b, long tile, long n_items) {
  const MvTcArgs& a = c.base;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ystride = cov_ystride(c.nmax);
  if (warp < P) {
    const int q = warp;
    const long rel = tile * P + q;
    CovItem it{};
    if (rel < n_items) {
      const long item = c.item_begin + rel;
      const long frame = item / c.n_list;
      const int pix = c.pix_list[item - frame * c.n_list];
      const int j = pix % a.n1;
      const float px = __ldg(a.points + 3 * pix), pz = __ldg(a.points + 3 * pix + 2);
      int* act = b.act + q * c.nmax;
      int n_act = 0;
      for (int c0 = 0; c0 < a.n_ch; c0 += 32) {
        const int ch = c0 + lane;
        bool on = false;
        if (ch < a.n_ch)
          on = aperture_weight((static_cast<float>(ch) - a.half_nm1) * a.pitch, px, pz, a.f_number, a.rx_window,
                               a.tukey_alpha) > 0.0f;
        const unsigned m = __ballot_sync(0xffffffffu, on);
        const int slot = n_act + __popc(m & ((1u << lane) - 1u));
        if (on && slot < c.nmax) act[slot] = ch;
        n_act += __popc(m);
      }
      int L = a.mv_subarray;
      const int hi = max(2, n_act / 2);
      if (L < 2) L = 2;
      if (L > hi) L = hi;
      // The solve kernel's rules (overflow, fewer than 4 channels) and the
      // operand tile's capacity: otherwise no covariance here.
      if (!(n_act > c.nmax || L > c.lmax || n_act < 4)) {
        int dlo = -a.range_avg, dhi = a.range_avg;
        while (j + dlo < 0) ++dlo;
        while (j + dhi >= a.n1) --dhi;
        const int n_sub = n_act - L + 1;
        const int s8 = (n_sub + 7) & ~7;
        const int n_d = dhi - dlo + 1;
        if (n_d * s8 <= c.kcap) {
          it.state = 2;
          it.L = L;
          it.n_act = n_act;
          it.n_sub = n_sub;
          it.n_d = n_d;
          it.dlo = dlo;
          it.pix = pix;
          it.frame = frame;
          it.s8 = s8;
          it.kq = n_d * s8;
        }
      }
    }
    if (lane == 0) b.it[q] = it;
  }
  __syncthreads();
  // Range rows of every staged pixel (zeros past n_act), all threads.
  for (int q = 0; q < P; ++q) {
    const CovItem& it = b.it[q];
    if (it.state != 2) continue;   // uniform across the CTA
    const float2* Y = a.y + it.frame * static_cast<long>(a.n_pix) * a.n_ch;
    const int* act = b.act + q * c.nmax;
    float m = 0.0f;
    for (int k = threadIdx.x; k < it.n_d * ystride; k += kCovThreads) {
      const int d = k / ystride, t = k - d * ystride;
      float2 v = make_float2(0.f, 0.f);
      if (t < it.n_act) {
        v = Y[static_cast<long>(it.pix + it.dlo + d) * a.n_ch + act[t]];
        m = fmaxf(m, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
      b.yst[(q * a.n_dmax + d) * ystride + t] = v;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if (lane == 0 && m > 0.0f) atomicMax(&b.it[q].amax_bits, __float_as_uint(m));
  }
  __syncthreads();
  if (threadIdx.x < P) {
    CovItem& it = b.it[threadIdx.x];
    if (it.state == 2) {
      const float amax = __uint_as_float(it.amax_bits);
      if (amax > 0.0f) {
        int e2;
        frexpf(amax, &e2);
        it.sc = ldexpf(1.0f, -e2);
        it.inv_k = 1.0f / static_cast<float>(it.n_d * it.n_sub);
        it.state = 1;
      } else {
        it.state = 0;
      }
    }
  }
  __syncthreads();
}

template <int P>
__global__ void __launch_bounds__(kCovThreads, 1) mv_cov_tc5_kernel(const MvCovArgs c) {
  constexpr int R = 128 / P;   // rows of one pixel's slot
  extern __shared__ __align__(1024) char cov_raw[];
  char* sA = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(cov_raw) + 1023) & ~uintptr_t(1023));
  const MvTcArgs& a = c.base;
  const int ystride = cov_ystride(c.nmax);
  const size_t buf_bytes = cov_buf_bytes(P, a.n_dmax, c.nmax);
  char* buf0 = sA + static_cast<size_t>(c.kcap) * 256;
  const CovBuf<P> bufs[2] = {cov_buf<P>(buf0, c), cov_buf<P>(buf0 + buf_bytes, c)};
  uint64_t* bar = reinterpret_cast<uint64_t*>(buf0 + 2 * buf_bytes);
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(bar + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(su32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = *tmem_slot;
  const uint32_t idesc = instr_desc(128, 128);
  unsigned phase = 0;
  const long n_items = c.item_end - c.item_begin;
  const long n_tiles = (n_items + P - 1) / P;

  long tile = blockIdx.x;
  int cur = 0;
  if (tile < n_tiles) cov_fill<P>(c, bufs[0], tile, n_items);
  for (; tile < n_tiles; tile += gridDim.x, cur ^= 1) {
    const CovBuf<P>& b = bufs[cur];
    int ktile = 0;
    bool any = false;
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const CovItem& it = b.it[q];
      if (it.state == 1) {
        any = true;
        ktile = max(ktile, it.kq);
      }
      // Which items this tile covers (the solve kernel forms the rest itself).
      const long rel = tile * P + q;
      if (threadIdx.x == q && rel < n_items) c.r_flag[rel] = it.state == 1 ? 1 : 0;
    }
    ktile = (ktile + 15) & ~15;
    const long next = tile + gridDim.x;
    if (!any) {
      if (next < n_tiles) cov_fill<P>(c, bufs[cur ^ 1], next, n_items);
      continue;
    }
    // ---- build A: window units (q, d, column chunk, element block of 8) --
    int off[P + 1];
    off[0] = 0;
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const CovItem& it = b.it[q];
      off[q + 1] = off[q] + (it.state == 1 ? it.n_d * (it.s8 >> 3) * ((it.L + 7) >> 3) : 0);
    }
    for (int f = threadIdx.x; f < off[P]; f += kCovThreads) {
      int q = 0;
#pragma unroll
      for (int z = 1; z < P; ++z)
        if (f >= off[z]) q = z;
      const CovItem& it = b.it[q];
      int u = f - off[q];
      const int nib = (it.L + 7) >> 3, nc = it.s8 >> 3;
      const int ib = u % nib;
      u /= nib;
      const int cc = u % nc, d = u / nc;
      const float2* y = b.yst + (q * a.n_dmax + d) * ystride + 8 * cc + 8 * ib;
      float2 win[15];
#pragma unroll
      for (int t = 0; t < 15; ++t) win[t] = y[t];
      const int s0 = 8 * cc, k0 = d * it.s8 + s0;
      bool in[8];
#pragma unroll
      for (int t = 0; t < 8; ++t) in[t] = s0 + t < it.n_sub;
#pragma unroll
      for (int ii = 0; ii < 8; ++ii) {
        const int i = 8 * ib + ii;
        if (i < it.L) {
          uint32_t re[4], im[4];
#pragma unroll
          for (int t = 0; t < 8; t += 2) {
            const float2 v0 = in[t] ? win[ii + t] : make_float2(0.f, 0.f);
            const float2 v1 = in[t + 1] ? win[ii + t + 1] : make_float2(0.f, 0.f);
            re[t >> 1] = pack_bf16(v0.x * it.sc, v1.x * it.sc);
            im[t >> 1] = pack_bf16(v0.y * it.sc, v1.y * it.sc);
          }
          const int row = q * R + 2 * i;
          *reinterpret_cast<uint4*>(sA + sw128_offset(128, row, k0)) = make_uint4(re[0], re[1], re[2], re[3]);
          *reinterpret_cast<uint4*>(sA + sw128_offset(128, row + 1, k0)) = make_uint4(im[0], im[1], im[2], im[3]);
        }
      }
    }
    // Zero columns [kq, ktile) of each pixel's rows.
    int zoff[P + 1];
    zoff[0] = 0;
#pragma unroll
    for (int q = 0; q < P; ++q) {
      const CovItem& it = b.it[q];
      zoff[q + 1] = zoff[q] + (it.state == 1 ? 2 * it.L * ((ktile - it.kq) >> 3) : 0);
    }
    for (int f = threadIdx.x; f < zoff[P]; f += kCovThreads) {
      int q = 0;
#pragma unroll
      for (int z = 1; z < P; ++z)
        if (f >= zoff[z]) q = z;
      const CovItem& it = b.it[q];
      const int u = f - zoff[q], nz = (ktile - it.kq) >> 3;
      const int row = q * R + u / nz, k0 = it.kq + 8 * (u % nz);
      *reinterpret_cast<uint4*>(sA + sw128_offset(128, row, k0)) = make_uint4(0u, 0u, 0u, 0u);
    }
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned a0 = su32(sA);
      for (int ks = 0; ks < ktile / 16; ++ks) {
        const uint64_t dsc = smem_desc(a0 + (ks >> 2) * 128 * 128 + (ks & 3) * 32);
        tc5_mma(tmem, dsc, dsc, idesc, ks > 0 ? 1u : 0u);
      }
      tc5_commit(su32(bar));
    }
    // The next tile's pixel data while the tensor core works.
    if (next < n_tiles) cov_fill<P>(c, bufs[cur ^ 1], next, n_items);
    const bool ok = mbar_wait(su32(bar), phase);
    if (__syncthreads_or(!ok)) {
      // Timed out: record it, give the tile's MMAs one more bounded wait so
      // that none is in flight when the TMEM is released, and stop.
      if (threadIdx.x == 0) {
        if (c.status) atomicExch(c.status, 1);
        mbar_wait(su32(bar), phase);
      }
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // ---- epilogue: warps w and w + 4 hold rows 32 (w % 4) .. + 31 (their
    // TMEM lane quarter) and take alternate 32-column chunks --------------
    {
      const int quarter = warp & 3, half = warp >> 2;
      const int q = (quarter * 32) / R;
      const CovItem& it = b.it[q];
      const int ml0 = quarter * 32 - q * R;  // first local row of this warp
      if (it.state == 1 && ml0 < 2 * it.L) {
        const long rel = tile * P + q;
        float2* dst = c.r_out + rel * c.r_stride;
        const int ml = ml0 + lane, a_el = ml >> 1;
        const bool even = (ml & 1) == 0;
        const unsigned taddr = tmem + (static_cast<unsigned>(quarter * 32) << 16) + static_cast<unsigned>(q * R);
        for (int j0 = 32 * half; j0 < 2 * it.L; j0 += 64) {
          uint32_t r[32];
          tc5_ld32(taddr + static_cast<unsigned>(j0), r);
#pragma unroll
          for (int t = 0; t < 32; t += 2) {
            // Odd row's G[2a+1][2b], G[2a+1][2b+1] from the neighbouring lane.
            const float g0 = __uint_as_float(r[t]), g1 = __uint_as_float(r[t + 1]);
            const float o0 = __shfl_xor_sync(0xffffffffu, g0, 1);
            const float o1 = __shfl_xor_sync(0xffffffffu, g1, 1);
            const int bb = (j0 + t) >> 1;
            if (even && a_el < it.L && bb < it.L && bb >= a_el)
              dst[tri(bb, a_el)] = make_float2((g0 + o1) * it.inv_k, -(o0 - g1) * it.inv_k);
          }
        }
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(128));
}

// FP64 re-solve of the pixels whose refined FP32 residual failed: covariance
// from the snapshots, Cholesky and solves in double, one warp per pixel.

__global__ void __launch_bounds__(32) mv_fp64_kernel(const MvTcArgs a) {
  extern __shared__ double2 f64_smem[];
  const int lane = threadIdx.x;
  const int count = min(*a.fallback_count, a.fallback_cap);
  double2* Rd = f64_smem;                                    // packed lower L(L+1)/2
  int* act = reinterpret_cast<int*>(Rd + a.lmax * (a.lmax + 1) / 2);
  for (int item = blockIdx.x; item < count; item += gridDim.x) {
    const int2 pf = a.fallback[item];
    const int pix = pf.x;
    const long frame = pf.y;
    const int j = pix % a.n1;
    const float px = __ldg(a.points + 3 * pix), pz = __ldg(a.points + 3 * pix + 2);
    const float2* Y = a.y + frame * static_cast<long>(a.n_pix) * a.n_ch;
    const float2* yc = Y + static_cast<long>(pix) * a.n_ch;
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
    const int n_d = dhi - dlo + 1;
    const double inv_k = 1.0 / static_cast<double>(n_d * n_sub);
    for (int e = lane; e < L * (L + 1) / 2; e += 32) {
      int i = 0, rem = e;
      while (rem > i) {
        rem -= i + 1;
        ++i;
      }
      const int jj = rem;
      double re = 0.0, im = 0.0;
      for (int d = dlo; d <= dhi; ++d) {
        const float2* yr = Y + static_cast<long>(pix + d) * a.n_ch;
        for (int s = 0; s < n_sub; ++s) {
          const float2 xi = yr[act[s + i]], xj = yr[act[s + jj]];
          re += static_cast<double>(xi.x) * xj.x + static_cast<double>(xi.y) * xj.y;
          im += static_cast<double>(xi.y) * xj.x - static_cast<double>(xi.x) * xj.y;
        }
      }
      Rd[e] = make_double2(re * inv_k, im * inv_k);
    }
    __syncwarp();
    double tr = 0.0;
    for (int i = lane; i < L; i += 32) tr += Rd[tri(i, i)].x;
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    const double eps = fmax(static_cast<double>(a.loading) * tr / L, 1e-20);
    for (int i = lane; i < L; i += 32) Rd[tri(i, i)].x += eps;
    __syncwarp();
    bool ok = true;
    for (int c = 0; c < L; ++c) {
      const double dgl = Rd[tri(c, c)].x;
      if (!(dgl > 0.0)) {
        ok = false;
        break;
      }
      const double ljj = sqrt(dgl);
      __syncwarp();
      for (int i = c + 1 + lane; i < L; i += 32) {
        const double2 v = Rd[tri(i, c)];
        Rd[tri(i, c)] = make_double2(v.x / ljj, v.y / ljj);
      }
      if (lane == 0) Rd[tri(c, c)] = make_double2(ljj, 0.0);
      __syncwarp();
      for (int i = c + 1 + lane; i < L; i += 32) {
        const double2 lic = Rd[tri(i, c)];
        for (int k = c + 1; k <= i; ++k) {
          const double2 lkc = Rd[tri(k, c)];
          double2 v = Rd[tri(i, k)];
          v.x -= lic.x * lkc.x + lic.y * lkc.y;
          v.y -= lic.y * lkc.x - lic.x * lkc.y;
          Rd[tri(i, k)] = v;
        }
      }
      __syncwarp();
    }
    cplx out;
    if (!ok) {
      if (a.w_export) {
        const long row = frame * a.n_pix + pix;
        float2* dst = reinterpret_cast<float2*>(a.w_export) + row * kTcMaxL;
        for (int i = lane; i < kTcMaxL; i += 32) dst[i] = make_float2(0.f, 0.f);
        if (lane == 0) a.w_valid[row] = 0;
      }
      if (a.stats && lane == 0) atomicAdd(a.stats + 1, 1);
      out = mk(0.f, 0.f);
      for (int q = 0; q < n_act; ++q) out = cadd(out, mk(yc[act[q]].x, yc[act[q]].y));
    } else {
      double2 v[2];
      for (int s2 = 0; s2 < 2; ++s2) v[s2] = (lane + 32 * s2 < L) ? make_double2(1.0, 0.0) : make_double2(0.0, 0.0);
      for (int c = 0; c < L; ++c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const double l = Rd[tri(c, c)].x;
          v[sl] = make_double2(v[sl].x / l, v[sl].y / l);
        }
        const double vx = __shfl_sync(0xffffffffu, sl ? v[1].x : v[0].x, own);
        const double vy = __shfl_sync(0xffffffffu, sl ? v[1].y : v[0].y, own);
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i > c && i < L) {
            const double2 l = Rd[tri(i, c)];
            v[s2].x -= l.x * vx - l.y * vy;
            v[s2].y -= l.x * vy + l.y * vx;
          }
        }
      }
      for (int c = L - 1; c >= 0; --c) {
        const int own = c & 31, sl = c >> 5;
        if (lane == own) {
          const double l = Rd[tri(c, c)].x;
          v[sl] = make_double2(v[sl].x / l, v[sl].y / l);
        }
        const double vx = __shfl_sync(0xffffffffu, sl ? v[1].x : v[0].x, own);
        const double vy = __shfl_sync(0xffffffffu, sl ? v[1].y : v[0].y, own);
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          if (i < c) {
            const double2 l = Rd[tri(c, i)];
            v[s2].x -= l.x * vx + l.y * vy;
            v[s2].y -= l.x * vy - l.y * vx;
          }
        }
      }
      double dre = 0, dim = 0, ore = 0, oim = 0;
      const float2* ycen = yc;
      for (int s2 = 0; s2 < 2; ++s2) {
        const int i = lane + 32 * s2;
        if (i >= L) continue;
        dre += v[s2].x;
        dim += v[s2].y;
        double are = 0, aim = 0;
        for (int s = 0; s < n_sub; ++s) {
          are += ycen[act[s + i]].x;
          aim += ycen[act[s + i]].y;
        }
        are /= n_sub;
        aim /= n_sub;
        ore += v[s2].x * are + v[s2].y * aim;
        oim += v[s2].x * aim - v[s2].y * are;
      }
      for (int o = 16; o > 0; o >>= 1) {
        dre += __shfl_xor_sync(0xffffffffu, dre, o);
        dim += __shfl_xor_sync(0xffffffffu, dim, o);
        ore += __shfl_xor_sync(0xffffffffu, ore, o);
        oim += __shfl_xor_sync(0xffffffffu, oim, o);
      }
      const double den = dre * dre + dim * dim;
      if (a.w_export) {
        const long row = frame * a.n_pix + pix;
        float2* dst = reinterpret_cast<float2*>(a.w_export) + row * kTcMaxL;
        const bool solved = !(sqrt(den) < 1e-30);
        for (int s2 = 0; s2 < 2; ++s2) {
          const int i = lane + 32 * s2;
          float2 val = make_float2(0.f, 0.f);
          if (i < L && solved) {
            val.x = static_cast<float>((v[s2].x * dre + v[s2].y * dim) / den * L);
            val.y = static_cast<float>((v[s2].y * dre - v[s2].x * dim) / den * L);
          }
          dst[i] = val;
        }
        if (lane == 0) a.w_valid[row] = solved ? 1 : 0;
      }
      if (sqrt(den) < 1e-30) {
        out = mk(0.f, 0.f);
        for (int q = 0; q < n_act; ++q) out = cadd(out, mk(yc[act[q]].x, yc[act[q]].y));
      } else {
        out = mk(static_cast<float>((ore * dre + oim * dim) / den * n_act),
                 static_cast<float>((oim * dre - ore * dim) / den * n_act));
      }
    }
    if (lane == 0) {
      if (a.cf) {
        cplx coh = mk(0.f, 0.f);
        float inc = 0.0f;
        for (int q = 0; q < n_act; ++q) {
          const float2 y = yc[act[q]];
          coh = cadd(coh, mk(y.x, y.y));
          inc += cnorm(mk(y.x, y.y));
        }
        out = cscale(out, (inc > 0.0f) ? cnorm(coh) / (static_cast<float>(n_act) * inc) : 0.0f);
      }
      if (a.incoherent)
        a.acc_out[frame * a.n_pix + pix] += cnorm(out);
      else
        a.out[frame * a.out_stride + pix] = make_float2(out.re, out.im);
    }
  }
}

}  // namespace

int mv_tc_supported(int n_ch, int mv_subarray, int range_avg) {
  const int lmax = std::min(std::max(mv_subarray, 2), std::max(2, n_ch / 2));
  if (n_ch > kTcMaxCh || lmax > kTcMaxL || range_avg > 4) return 0;
  const MvTcLayout l = mv_tc_layout(n_ch, 2 * range_avg + 1, lmax);
  return l.bytes <= 200 * 1024 ? 1 : 0;
}

int launch_mv_tc(usx_ctx* ctx, const float2* y, const float* points, float2* out, long out_stride,
                 float* acc_out, int n_ch, int n_pix, int n1, int n_frames, int mv_subarray, int range_avg,
                 float loading, float f_number, float tukey_alpha, int rx_window, float half_nm1, float pitch,
                 int cf, int incoherent, int* stats, int* fallback_count, int2* fallback, int fallback_cap,
                 const MvTcExtra& extra) {
  MvTcArgs a;
  a.y = y;
  a.points = points;
  a.out = out;
  a.out_stride = out_stride;
  a.acc_out = acc_out;
  a.n_ch = n_ch;
  a.n_pix = n_pix;
  a.n1 = n1;
  a.mv_subarray = mv_subarray;
  a.range_avg = range_avg;
  a.loading = loading;
  a.f_number = f_number;
  a.tukey_alpha = tukey_alpha;
  a.half_nm1 = half_nm1;
  a.pitch = pitch;
  a.rx_window = rx_window;
  a.cf = cf;
  a.incoherent = incoherent;
  a.n_dmax = 2 * range_avg + 1;
  a.lmax = std::min(std::max(mv_subarray, 2), std::max(2, n_ch / 2));
  a.stats = stats;
  a.fallback_count = fallback_count;
  a.fallback = fallback;
  a.fallback_cap = fallback_cap;
  a.list = extra.list;
  a.list_count = extra.list_count;
  a.list_cap = extra.list_cap;
  a.w_export = extra.w_export;
  a.w_valid = extra.w_valid;
  auto launch_cta = [&](const MvTcArgs& b, bool list_mode) -> int {
    const MvTcLayout l = mv_tc_layout(n_ch, b.n_dmax, b.lmax);
    const size_t smem = l.bytes;
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(mv_tc_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
    int per_sm = 0;
    if (int rc_ = occupancy(reinterpret_cast<const void*>(mv_tc_kernel), 32 * kTcWarps, static_cast<size_t>(smem), &per_sm)) return rc_;
    // Full frames: a grid-stride loop over pixels, frames on y. Work list: its
    // length is only known on the device, so one resident wave loops over it.
    const long resident = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count;
    const long want = resident * 4 / std::max(1, n_frames);
    const dim3 grid = list_mode ? dim3(static_cast<unsigned>(resident), 1)
                                : dim3(static_cast<unsigned>(std::max(1L, std::min<long>(n_pix, want))), n_frames);
    prof_begin(ctx, "mv_tc_kernel");
    mv_tc_kernel<<<grid, 32 * kTcWarps, smem, ctx->stream>>>(b);
    prof_end(ctx);
    USX_CHECK_LAUNCH("mv_tc_kernel");
    return USX_OK;
  };
  auto launch_warp = [&](MvWarpArgs& w, long items, const char* name) -> int {
    w.cov_recur = extra.cov_engine == 2 ? 1 : 0;
    const MvWarpLayout l = mv_warp_layout(w.nmax, a.n_dmax, w.lmax, w.cov_recur != 0);
    const size_t smem = l.bytes * kWarpMvWarps;
    if (smem > 227 * 1024) return fail(USX_ERR_UNSUPPORTED, "minimum variance: class too large for shared memory");
    // The FP32 instance compiles only the lag recurrence and one solve (64
    // registers against 124 with the BF16 paths: twice the resident warps).
    const bool recur = w.cov_recur != 0;
    const void* kern = recur ? reinterpret_cast<const void*>(mv_warp_kernel<2, true>)
                             : reinterpret_cast<const void*>(mv_warp_kernel<2, false>);
    if (int rc_ = smem_limit(kern, static_cast<size_t>(static_cast<int>(smem)))) return rc_;
    int per_sm = 0;
    if (int rc_ = occupancy(kern, 32 * kWarpMvWarps, static_cast<size_t>(smem), &per_sm)) return rc_;
    const long resident = static_cast<long>(std::max(1, per_sm)) * ctx->sm_count;
    const long need = (items + kWarpMvWarps - 1) / kWarpMvWarps;
    const long blocks = items < 0 ? resident : std::max(1L, std::min(need, resident * 8));
    prof_begin(ctx, name);
    const dim3 gr(static_cast<unsigned>(blocks));
    if (recur)
      mv_warp_kernel<2, true><<<gr, 32 * kWarpMvWarps, smem, ctx->stream>>>(w);
    else
      mv_warp_kernel<2, false><<<gr, 32 * kWarpMvWarps, smem, ctx->stream>>>(w);
    prof_end(ctx);
    USX_CHECK_LAUNCH(name);
    return USX_OK;
  };
  if (extra.list) {
    // Work list of (pixel, frame): one warp per pixel, sized for the plan's
    // largest subarray and the whole array.
    MvWarpArgs w{};
    w.base = a;
    w.lmax = extra.list_lmax > 0 ? std::min(extra.list_lmax, a.lmax) : a.lmax;
    w.nmax = extra.list_nmax > 0 ? std::min(extra.list_nmax, n_ch) : n_ch;
    w.pair_list = extra.list;
    w.pair_count = extra.list_count;
    w.pair_cap = extra.list_cap;
    const bool limited = w.lmax < a.lmax || w.nmax < n_ch;
    if (limited && !extra.overflow_count)
      return fail(USX_ERR_INVALID, "minimum variance: a limited work list needs an overflow list");
    w.overflow_count = limited ? extra.overflow_count : nullptr;
    w.overflow = extra.overflow;
    w.overflow_cap = limited ? extra.overflow_cap : 0;
    if (limited) USX_CUDA(cudaMemsetAsync(extra.overflow_count, 0, sizeof(int), ctx->stream));
    if (int rc = launch_warp(w, -1, "mv_warp_kernel(list)")) return rc;
    if (limited) {
      MvTcArgs b = a;
      b.list = extra.overflow;
      b.list_count = extra.overflow_count;
      b.list_cap = extra.overflow_cap;
      if (int rc = launch_cta(b, true)) return rc;
    }
  } else if (extra.n_classes > 0 && extra.overflow_count) {
    // Pixel classes of similar subarray length, one launch each; pixels past
    // a class's limits go to the CTA kernel through the overflow list.
    USX_CUDA(cudaMemsetAsync(extra.overflow_count, 0, sizeof(int), ctx->stream));
    for (int c = 0; c < extra.n_classes; ++c) {
      const MvClass& k = extra.classes[c];
      if (k.count <= 0) continue;
      MvWarpArgs w{};
      w.base = a;
      w.lmax = k.lmax;
      w.nmax = k.nmax;
      w.pix_list = k.pixels;
      w.n_list = k.count;
      w.n_frames = n_frames;
      w.overflow_count = extra.overflow_count;
      w.overflow = extra.overflow;
      w.overflow_cap = extra.overflow_cap;
      const long items = static_cast<long>(k.count) * n_frames;
      // K capacity: a class's pixels have L >= its lower bound (less one at
      // an aperture edge), so n_sub <= nmax - lmax + 18; pixels beyond it are
      // flagged and the solve kernel forms their covariance itself.
      const int nsub_cap = std::max(1, std::min(k.nmax, k.nmax - k.lmax + 18));
      const int kcap = (a.n_dmax * ((nsub_cap + 7) & ~7) + 63) & ~63;
      const int P_cov = 2 * k.lmax <= 32 ? 4 : (2 * k.lmax <= 64 ? 2 : 1);
      // Classes whose operand tile does not fit shared memory keep the mma.sync covariance.
      if (extra.cov_engine == 1 && 2 * k.lmax <= 128 && cov_smem_bytes(P_cov, a.n_dmax, k.nmax, kcap) <= 227 * 1024) {
        // Covariances on tcgen05 in chunks whose R~ (about 96 MB) stays in L2
        // until the solve kernel reads it.
        const int P = P_cov;
        const int r_stride = k.lmax * (k.lmax + 1) / 2;
        const long chunk = std::max(1024L, static_cast<long>((96u << 20) / (sizeof(float2) * r_stride)));
        const size_t n_chunk = static_cast<size_t>(std::min(chunk, items));
        const size_t flag_off = (sizeof(float2) * static_cast<size_t>(r_stride) * n_chunk + 255) / 256 * 256;
        const size_t need = flag_off + n_chunk;
        if (need > ctx->mv_cov_bytes) {
          if (ctx->mv_cov) {
            USX_CUDA(cudaStreamSynchronize(ctx->stream));
            USX_CUDA(cudaFree(ctx->mv_cov));
            ctx->mv_cov = nullptr;
            ctx->mv_cov_bytes = 0;
          }
          USX_CUDA(cudaMalloc(&ctx->mv_cov, need));
          ctx->mv_cov_bytes = need;
        }
        MvCovArgs cv{};
        cv.base = a;
        cv.pix_list = k.pixels;
        cv.n_list = k.count;
        cv.n_frames = n_frames;
        cv.lmax = k.lmax;
        cv.nmax = k.nmax;
        cv.kcap = kcap;
        cv.r_out = static_cast<float2*>(ctx->mv_cov);
        cv.r_flag = static_cast<uint8_t*>(ctx->mv_cov) + flag_off;
        cv.r_stride = r_stride;
        cv.status = ctx->d_status + 14;
        const size_t smem = cov_smem_bytes(P, a.n_dmax, k.nmax, cv.kcap);
        const void* kern = P == 4 ? reinterpret_cast<const void*>(mv_cov_tc5_kernel<4>)
                         : P == 2 ? reinterpret_cast<const void*>(mv_cov_tc5_kernel<2>)
                                  : reinterpret_cast<const void*>(mv_cov_tc5_kernel<1>);
        if (int rc_ = smem_limit(kern, smem)) return rc_;
        // The kernel reads nothing through L1 that it does not stage: all of
        // the SM's unified memory may go to shared memory, two CTAs of ~100 KB.
        USX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                                      static_cast<int>(cudaSharedmemCarveoutMaxShared)));
        int per_sm = 0;
        if (int rc_ = occupancy(kern, kCovThreads, smem, &per_sm)) return rc_;
        // At most four CTAs per SM: each holds 128 of the SM's 512 TMEM columns.
        const long resident = static_cast<long>(std::max(1, std::min(per_sm, 4))) * ctx->sm_count;
        w.r_pre = static_cast<const float2*>(ctx->mv_cov);
        w.r_flag = cv.r_flag;
        w.r_stride = r_stride;
        for (long i0 = 0; i0 < items; i0 += chunk) {
          const long i1 = std::min(items, i0 + chunk);
          cv.item_begin = i0;
          cv.item_end = i1;
          const long tiles = (i1 - i0 + P - 1) / P;
          const unsigned grid = static_cast<unsigned>(std::max(1L, std::min(tiles, resident)));
          prof_begin(ctx, "mv_cov_tc5_kernel");
          if (P == 4)
            mv_cov_tc5_kernel<4><<<grid, kCovThreads, smem, ctx->stream>>>(cv);
          else if (P == 2)
            mv_cov_tc5_kernel<2><<<grid, kCovThreads, smem, ctx->stream>>>(cv);
          else
            mv_cov_tc5_kernel<1><<<grid, kCovThreads, smem, ctx->stream>>>(cv);
          prof_end(ctx);
          USX_CHECK_LAUNCH("mv_cov_tc5_kernel");
          w.item_begin = i0;
          w.item_end = i1;
          if (int rc = launch_warp(w, i1 - i0, "mv_warp_kernel")) return rc;
        }
        continue;
      }
      if (int rc = launch_warp(w, items, "mv_warp_kernel")) return rc;
    }
    MvTcArgs b = a;
    b.list = extra.overflow;
    b.list_count = extra.overflow_count;
    b.list_cap = extra.overflow_cap;
    if (int rc = launch_cta(b, true)) return rc;
  } else {
    if (int rc = launch_cta(a, false)) return rc;
  }
  // FP64 re-solve of the pixels whose refined residual failed (usually none).
  const size_t smem64 = sizeof(double2) * (a.lmax * (a.lmax + 1) / 2) + sizeof(int) * n_ch;
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(mv_fp64_kernel), static_cast<size_t>(static_cast<int>(smem64)))) return rc_;
  prof_begin(ctx, "mv_fp64_kernel");
  mv_fp64_kernel<<<ctx->sm_count * 4, 32, smem64, ctx->stream>>>(a);
  prof_end(ctx);
  USX_CHECK_LAUNCH("mv_fp64_kernel");
  return USX_OK;
}

}  // namespace usxcu
