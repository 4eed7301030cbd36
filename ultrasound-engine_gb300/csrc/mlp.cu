// mlp.cu — the learned minimum-variance surrogate's network (no reference
// counterpart): a fully connected net with BF16 weights and activations, FP32
// accumulation, trained on the device with hand-written forward and backward
// GEMMs and Adam.
//
// GEMM: C[M x N] (+)= op(A)[M x K] * op(B)[K x N], BF16 operands, FP32
// accumulators, mma.sync m16n8k16 fed by ldmatrix from a two-stage cp.async
// shared-memory pipeline. 128 x 128 x 32 block tiles, 8 warps of 64 x 32.
// Operand layouts cover the three products of training:
//   forward   H = X W        A row-major (k contiguous), B row-major (n contiguous)
//   input     dX = dH W^T    B given as W: element (k, n) at W[n*ldb + k]
//   weight    dW = X^T dH    A given as X: element (m, k) at X[k*lda + m]
// Epilogues: bias add, ReLU, ReLU-derivative mask (by the forward activation),
// BF16 and/or FP32 stores, or FP32 atomic accumulation for split-K weight
// gradients. M, N must be multiples of 128 and K of 32 (callers pad).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int BM = 128, BN = 128, BK = 32;
constexpr int kGemmThreads = 256;
constexpr int kPad = 8;  // bf16 elements of padding per smem row (bank-conflict free ldmatrix)

struct GemmArgs {
  const __nv_bfloat16* A;
  const __nv_bfloat16* B;
  int M, N, K, lda, ldb;
  int a_kmajor;   // A(m, k) at A[m*lda + k] (else A[k*lda + m])
  int b_nmajor;   // B(k, n) at B[k*ldb + n] (else B[n*ldb + k])
  const float* bias;               // [N] or null
  int relu;                        // apply max(0, .)
  const __nv_bfloat16* relu_mask;  // zero where mask <= 0 ([M x ldc_mask]) or null
  int ld_mask;
  __nv_bfloat16* C16;              // BF16 output or null
  float* C32;                      // FP32 output or null
  int ldc;
  int atomic;                      // accumulate into C32 with atomicAdd (split-K)
  int k_per_split;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void ldmatrix_x4(uint32_t (&r)[4], const void* smem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(s));
}
__device__ __forceinline__ void ldmatrix_x4_trans(uint32_t (&r)[4], const void* smem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]) : "r"(s));
}
__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared tile shapes (elements): A k-major [BM][BK+pad] or m-major [BK][BM+pad];
// B n-major [BK][BN+pad] or k-major [BN][BK+pad].
constexpr int kAkm = BM * (BK + kPad), kAmm = BK * (BM + kPad);
constexpr int kBnm = BK * (BN + kPad), kBkm = BN * (BK + kPad);
constexpr int kAtile = kAkm > kAmm ? kAkm : kAmm;
constexpr int kBtile = kBnm > kBkm ? kBnm : kBkm;
constexpr size_t kGemmSmem = sizeof(__nv_bfloat16) * 2 * (kAtile + kBtile);

__global__ void __launch_bounds__(kGemmThreads) gemm_bf16_kernel(const GemmArgs g) {
  extern __shared__ __align__(16) __nv_bfloat16 gsm[];
  __nv_bfloat16* As = gsm;                   // [2][kAtile]
  __nv_bfloat16* Bs = gsm + 2 * kAtile;      // [2][kBtile]
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = warp >> 2, wn = warp & 3;  // 2 x 4 warps, warp tile 64 x 32
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const int k_begin = blockIdx.z * g.k_per_split;
  const int k_end = min(g.K, k_begin + g.k_per_split);

  float acc[4][4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j][0] = acc[i][j][1] = acc[i][j][2] = acc[i][j][3] = 0.f;

  auto load_tile = [&](int stage, int k0) {
    __nv_bfloat16* as = As + stage * kAtile;
    __nv_bfloat16* bs = Bs + stage * kBtile;
    // 512 16-byte chunks per operand tile; 256 threads x 2.
#pragma unroll
    for (int r = 0; r < 2; ++r) {
      const int c = tid + r * kGemmThreads;
      if (g.a_kmajor) {  // [BM][BK]: 4 chunks per row
        const int row = c >> 2, col = (c & 3) * 8;
        cp_async16(as + row * (BK + kPad) + col, g.A + static_cast<long>(m0 + row) * g.lda + k0 + col);
      } else {           // [BK][BM]: 16 chunks per row
        const int row = c >> 4, col = (c & 15) * 8;
        cp_async16(as + row * (BM + kPad) + col, g.A + static_cast<long>(k0 + row) * g.lda + m0 + col);
      }
      if (g.b_nmajor) {  // [BK][BN]
        const int row = c >> 4, col = (c & 15) * 8;
        cp_async16(bs + row * (BN + kPad) + col, g.B + static_cast<long>(k0 + row) * g.ldb + n0 + col);
      } else {           // [BN][BK]
        const int row = c >> 2, col = (c & 3) * 8;
        cp_async16(bs + row * (BK + kPad) + col, g.B + static_cast<long>(n0 + row) * g.ldb + k0 + col);
      }
    }
    cp_async_commit();
  };

  const int n_tiles = (k_end - k_begin + BK - 1) / BK;
  if (n_tiles > 0) load_tile(0, k_begin);
  for (int t = 0; t < n_tiles; ++t) {
    cp_async_wait_all();
    __syncthreads();
    if (t + 1 < n_tiles) load_tile((t + 1) & 1, k_begin + (t + 1) * BK);
    const __nv_bfloat16* as = As + (t & 1) * kAtile;
    const __nv_bfloat16* bs = Bs + (t & 1) * kBtile;
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[4][4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int mrow = wm * 64 + i * 16;
        if (g.a_kmajor) {
          const int r = mrow + (lane & 15), cc = kk + (lane >> 4) * 8;
          ldmatrix_x4(af[i], as + r * (BK + kPad) + cc);
        } else {
          // Stored [k][m]: matrices (k lo, m lo), (k lo, m hi), (k hi, m lo), (k hi, m hi)
          // map to a0a1, a2a3, a4a5, a6a7 via .trans.
          const int j = lane >> 3;
          const int krow = kk + (lane & 7) + ((j >> 1) << 3);
          const int mcol = mrow + ((j & 1) << 3);
          ldmatrix_x4_trans(af[i], as + krow * (BM + kPad) + mcol);
        }
      }
      uint32_t bf[4][2];
#pragma unroll
      for (int jp = 0; jp < 2; ++jp) {  // two n8 tiles per ldmatrix.x4
        const int ncol = wn * 32 + jp * 16;
        uint32_t r4[4];
        if (g.b_nmajor) {
          // Stored [k][n]: matrices (k lo, n lo), (k hi, n lo), (k lo, n hi), (k hi, n hi).
          const int j = lane >> 3;
          const int krow = kk + (lane & 7) + ((j & 1) << 3);
          const int nc = ncol + ((j >> 1) << 3);
          ldmatrix_x4_trans(r4, bs + krow * (BN + kPad) + nc);
        } else {
          // Stored [n][k]: matrices (n lo, k lo), (n lo, k hi), (n hi, k lo), (n hi, k hi).
          const int j = lane >> 3;
          const int nrow = ncol + (lane & 7) + ((j >> 1) << 3);
          const int kc = kk + ((j & 1) << 3);
          ldmatrix_x4(r4, bs + nrow * (BK + kPad) + kc);
        }
        bf[jp * 2][0] = r4[0];
        bf[jp * 2][1] = r4[1];
        bf[jp * 2 + 1][0] = r4[2];
        bf[jp * 2 + 1][1] = r4[3];
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) mma_bf16(acc[i][j], af[i], bf[j][0], bf[j][1]);
    }
  }

  // Epilogue.
  const int gq = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int col = n0 + wn * 32 + j * 8 + 2 * t4;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int row = m0 + wm * 64 + i * 16 + gq + h * 8;
        float v0 = acc[i][j][2 * h], v1 = acc[i][j][2 * h + 1];
        if (g.bias) {
          v0 += g.bias[col];
          v1 += g.bias[col + 1];
        }
        if (g.relu) {
          v0 = fmaxf(v0, 0.f);
          v1 = fmaxf(v1, 0.f);
        }
        if (g.relu_mask) {
          const __nv_bfloat162 m2 =
              *reinterpret_cast<const __nv_bfloat162*>(g.relu_mask + static_cast<long>(row) * g.ld_mask + col);
          if (!(__bfloat162float(m2.x) > 0.f)) v0 = 0.f;
          if (!(__bfloat162float(m2.y) > 0.f)) v1 = 0.f;
        }
        const long off = static_cast<long>(row) * g.ldc + col;
        if (g.C32) {
          if (g.atomic) {
            atomicAdd(g.C32 + off, v0);
            atomicAdd(g.C32 + off + 1, v1);
          } else {
            *reinterpret_cast<float2*>(g.C32 + off) = make_float2(v0, v1);
          }
        }
        if (g.C16) *reinterpret_cast<__nv_bfloat162*>(g.C16 + off) = __floats2bfloat162_rn(v0, v1);
      }
    }
  }
}

// ---------------------------------------------------------------- helpers

__global__ void f32_to_bf16_kernel(const float* x, __nv_bfloat16* y, long n) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// Deterministic uniform(-a, a) initialisation from a counter hash.
__global__ void init_uniform_kernel(float* p, long n, float a, unsigned long long seed) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  unsigned long long z = seed + 0x9E3779B97F4A7C15ull * static_cast<unsigned long long>(i + 1);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  const float u = static_cast<float>(z >> 40) * (1.0f / 16777216.0f);  // [0, 1)
  p[i] = (2.0f * u - 1.0f) * a;
}

// dY = 2 (Y - T) * mask / count over the valid outputs; loss sum into *loss.
__global__ void mse_grad_kernel(const float* y, const float* t, const float* mask, long rows, int n_out,
                                int ld, float inv_count, float* dy32, __nv_bfloat16* dy16, float* loss) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  float l = 0.f;
  if (i < rows * n_out) {
    const long r = i / n_out;
    const int c = static_cast<int>(i - r * n_out);
    const long off = r * ld + c;
    const float m = mask ? mask[off] : 1.0f;
    const float d = (y[off] - t[off]) * m;
    l = d * d;
    const float gr = 2.0f * d * inv_count;
    if (dy32) dy32[off] = gr;
    dy16[off] = __float2bfloat16_rn(gr);
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0 && loss) atomicAdd(loss, l * inv_count);
}

// Learned-MV output loss, one warp per row. The network's 128 outputs are 64
// complex weights w (interleaved); the row's input features hold the
// normalised subarray-averaged snapshot a at 128 + 2i; the mask selects
// i < L. With num = sum conj(w) a and D = conj(sum w) the combiner outputs
// o = num / D; the loss is |o - o_ref|^2 (o_ref from the target weights) plus
// |sum w / L - 1|^2 (the distortionless residual the plan gates on; it also
// keeps D away from zero) plus beta * |w - t|^2 over the masked outputs, all
// divided by `rows`. Gradients with respect to (Re w_i, Im w_i) are the real
// and imaginary parts of 2 conj(e) (a_i - o) / D + 2 (sum w / L - 1) / L +
// 2 beta (w_i - t_i).
__global__ void lmv_output_loss_kernel(const float* y, const float* t, const float* mask, const float* x,
                                       long rows, float beta, float inv_rows, __nv_bfloat16* dy16, float* loss) {
  const int lane = threadIdx.x & 31;
  const long r = (blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x) >> 5;
  if (r >= rows) return;
  const float4 w4 = reinterpret_cast<const float4*>(y + r * 128)[lane];
  const float4 t4 = reinterpret_cast<const float4*>(t + r * 128)[lane];
  const float4 m4 = mask ? reinterpret_cast<const float4*>(mask + r * 128)[lane] : make_float4(1.f, 1.f, 1.f, 1.f);
  const float4 a4 = reinterpret_cast<const float4*>(x + r * 256 + 128)[lane];
  // Two complex weights per lane: (w4.x, w4.y), (w4.z, w4.w).
  float nre = 0.f, nim = 0.f, dre = 0.f, dim = 0.f, rre = 0.f, rim = 0.f, tre = 0.f, tim = 0.f, wse = 0.f;
  float cnt = 0.f;
  auto acc = [&](float wr, float wi, float tr, float ti, float m, float ar, float ai) {
    if (m <= 0.f) return;
    cnt += 1.f;
    nre += wr * ar + wi * ai;   // conj(w) a
    nim += wr * ai - wi * ar;
    dre += wr;
    dim += wi;
    rre += tr * ar + ti * ai;
    rim += tr * ai - ti * ar;
    tre += tr;
    tim += ti;
    wse += (wr - tr) * (wr - tr) + (wi - ti) * (wi - ti);
  };
  acc(w4.x, w4.y, t4.x, t4.y, m4.x, a4.x, a4.y);
  acc(w4.z, w4.w, t4.z, t4.w, m4.z, a4.z, a4.w);
  for (int o = 16; o > 0; o >>= 1) {
    nre += __shfl_xor_sync(0xffffffffu, nre, o);
    nim += __shfl_xor_sync(0xffffffffu, nim, o);
    dre += __shfl_xor_sync(0xffffffffu, dre, o);
    dim += __shfl_xor_sync(0xffffffffu, dim, o);
    rre += __shfl_xor_sync(0xffffffffu, rre, o);
    rim += __shfl_xor_sync(0xffffffffu, rim, o);
    tre += __shfl_xor_sync(0xffffffffu, tre, o);
    tim += __shfl_xor_sync(0xffffffffu, tim, o);
    wse += __shfl_xor_sync(0xffffffffu, wse, o);
    cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  }
  const float inv_l = cnt > 0.f ? 1.0f / cnt : 0.f;
  const float sre = dre * inv_l - 1.0f, sim = dim * inv_l;   // sum w / L - 1
  // D = conj(sum w), guarded away from zero.
  float Dr = dre, Di = -dim;
  float dn = Dr * Dr + Di * Di;
  if (dn < 1e-6f) {
    Dr = 1e-3f;
    Di = 0.f;
    dn = 1e-6f;
  }
  // o = num / D; o_ref = (sum conj(t) a) / conj(sum t).
  const float ore = (nre * Dr + nim * Di) / dn, oim = (nim * Dr - nre * Di) / dn;
  const float Tr = tre, Ti = -tim, tn = fmaxf(Tr * Tr + Ti * Ti, 1e-12f);
  const float fre = (rre * Tr + rim * Ti) / tn, fim = (rim * Tr - rre * Ti) / tn;
  const float ere = ore - fre, eim = oim - fim;
  // c = 2 conj(e) / D
  const float cre0 = 2.f * ere, cim0 = -2.f * eim;
  const float cre = (cre0 * Dr + cim0 * Di) / dn, cim = (cim0 * Dr - cre0 * Di) / dn;
  auto grad = [&](float wr, float wi, float tr, float ti, float m, float ar, float ai, float& gr, float& gi) {
    gr = gi = 0.f;
    if (m <= 0.f) return;
    const float ur = ar - ore, ui = ai - oim;        // a_i - o
    gr = (cre * ur - cim * ui + 2.f * sre * inv_l + 2.f * beta * (wr - tr)) * inv_rows;
    gi = (cre * ui + cim * ur + 2.f * sim * inv_l + 2.f * beta * (wi - ti)) * inv_rows;
  };
  float g0, g1, g2, g3;
  grad(w4.x, w4.y, t4.x, t4.y, m4.x, a4.x, a4.y, g0, g1);
  grad(w4.z, w4.w, t4.z, t4.w, m4.z, a4.z, a4.w, g2, g3);
  __nv_bfloat162* d2 = reinterpret_cast<__nv_bfloat162*>(dy16 + r * 128) + 2 * lane;
  d2[0] = __floats2bfloat162_rn(g0, g1);
  d2[1] = __floats2bfloat162_rn(g2, g3);
  if (lane == 0 && loss) atomicAdd(loss, (ere * ere + eim * eim + sre * sre + sim * sim + beta * wse) * inv_rows);
}

// Learned-subspace loss, one warp per row. The refinement solves the Capon
// problem within span{DFT beams b = 0, +1, -1, +2, -2 (the first min(5, L)),
// network weights}, so what the network must supply is the direction of the
// Capon weights outside the beams. With P the projector onto the complement
// of the beams (length L = the masked count), u = P w, v = P t (w, t the
// predicted and target complex weights, i < L):
//   loss = 1 - |u^H v|^2 / (|u|^2 |v|^2)  +  beta * sum_i |w_i - t_i|^2 / L,
// scale- and phase-free in u; rows whose target lies in the beams' span
// (|v|^2 <= 1e-8 |t|^2) keep only the second term. d loss / d(Re w_i, Im w_i)
// is P applied to -2 (v conj(c) / (a b) - |c|^2 u / (a^2 b)) (c = u^H v,
// a = |u|^2, b = |v|^2) plus 2 beta (w_i - t_i) / L; all divided by `rows`.
__device__ __forceinline__ float2 wsum2(float2 v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
    v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
  }
  return v;
}

__global__ void lmv_subspace_loss_kernel(const float* y, const float* t, const float* mask, long rows,
                                         float beta, float inv_rows, __nv_bfloat16* dy16, float* loss) {
  const int lane = threadIdx.x & 31;
  const long r = (blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x) >> 5;
  if (r >= rows) return;
  const float4 w4 = reinterpret_cast<const float4*>(y + r * 128)[lane];
  const float4 t4 = reinterpret_cast<const float4*>(t + r * 128)[lane];
  const float4 m4 = mask ? reinterpret_cast<const float4*>(mask + r * 128)[lane] : make_float4(1.f, 1.f, 1.f, 1.f);
  float cnt = (m4.x > 0.f ? 1.f : 0.f) + (m4.z > 0.f ? 1.f : 0.f);
  for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
  const int L = static_cast<int>(cnt);
  float2 w[2] = {make_float2(w4.x, w4.y), make_float2(w4.z, w4.w)};
  float2 tv[2] = {make_float2(t4.x, t4.y), make_float2(t4.z, t4.w)};
  const bool in[2] = {2 * lane < L, 2 * lane + 1 < L};
  float2 tw1[2];   // e^{-j 2 pi i / L}
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    float sn = 0.f, cs = 1.f;
    if (in[h]) sincospif(2.0f * static_cast<float>((2 * lane + h) % max(L, 1)) / static_cast<float>(max(L, 1)), &sn, &cs);
    tw1[h] = make_float2(cs, -sn);
    if (!in[h]) w[h] = tv[h] = make_float2(0.f, 0.f);
  }
  const int nb = min(5, L);
  const float rs = L > 0 ? rsqrtf(static_cast<float>(L)) : 0.f;
  auto twk = [&](int h, int k) -> float2 {  // e^{-j 2 pi b i / L}, b = 0, 1, -1, 2, -2
    const float2 t1 = tw1[h];
    if (k == 0) return make_float2(1.f, 0.f);
    float2 q = t1;
    if (k >= 3) q = make_float2(t1.x * t1.x - t1.y * t1.y, 2.f * t1.x * t1.y);
    return (k & 1) ? q : make_float2(q.x, -q.y);
  };
  // u = P w, v = P t: subtract sum_b u_b (u_b^H x), u_b[i] = conj(twk) / sqrt(L).
  float2 u[2] = {w[0], w[1]}, v[2] = {tv[0], tv[1]};
  float tn = 0.f;
#pragma unroll
  for (int h = 0; h < 2; ++h) tn += tv[h].x * tv[h].x + tv[h].y * tv[h].y;
  for (int o = 16; o > 0; o >>= 1) tn += __shfl_xor_sync(0xffffffffu, tn, o);
  for (int k = 0; k < 5; ++k) {
    if (k >= nb) break;
    float2 cw = make_float2(0.f, 0.f), ct = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 q = twk(h, k);  // conj(u_b) sqrt(L)
      cw.x += q.x * w[h].x - q.y * w[h].y;
      cw.y += q.x * w[h].y + q.y * w[h].x;
      ct.x += q.x * tv[h].x - q.y * tv[h].y;
      ct.y += q.x * tv[h].y + q.y * tv[h].x;
    }
    cw = wsum2(cw);
    ct = wsum2(ct);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!in[h]) continue;
      const float2 q = twk(h, k);
      const float ubx = q.x * rs * rs, uby = -q.y * rs * rs;  // u_b / sqrt(L) (the coefficient carries sqrt(L))
      u[h].x -= cw.x * ubx - cw.y * uby;
      u[h].y -= cw.x * uby + cw.y * ubx;
      v[h].x -= ct.x * ubx - ct.y * uby;
      v[h].y -= ct.x * uby + ct.y * ubx;
    }
  }
  float2 c = make_float2(0.f, 0.f);
  float a = 0.f, b = 0.f, se = 0.f;
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    c.x += u[h].x * v[h].x + u[h].y * v[h].y;   // conj(u) v
    c.y += u[h].x * v[h].y - u[h].y * v[h].x;
    a += u[h].x * u[h].x + u[h].y * u[h].y;
    b += v[h].x * v[h].x + v[h].y * v[h].y;
    se += (w[h].x - tv[h].x) * (w[h].x - tv[h].x) + (w[h].y - tv[h].y) * (w[h].y - tv[h].y);
  }
  c = wsum2(c);
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    se += __shfl_xor_sync(0xffffffffu, se, o);
  }
  const float inv_l = L > 0 ? 1.0f / static_cast<float>(L) : 0.f;
  const bool dir = b > 1e-8f * tn && a > 1e-30f;
  const float c2 = c.x * c.x + c.y * c.y;
  const float f = dir ? c2 / (a * b) : 1.0f;
  // g = -2 (v conj(c) / (a b) - |c|^2 u / (a^2 b)) on the complement, then P.
  float2 g[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    g[h] = make_float2(0.f, 0.f);
    if (dir && in[h]) {
      const float2 vc = make_float2(v[h].x * c.x + v[h].y * c.y, v[h].y * c.x - v[h].x * c.y);  // v conj(c)
      const float s1 = 1.0f / (a * b), s2 = c2 / (a * a * b);
      g[h] = make_float2(-2.f * (vc.x * s1 - u[h].x * s2), -2.f * (vc.y * s1 - u[h].y * s2));
    }
  }
  for (int k = 0; k < 5; ++k) {   // P g (P is self-adjoint)
    if (k >= nb) break;
    float2 cg = make_float2(0.f, 0.f);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 q = twk(h, k);
      cg.x += q.x * g[h].x - q.y * g[h].y;
      cg.y += q.x * g[h].y + q.y * g[h].x;
    }
    cg = wsum2(cg);
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      if (!in[h]) continue;
      const float2 q = twk(h, k);
      const float ubx = q.x * rs * rs, uby = -q.y * rs * rs;
      g[h].x -= cg.x * ubx - cg.y * uby;
      g[h].y -= cg.x * uby + cg.y * ubx;
    }
  }
  float gg[4];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const float ex = in[h] ? 2.f * beta * (w[h].x - tv[h].x) * inv_l : 0.f;
    const float ey = in[h] ? 2.f * beta * (w[h].y - tv[h].y) * inv_l : 0.f;
    gg[2 * h] = (g[h].x + ex) * inv_rows;
    gg[2 * h + 1] = (g[h].y + ey) * inv_rows;
  }
  __nv_bfloat162* d2 = reinterpret_cast<__nv_bfloat162*>(dy16 + r * 128) + 2 * lane;
  d2[0] = __floats2bfloat162_rn(gg[0], gg[1]);
  d2[1] = __floats2bfloat162_rn(gg[2], gg[3]);
  if (lane == 0 && loss) atomicAdd(loss, ((dir ? 1.0f - f : 0.0f) + beta * se * inv_l) * inv_rows);
}

// db[n] += sum_m dY[m][n] (FP32 gradient rows as BF16 tiles were used in GEMMs).
__global__ void bias_grad_kernel(const __nv_bfloat16* dy, long rows, int n, int ld, float* db) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= n) return;
  float s = 0.f;
  for (long r = blockIdx.y; r < rows; r += gridDim.y) s += __bfloat162float(dy[r * ld + col]);
  atomicAdd(db + col, s);
}

__global__ void adam_kernel(float* p, const float* grad, float* m, float* v, long n, float lr, float b1, float b2,
                            float c1, float c2, float eps, __nv_bfloat16* p16) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float gr = grad[i];
  const float mi = b1 * m[i] + (1.f - b1) * gr;
  const float vi = b2 * v[i] + (1.f - b2) * gr * gr;
  m[i] = mi;
  v[i] = vi;
  const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  p[i] = pi;
  if (p16) p16[i] = __float2bfloat16_rn(pi);
}

}  // namespace

int launch_gemm(cudaStream_t st, const __nv_bfloat16* A, int lda, bool a_kmajor, const __nv_bfloat16* B, int ldb,
                bool b_nmajor, int M, int N, int K, const float* bias, bool relu, const __nv_bfloat16* relu_mask,
                int ld_mask, __nv_bfloat16* C16, float* C32, int ldc, int split_k) {
  if (M % BM || N % BN || K % BK) return fail(USX_ERR_INVALID, "gemm: M, N must be multiples of 128 and K of 32");
  GemmArgs g;
  g.A = A;
  g.B = B;
  g.M = M;
  g.N = N;
  g.K = K;
  g.lda = lda;
  g.ldb = ldb;
  g.a_kmajor = a_kmajor;
  g.b_nmajor = b_nmajor;
  g.bias = bias;
  g.relu = relu;
  g.relu_mask = relu_mask;
  g.ld_mask = ld_mask;
  g.C16 = C16;
  g.C32 = C32;
  g.ldc = ldc;
  split_k = std::max(1, split_k);
  g.atomic = split_k > 1;
  g.k_per_split = ((K / split_k + BK - 1) / BK) * BK;
  const int nz = (K + g.k_per_split - 1) / g.k_per_split;
  if (int rc_ = smem_limit(reinterpret_cast<const void*>(gemm_bf16_kernel), static_cast<size_t>(static_cast<int>(kGemmSmem)))) return rc_;
  gemm_bf16_kernel<<<dim3(N / BN, M / BM, nz), kGemmThreads, kGemmSmem, st>>>(g);
  USX_CHECK_LAUNCH("gemm_bf16_kernel");
  return USX_OK;
}

}  // namespace usxcu

using namespace usxcu;

// The network: layers l = 0..n_layers-1, W_l [in_l x out_l] row-major, b_l [out_l].
struct usx_mlp {
  usx_ctx* ctx = nullptr;
  int device = 0;
  int n_layers = 0;
  std::vector<int> dims;            // n_layers + 1
  std::vector<size_t> w_off, b_off; // offsets into the parameter vector
  size_t n_params = 0;
  float* p = nullptr;               // FP32 master parameters
  float* grad = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  __nv_bfloat16* p16 = nullptr;     // BF16 copy used by the GEMMs
  __nv_bfloat16* p16t = nullptr;    // the same with each W_l transposed ([out][in]) for the tcgen05 GEMM
  int gemm_path = USX_MLP_GEMM_AUTO;
  long step = 0;
  // Activation workspace for `cap` rows.
  long cap = 0;
  std::vector<__nv_bfloat16*> act;  // n_layers + 1 BF16 activations (act[0] = input)
  float* out32 = nullptr;           // final FP32 output
  __nv_bfloat16* g16a = nullptr;    // gradient buffers
  __nv_bfloat16* g16b = nullptr;
  float* loss = nullptr;
  int loss_kind = USX_MLP_LOSS_MSE;
  float loss_beta = 0.0f;
};

namespace {

int mlp_reserve(usx_mlp* n, long rows) {
  rows = (rows + 127) / 128 * 128;
  if (rows <= n->cap) return USX_OK;
  USX_CUDA(cudaStreamSynchronize(n->ctx->stream));
  for (auto* a : n->act) cudaFree(a);
  cudaFree(n->out32);
  cudaFree(n->g16a);
  cudaFree(n->g16b);
  n->act.assign(static_cast<size_t>(n->n_layers + 1), nullptr);
  int widest = 0;
  for (int d : n->dims) widest = std::max(widest, d);
  for (int l = 0; l <= n->n_layers; ++l)
    USX_CUDA(cudaMalloc(&n->act[static_cast<size_t>(l)], sizeof(__nv_bfloat16) * rows * n->dims[static_cast<size_t>(l)]));
  USX_CUDA(cudaMalloc(&n->out32, sizeof(float) * rows * n->dims.back()));
  USX_CUDA(cudaMalloc(&n->g16a, sizeof(__nv_bfloat16) * rows * widest));
  USX_CUDA(cudaMalloc(&n->g16b, sizeof(__nv_bfloat16) * rows * widest));
  n->cap = rows;
  return USX_OK;
}

// p16t <- per-layer transposes of p16, after every change of the weights.
int refresh_transposed(usx_mlp* n) {
  for (int l = 0; l < n->n_layers; ++l)
    if (int rc = transpose_bf16(n->ctx->stream, n->p16 + n->w_off[static_cast<size_t>(l)],
                                n->dims[static_cast<size_t>(l)], n->dims[static_cast<size_t>(l + 1)],
                                n->p16t + n->w_off[static_cast<size_t>(l)]))
      return rc;
  return USX_OK;
}

// Layer l forward: out = act(in W_l + b_l), ReLU on all but the last layer,
// BF16 (dst16) and / or FP32 (dst32) output. The tcgen05 GEMM takes the
// layers whose shape it supports; the mma.sync GEMM the rest.
int layer_forward(usx_mlp* n, usx_ctx* ctx, int l, const __nv_bfloat16* in, long rows, __nv_bfloat16* dst16,
                  float* dst32, const char* tc5_tag, const char* mma_tag) {
  const int din = n->dims[static_cast<size_t>(l)], dout = n->dims[static_cast<size_t>(l + 1)];
  const bool relu = l < n->n_layers - 1;
  const float* bias = n->p + n->b_off[static_cast<size_t>(l)];
  if (n->gemm_path == USX_MLP_GEMM_AUTO && gemm_tc5_supported(static_cast<int>(rows), dout, din)) {
    prof_begin(ctx, tc5_tag);
    const int rc = launch_gemm_tc5(ctx, in, n->p16t + n->w_off[static_cast<size_t>(l)], bias, relu, dst16, dst32,
                                   static_cast<int>(rows), dout, din);
    prof_end(ctx);
    return rc;
  }
  prof_begin(ctx, mma_tag);
  const int rc = launch_gemm(ctx->stream, in, din, true, n->p16 + n->w_off[static_cast<size_t>(l)], dout, true,
                             static_cast<int>(rows), dout, din, bias, relu, nullptr, 0, dst16, dst32, dout, 1);
  prof_end(ctx);
  return rc;
}

int mlp_forward_rows(usx_mlp* n, long rows) {
  for (int l = 0; l < n->n_layers; ++l) {
    const bool last = l == n->n_layers - 1;
    if (int rc = layer_forward(n, n->ctx, l, n->act[static_cast<size_t>(l)], rows, n->act[static_cast<size_t>(l + 1)],
                               last ? n->out32 : nullptr, "gemm_tc5_kernel(fwd)", "gemm_bf16_kernel(fwd)"))
      return rc;
  }
  return USX_OK;
}

}  // namespace

namespace usxcu {

int mlp_widest(const usx_mlp* n) {
  int widest = 0;
  for (int d : n->dims) widest = std::max(widest, d);
  return widest;
}

bool mlp_is_lmv(const usx_mlp* n) { return n->dims.front() == kLmvFeatures && n->dims.back() == kLmvOutputs; }

int mlp_infer(usx_mlp* n, usx_ctx* ctx, const void* x16, long rows, void* t0, void* t1, float* out32) {
  if (rows % 128) return fail(USX_ERR_INVALID, "mlp_infer: rows must be a multiple of 128");
  const __nv_bfloat16* in = static_cast<const __nv_bfloat16*>(x16);
  __nv_bfloat16* ping[2] = {static_cast<__nv_bfloat16*>(t0), static_cast<__nv_bfloat16*>(t1)};
  for (int l = 0; l < n->n_layers; ++l) {
    const bool last = l == n->n_layers - 1;
    __nv_bfloat16* dst = last ? nullptr : ping[l & 1];
    if (int rc = layer_forward(n, ctx, l, in, rows, dst, last ? out32 : nullptr, "gemm_tc5_kernel(lmv)",
                               "gemm_bf16_kernel(lmv)"))
      return rc;
    in = dst;
  }
  return USX_OK;
}

}  // namespace usxcu

extern "C" {

int usx_cu_mlp_create(usx_ctx* ctx, int n_layers, const int* dims, uint64_t seed, usx_mlp** out) {
  if (!ctx || !dims || !out || n_layers < 1) return fail(USX_ERR_INVALID, "usx_cu_mlp_create: bad arguments");
  for (int l = 0; l <= n_layers; ++l)
    if (dims[l] <= 0 || dims[l] % 128)
      return fail(USX_ERR_INVALID, "usx_cu_mlp_create: layer widths must be positive multiples of 128");
  usx_mlp* n = new usx_mlp();
  n->ctx = ctx;
  n->device = ctx->device;
  n->n_layers = n_layers;
  n->dims.assign(dims, dims + n_layers + 1);
  size_t off = 0;
  for (int l = 0; l < n_layers; ++l) {
    n->w_off.push_back(off);
    off += static_cast<size_t>(dims[l]) * dims[l + 1];
    n->b_off.push_back(off);
    off += static_cast<size_t>(dims[l + 1]);
  }
  n->n_params = off;
  cudaError_t e = cudaSuccess;
  e = e == cudaSuccess ? cudaMalloc(&n->p, sizeof(float) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->grad, sizeof(float) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->m, sizeof(float) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->v, sizeof(float) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->p16, sizeof(__nv_bfloat16) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->p16t, sizeof(__nv_bfloat16) * off) : e;
  e = e == cudaSuccess ? cudaMalloc(&n->loss, sizeof(float) * 4) : e;
  if (e != cudaSuccess) {
    usx_cu_mlp_destroy(n);
    return cuda_fail(e, "usx_cu_mlp_create");
  }
  cudaStream_t st = ctx->stream;
  cudaMemsetAsync(n->m, 0, sizeof(float) * off, st);
  cudaMemsetAsync(n->v, 0, sizeof(float) * off, st);
  for (int l = 0; l < n_layers; ++l) {
    // He-uniform weights (ReLU net), zero biases.
    const long nw = static_cast<long>(dims[l]) * dims[l + 1];
    const float a = std::sqrt(6.0f / static_cast<float>(dims[l]));
    init_uniform_kernel<<<ceil_div(nw, 256), 256, 0, st>>>(n->p + n->w_off[static_cast<size_t>(l)], nw, a,
                                                           seed * 1315423911ull + static_cast<unsigned long long>(l));
    cudaMemsetAsync(n->p + n->b_off[static_cast<size_t>(l)], 0, sizeof(float) * dims[l + 1], st);
  }
  f32_to_bf16_kernel<<<ceil_div(static_cast<long>(off), 256), 256, 0, st>>>(n->p, n->p16, static_cast<long>(off));
  USX_CHECK_LAUNCH("usx_cu_mlp_create");
  if (int rc = refresh_transposed(n)) {
    usx_cu_mlp_destroy(n);
    return rc;
  }
  *out = n;
  return USX_OK;
}

int usx_cu_mlp_destroy(usx_mlp* n) {
  if (!n) return USX_OK;
  // The context may already be gone: synchronise the device, not its stream.
  cudaSetDevice(n->device);
  cudaDeviceSynchronize();
  for (auto* a : n->act) cudaFree(a);
  cudaFree(n->out32);
  cudaFree(n->g16a);
  cudaFree(n->g16b);
  cudaFree(n->p);
  cudaFree(n->grad);
  cudaFree(n->m);
  cudaFree(n->v);
  cudaFree(n->p16);
  cudaFree(n->p16t);
  cudaFree(n->loss);
  delete n;
  return USX_OK;
}

int usx_cu_mlp_num_params(const usx_mlp* n, int64_t* count) {
  if (!n || !count) return fail(USX_ERR_INVALID, "usx_cu_mlp_num_params: null argument");
  *count = static_cast<int64_t>(n->n_params);
  return USX_OK;
}

int usx_cu_mlp_get_params(usx_mlp* n, float* host) {
  if (!n || !host) return fail(USX_ERR_INVALID, "usx_cu_mlp_get_params: null argument");
  USX_CUDA(cudaMemcpyAsync(host, n->p, sizeof(float) * n->n_params, cudaMemcpyDeviceToHost, n->ctx->stream));
  USX_CUDA(cudaStreamSynchronize(n->ctx->stream));
  return USX_OK;
}

int usx_cu_mlp_set_params(usx_mlp* n, const float* host) {
  if (!n || !host) return fail(USX_ERR_INVALID, "usx_cu_mlp_set_params: null argument");
  USX_CUDA(cudaMemcpyAsync(n->p, host, sizeof(float) * n->n_params, cudaMemcpyHostToDevice, n->ctx->stream));
  f32_to_bf16_kernel<<<ceil_div(static_cast<long>(n->n_params), 256), 256, 0, n->ctx->stream>>>(
      n->p, n->p16, static_cast<long>(n->n_params));
  USX_CHECK_LAUNCH("f32_to_bf16_kernel");
  if (int rc = refresh_transposed(n)) return rc;
  USX_CUDA(cudaStreamSynchronize(n->ctx->stream));
  return USX_OK;
}

int usx_cu_mlp_set_gemm_path(usx_mlp* n, int path) {
  if (!n) return fail(USX_ERR_INVALID, "usx_cu_mlp_set_gemm_path: null network");
  if (path != USX_MLP_GEMM_AUTO && path != USX_MLP_GEMM_MMA_SYNC)
    return fail(USX_ERR_INVALID, "usx_cu_mlp_set_gemm_path: unknown path");
  n->gemm_path = path;
  return USX_OK;
}

int usx_cu_mlp_set_loss(usx_mlp* n, int kind, float beta) {
  if (!n) return fail(USX_ERR_INVALID, "usx_cu_mlp_set_loss: null network");
  if (kind != USX_MLP_LOSS_MSE && kind != USX_MLP_LOSS_LMV_OUTPUT && kind != USX_MLP_LOSS_LMV_SUBSPACE)
    return fail(USX_ERR_INVALID, "usx_cu_mlp_set_loss: unknown loss");
  if (kind != USX_MLP_LOSS_MSE && !(n->dims.front() == 256 && n->dims.back() == 128))
    return fail(USX_ERR_INVALID, "usx_cu_mlp_set_loss: the output loss needs a 256 -> 128 network");
  if (!(beta >= 0.0f)) return fail(USX_ERR_INVALID, "usx_cu_mlp_set_loss: beta must be >= 0");
  n->loss_kind = kind;
  n->loss_beta = beta;
  return USX_OK;
}

// y[rows x dims.back()] (FP32) = net(x[rows x dims[0]] FP32), device pointers.
int usx_cu_mlp_forward(usx_mlp* n, const float* x, int64_t rows, float* y) {
  if (!n || !x || !y) return fail(USX_ERR_INVALID, "usx_cu_mlp_forward: null argument");
  if (rows <= 0) return USX_OK;
  if (int rc = mlp_reserve(n, rows)) return rc;
  const long padded = (rows + 127) / 128 * 128;
  cudaStream_t st = n->ctx->stream;
  const long nin = static_cast<long>(rows) * n->dims[0];
  if (padded > rows)
    USX_CUDA(cudaMemsetAsync(n->act[0] + nin, 0, sizeof(__nv_bfloat16) * (padded - rows) * n->dims[0], st));
  f32_to_bf16_kernel<<<ceil_div(nin, 256), 256, 0, st>>>(x, n->act[0], nin);
  USX_CHECK_LAUNCH("f32_to_bf16_kernel");
  if (int rc = mlp_forward_rows(n, padded)) return rc;
  USX_CUDA(cudaMemcpyAsync(y, n->out32, sizeof(float) * rows * n->dims.back(), cudaMemcpyDeviceToDevice, st));
  return USX_OK;
}

// Gradients of the mean squared error over the masked outputs for one batch;
// with `lr` > 0 also one Adam step. grad_host (optional) receives the
// gradient vector (same layout as the parameters); loss_host the batch loss.
int usx_cu_mlp_train_step(usx_mlp* n, const float* x, const float* target, const float* mask, int64_t rows,
                          float lr, float* loss_host, float* grad_host) {
  if (!n || !x || !target) return fail(USX_ERR_INVALID, "usx_cu_mlp_train_step: null argument");
  if (rows <= 0 || rows % 128) return fail(USX_ERR_INVALID, "usx_cu_mlp_train_step: rows must be a positive multiple of 128");
  if (int rc = mlp_reserve(n, rows)) return rc;
  cudaStream_t st = n->ctx->stream;
  const int L = n->n_layers;
  const long nin = static_cast<long>(rows) * n->dims[0];
  f32_to_bf16_kernel<<<ceil_div(nin, 256), 256, 0, st>>>(x, n->act[0], nin);
  USX_CHECK_LAUNCH("f32_to_bf16_kernel");
  if (int rc = mlp_forward_rows(n, rows)) return rc;
  USX_CUDA(cudaMemsetAsync(n->grad, 0, sizeof(float) * n->n_params, st));
  USX_CUDA(cudaMemsetAsync(n->loss, 0, sizeof(float), st));
  const int n_out = n->dims.back();
  if (n->loss_kind == USX_MLP_LOSS_LMV_SUBSPACE) {
    lmv_subspace_loss_kernel<<<ceil_div(static_cast<long>(rows) * 32, 256), 256, 0, st>>>(
        n->out32, target, mask, rows, n->loss_beta, 1.0f / static_cast<float>(rows), n->g16a, n->loss);
    USX_CHECK_LAUNCH("lmv_subspace_loss_kernel");
  } else if (n->loss_kind == USX_MLP_LOSS_LMV_OUTPUT) {
    lmv_output_loss_kernel<<<ceil_div(static_cast<long>(rows) * 32, 256), 256, 0, st>>>(
        n->out32, target, mask, x, rows, n->loss_beta, 1.0f / static_cast<float>(rows), n->g16a, n->loss);
    USX_CHECK_LAUNCH("lmv_output_loss_kernel");
  } else {
    // Count of valid outputs (mask sum) is taken as rows * n_out when no mask.
    const float inv_count = 1.0f / static_cast<float>(rows * n_out);
    mse_grad_kernel<<<ceil_div(static_cast<long>(rows) * n_out, 256), 256, 0, st>>>(
        n->out32, target, mask, rows, n_out, n_out, inv_count, nullptr, n->g16a, n->loss);
    USX_CHECK_LAUNCH("mse_grad_kernel");
  }
  __nv_bfloat16* dcur = n->g16a;   // gradient w.r.t. layer l output
  __nv_bfloat16* dnext = n->g16b;
  for (int l = L - 1; l >= 0; --l) {
    const int din = n->dims[static_cast<size_t>(l)], dout = n->dims[static_cast<size_t>(l + 1)];
    // dW_l = act_l^T dcur  (K = rows, split to fill the GPU)
    const int split = static_cast<int>(std::max<long>(1, std::min<long>(rows / 512, 64)));
    prof_begin(n->ctx, "gemm_bf16_kernel(dW)");
    if (int rc = launch_gemm(st, n->act[static_cast<size_t>(l)], din, false, dcur, dout, true, din, dout,
                             static_cast<int>(rows), nullptr, false, nullptr, 0, nullptr,
                             n->grad + n->w_off[static_cast<size_t>(l)], dout, split))
      return rc;
    prof_end(n->ctx);
    bias_grad_kernel<<<dim3(ceil_div(dout, 128), 64), 128, 0, st>>>(dcur, rows, dout, dout,
                                                                    n->grad + n->b_off[static_cast<size_t>(l)]);
    USX_CHECK_LAUNCH("bias_grad_kernel");
    if (l > 0) {
      // d act_l = dcur W_l^T, masked by ReLU'(act_l)
      prof_begin(n->ctx, "gemm_bf16_kernel(dX)");
      if (int rc = launch_gemm(st, dcur, dout, true, n->p16 + n->w_off[static_cast<size_t>(l)], dout, false,
                               static_cast<int>(rows), din, dout, nullptr, false, n->act[static_cast<size_t>(l)], din,
                               dnext, nullptr, din, 1))
        return rc;
      prof_end(n->ctx);
      std::swap(dcur, dnext);
    }
  }
  if (lr > 0.0f) {
    ++n->step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, static_cast<float>(n->step));
    const float c2 = 1.0f - std::pow(b2, static_cast<float>(n->step));
    adam_kernel<<<ceil_div(static_cast<long>(n->n_params), 256), 256, 0, st>>>(
        n->p, n->grad, n->m, n->v, static_cast<long>(n->n_params), lr, b1, b2, c1, c2, 1e-8f, n->p16);
    USX_CHECK_LAUNCH("adam_kernel");
    if (int rc = refresh_transposed(n)) return rc;
  }
  if (grad_host) {
    USX_CUDA(cudaMemcpyAsync(grad_host, n->grad, sizeof(float) * n->n_params, cudaMemcpyDeviceToHost, st));
  }
  if (loss_host) {
    USX_CUDA(cudaMemcpyAsync(loss_host, n->loss, sizeof(float), cudaMemcpyDeviceToHost, st));
  }
  if (grad_host || loss_host) USX_CUDA(cudaStreamSynchronize(st));
  return USX_OK;
}

}  // extern "C"
