// post.cu — envelope (|IQ| or Hilbert), time-gain compensation, log
// compression and polar-to-Cartesian scan conversion (reference
// postprocess.cpp:12-178). All are HBM-bound elementwise or per-line kernels.
//
// The Hilbert transform reproduces the reference's radix-2 FFT exactly: the
// per-stage twiddle sequence w_k = w_{k-1} * w_len is generated on the host
// with the same float recurrence and uploaded, so every butterfly sees the
// same twiddle value the reference's serial loop does.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "usx_internal.cuh"

namespace usxcu {
namespace {

__global__ void envelope_iq_kernel(const float2* frame, float* env, long n) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i < n) {
    const float2 z = frame[i];
    env[i] = hypotf(z.x, z.y);
  }
}

// One block per line: analytic signal of the real part, modulus out.
// tw holds the forward then the inverse twiddle tables, (n_fft - 1) each,
// stage `len` starting at offset len/2 - 1.
__global__ void hilbert_kernel(const float2* frame, int n1, int n_fft, int log2n, const float2* tw,
                               float* env) {
  extern __shared__ float2 buf[];
  const long line = blockIdx.x;
  const float2* src = frame + line * n1;
  // Load with bit-reversed placement (the reference's in-place reversal).
  for (int i = threadIdx.x; i < n_fft; i += blockDim.x) {
    const int r = static_cast<int>(__brev(static_cast<unsigned>(i)) >> (32 - log2n));
    buf[r] = make_float2(i < n1 ? src[i].x : 0.0f, 0.0f);
  }
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass) {
    const float2* twp = tw + (pass == 0 ? 0 : (n_fft - 1));
    for (int len = 2; len <= n_fft; len <<= 1) {
      const int half = len >> 1;
      const float2* w = twp + (half - 1);
      for (int b = threadIdx.x; b < n_fft / 2; b += blockDim.x) {
        const int grp = b / half, k = b - grp * half;
        const int i0 = grp * len + k, i1 = i0 + half;
        const cplx u = mk(buf[i0].x, buf[i0].y);
        const cplx v = cmul(mk(buf[i1].x, buf[i1].y), mk(w[k].x, w[k].y));
        const cplx s = cadd(u, v), d = csub(u, v);
        buf[i0] = make_float2(s.re, s.im);
        buf[i1] = make_float2(d.re, d.im);
      }
      __syncthreads();
    }
    if (pass == 0) {
      // Double positive frequencies, zero negative ones, then bit-reverse for
      // the inverse transform.
      for (int k = threadIdx.x; k < n_fft; k += blockDim.x) {
        float2 v = buf[k];
        if (k >= 1 && k < n_fft / 2) v = make_float2(v.x * 2.0f, v.y * 2.0f);
        else if (k > n_fft / 2) v = make_float2(0.0f, 0.0f);
        buf[k] = v;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < n_fft; i += blockDim.x) {
        const int r = static_cast<int>(__brev(static_cast<unsigned>(i)) >> (32 - log2n));
        if (i < r) {
          const float2 t = buf[i];
          buf[i] = buf[r];
          buf[r] = t;
        }
      }
      __syncthreads();
    }
  }
  const float inv_n = static_cast<float>(n_fft);
  for (int j = threadIdx.x; j < n1; j += blockDim.x) {
    const float2 v = buf[j];
    env[line * n1 + j] = hypotf(v.x / inv_n, v.y / inv_n);
  }
}

__global__ void tgc_kernel(const float* env, const float* points, float atten, float f_mhz, long n,
                           float* out) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float depth_cm = points[3 * i + 2] * 100.0f;
  const float gain_db = 2.0f * atten * f_mhz * fmaxf(depth_cm, 0.0f);
  out[i] = env[i] * powf(10.0f, gain_db / 20.0f);
}

// Launched with 256 threads. The block reduces in shared memory and issues one
// atomic: one atomic per warp onto a single word serialises thousands of them.
__global__ void __launch_bounds__(256) max_kernel(const float* x, long n, unsigned* out_bits) {
  __shared__ float warp_max[8];
  float m = 0.0f;
  for (long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long>(gridDim.x) * blockDim.x)
    m = fmaxf(m, x[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x < 32) {
    m = threadIdx.x < 8 ? warp_max[threadIdx.x] : 0.0f;
    for (int o = 4; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    // Non-negative floats order like their bit patterns.
    if (threadIdx.x == 0 && m > 0.0f) atomicMax(out_bits, __float_as_uint(m));
  }
}

__global__ void log_compress_kernel(const float* env, long n, float dr_db, float gain_db,
                                    float reference, const unsigned* ref_bits, float* out) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  const float ref = reference > 0.0f ? reference : __uint_as_float(*ref_bits);
  if (ref <= 0.0f) {
    out[i] = 0.0f;
    return;
  }
  const float dr = fmaxf(dr_db, 1.0f);
  const float v = env[i] / ref;
  const float db = (v > 0.0f) ? 20.0f * log10f(v) : -1e6f;
  out[i] = fclamp((db + gain_db + dr) / dr, 0.0f, 1.0f);
}

struct ScanArgs {
  const float* image;
  float* pixels;
  int n0, n1, width, height, cart;
  float x_min, x_max, z_min, z_max;
  float a0_first, a0_last, a1_first, a1_last;
  float apex_x, apex_z;
  float fill;
};

// One output pixel of the backward mapping (postprocess.cpp:139-176):
// `fill` outside the grid, else the bilinear interpolation of the image.
__device__ __forceinline__ float scan_pixel(const ScanArgs& s, int px, int py) {
  float val = s.fill;
  const float z = s.z_min + (s.z_max - s.z_min) *
                                (s.height == 1 ? 0.0f : static_cast<float>(py) / static_cast<float>(s.height - 1));
  const float x = s.x_min + (s.x_max - s.x_min) *
                                (s.width == 1 ? 0.0f : static_cast<float>(px) / static_cast<float>(s.width - 1));
  float u, v;
  bool inside = true;
  if (s.cart) {
    u = (x - s.a0_first) / fmaxf(s.a0_last - s.a0_first, 1e-9f) * static_cast<float>(s.n0 - 1);
    v = (z - s.a1_first) / fmaxf(s.a1_last - s.a1_first, 1e-9f) * static_cast<float>(s.n1 - 1);
  } else {
    const float dx = x - s.apex_x, dz = z - s.apex_z;
    const float r = sqrtf(dx * dx + dz * dz);
    const float th = atan2f(dx, dz);
    const float th0 = s.a0_first, th1 = s.a0_last, r0 = s.a1_first, r1 = s.a1_last;
    if (r < fminf(r0, r1) || r > fmaxf(r0, r1) || th < fminf(th0, th1) || th > fmaxf(th0, th1))
      inside = false;
    u = (th - th0) / fmaxf(th1 - th0, 1e-9f) * static_cast<float>(s.n0 - 1);
    v = (r - r0) / fmaxf(r1 - r0, 1e-9f) * static_cast<float>(s.n1 - 1);
  }
  if (inside) {
    const int i0 = static_cast<int>(floorf(u)), j0 = static_cast<int>(floorf(v));
    if (i0 >= 0 && j0 >= 0 && i0 + 1 < s.n0 && j0 + 1 < s.n1) {
      const float fu = u - static_cast<float>(i0), fv = v - static_cast<float>(j0);
      const long n1 = s.n1;
      const float a = s.image[i0 * n1 + j0];
      const float b = s.image[(i0 + 1) * n1 + j0];
      const float cc = s.image[i0 * n1 + j0 + 1];
      const float d = s.image[(i0 + 1) * n1 + j0 + 1];
      val = (a * (1.0f - fu) + b * fu) * (1.0f - fv) + (cc * (1.0f - fu) + d * fu) * fv;
    }
  }
  return val;
}

// A 32 x 32 tile of the raster per 256-thread block. The image is stored
// lateral-major (axis 1, depth, contiguous) while the raster is row-major in
// depth, so the lanes of a warp first walk depth (py) at one px, which makes
// the four bilinear taps contiguous reads along the image's rows; the tile is
// then transposed through shared memory so that each warp writes 32
// consecutive raster pixels.
constexpr int kScanTile = 32;
__global__ void __launch_bounds__(256) scan_convert_kernel(const ScanArgs s) {
  __shared__ float tile[kScanTile][kScanTile + 1];
  const int lane = threadIdx.x & 31, row = threadIdx.x >> 5;
  const int px0 = blockIdx.x * kScanTile, py0 = blockIdx.y * kScanTile;
#pragma unroll
  for (int k = 0; k < kScanTile / 8; ++k) {
    const int lx = row + 8 * k, px = px0 + lx, py = py0 + lane;
    if (px < s.width && py < s.height) tile[lx][lane] = scan_pixel(s, px, py);
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < kScanTile / 8; ++k) {
    const int ly = row + 8 * k, px = px0 + lane, py = py0 + ly;
    if (px < s.width && py < s.height) s.pixels[static_cast<long>(py) * s.width + px] = tile[lane][ly];
  }
}

}  // namespace
}  // namespace usxcu

using namespace usxcu;

namespace {
// Running extent of (x, z) over sample points [x, y, z].
struct Extent {
  float x_min = std::numeric_limits<float>::max(), x_max = -std::numeric_limits<float>::max();
  float z_min = std::numeric_limits<float>::max(), z_max = -std::numeric_limits<float>::max();
  void add(const float* p) {
    x_min = std::min(x_min, p[0]);
    x_max = std::max(x_max, p[0]);
    z_min = std::min(z_min, p[2]);
    z_max = std::max(z_max, p[2]);
  }
  void merge(const Extent& o) {
    x_min = std::min(x_min, o.x_min);
    x_max = std::max(x_max, o.x_max);
    z_min = std::min(z_min, o.z_min);
    z_max = std::max(z_max, o.z_max);
  }
};
}  // namespace

extern "C" {

int usx_cu_envelope(usx_ctx* ctx, const float* frame, int n0, int n1, float fdem, float* env) {
  if (!ctx || !frame || !env) return fail(USX_ERR_INVALID, "usx_cu_envelope: null argument");
  if (n0 <= 0 || n1 <= 0) return fail(USX_ERR_INVALID, "usx_cu_envelope: empty frame");
  const long n = static_cast<long>(n0) * n1;
  if (fdem > 0.0f) {
    prof_begin(ctx, "envelope_iq_kernel");
    envelope_iq_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(
        reinterpret_cast<const float2*>(frame), env, n);
    prof_end(ctx);
    USX_CHECK_LAUNCH("envelope_iq_kernel");
    return USX_OK;
  }
  int n_fft = 1, log2n = 0;
  while (n_fft < n1) {
    n_fft <<= 1;
    ++log2n;
  }
  if (n_fft > 16384) return fail(USX_ERR_UNSUPPORTED, "usx_cu_envelope: lines longer than 16384");
  if (n_fft < 2) {
    // A one-sample line: the reference's FFT is the identity.
    prof_begin(ctx, "envelope_iq_kernel");
    envelope_iq_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(
        reinterpret_cast<const float2*>(frame), env, n);
    prof_end(ctx);
    USX_CHECK_LAUNCH("envelope_iq_kernel");
    return USX_OK;
  }
  // Twiddle tables with the reference's recurrence (postprocess.cpp:22-33).
  std::vector<float2> tw(2 * static_cast<size_t>(n_fft - 1));
  for (int pass = 0; pass < 2; ++pass) {
    const bool inverse = pass == 1;
    float2* t = tw.data() + (inverse ? n_fft - 1 : 0);
    for (int len = 2; len <= n_fft; len <<= 1) {
      const float ang = 2.0f * kPi / static_cast<float>(len) * (inverse ? 1.0f : -1.0f);
      const float wr = std::cos(ang), wi = std::sin(ang);
      float cr = 1.0f, ci = 0.0f;
      for (int k = 0; k < len / 2; ++k) {
        t[len / 2 - 1 + k] = make_float2(cr, ci);
        const float nr = cr * wr - ci * wi, ni = cr * wi + ci * wr;
        cr = nr;
        ci = ni;
      }
    }
  }
  void* ws = nullptr;
  if (int rc = scratch(ctx, tw.size() * sizeof(float2), &ws)) return rc;
  USX_CUDA(cudaMemcpyAsync(ws, tw.data(), tw.size() * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
  const size_t smem = sizeof(float2) * n_fft;
  if (smem > 48 * 1024)
    if (int rc_ = smem_limit(reinterpret_cast<const void*>(hilbert_kernel), static_cast<size_t>(static_cast<int>(smem)))) return rc_;
  prof_begin(ctx, "hilbert_kernel");
  hilbert_kernel<<<n0, 256, smem, ctx->stream>>>(reinterpret_cast<const float2*>(frame), n1, n_fft,
                                                 log2n, static_cast<const float2*>(ws), env);
  prof_end(ctx);
  USX_CHECK_LAUNCH("hilbert_kernel");
  // The host table must outlive the asynchronous copy.
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  return USX_OK;
}

int usx_cu_apply_tgc(usx_ctx* ctx, const float* env, int n0, int n1, const float* points,
                     float attenuation_db_cm_mhz, float center_frequency_hz, float* out) {
  if (!ctx || !env || !points || !out) return fail(USX_ERR_INVALID, "usx_cu_apply_tgc: null argument");
  const long n = static_cast<long>(n0) * n1;
  if (n <= 0) return USX_OK;
  prof_begin(ctx, "tgc_kernel");
  tgc_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(env, points, attenuation_db_cm_mhz,
                                                        center_frequency_hz * 1e-6f, n, out);
  prof_end(ctx);
  USX_CHECK_LAUNCH("tgc_kernel");
  return USX_OK;
}

int usx_cu_log_compress(usx_ctx* ctx, const float* env, int64_t n, float dynamic_range_db,
                        float gain_db, float reference, float* out) {
  if (!ctx || !env || !out) return fail(USX_ERR_INVALID, "usx_cu_log_compress: null argument");
  if (n <= 0) return USX_OK;
  unsigned* ref_bits = reinterpret_cast<unsigned*>(ctx->d_status + 8);
  if (reference <= 0.0f) {
    USX_CUDA(cudaMemsetAsync(ref_bits, 0, sizeof(unsigned), ctx->stream));
    const int blocks = std::max(1, std::min(ceil_div(n, 256), ctx->sm_count * 8));
    prof_begin(ctx, "max_kernel");
    max_kernel<<<blocks, 256, 0, ctx->stream>>>(env, n, ref_bits);
    prof_end(ctx);
    USX_CHECK_LAUNCH("max_kernel");
  }
  prof_begin(ctx, "log_compress_kernel");
  log_compress_kernel<<<ceil_div(n, 256), 256, 0, ctx->stream>>>(env, n, dynamic_range_db, gain_db,
                                                                 reference, ref_bits, out);
  prof_end(ctx);
  USX_CHECK_LAUNCH("log_compress_kernel");
  return USX_OK;
}

int usx_cu_max(usx_ctx* ctx, const float* x, int64_t n, float* out_host) {
  if (!ctx || !x || !out_host) return fail(USX_ERR_INVALID, "usx_cu_max: null argument");
  unsigned* bits = reinterpret_cast<unsigned*>(ctx->d_status + 9);
  USX_CUDA(cudaMemsetAsync(bits, 0, sizeof(unsigned), ctx->stream));
  if (n > 0) {
    const int blocks = std::max(1, std::min(ceil_div(n, 256), ctx->sm_count * 8));
    max_kernel<<<blocks, 256, 0, ctx->stream>>>(x, n, bits);
    USX_CHECK_LAUNCH("max_kernel");
  }
  unsigned h = 0;
  USX_CUDA(cudaMemcpyAsync(&h, bits, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  USX_CUDA(cudaStreamSynchronize(ctx->stream));
  float f;
  std::memcpy(&f, &h, sizeof(f));
  *out_host = f;
  return USX_OK;
}

int usx_cu_scan_convert(usx_ctx* ctx, const float* image, const usx_grid_desc* grid,
                        const float* points_host, int width, int height, float fill,
                        float* pixels, float* extent) {
  if (!ctx || !image || !grid || !points_host || !pixels)
    return fail(USX_ERR_INVALID, "usx_cu_scan_convert: null argument");
  if (width <= 0 || height <= 0) return fail(USX_ERR_INVALID, "usx_cu_scan_convert: empty raster");
  const int n0 = grid->n_axis0, n1 = grid->n_axis1;
  if (n0 <= 0 || n1 <= 0 || !grid->axis0 || !grid->axis1)
    return fail(USX_ERR_INVALID, "usx_cu_scan_convert: invalid grid");
  ScanArgs s;
  // The extent of the sample points (postprocess.cpp:126-132). The points are
  // scanned as four contiguous quarters side by side (independent dependency
  // chains; the tail joins the last quarter), then the quarters' extents are
  // combined in order: with std::min/max keeping the earlier of equal values,
  // that returns the same value (down to the sign of a zero) as one
  // sequential pass.
  const long n = static_cast<long>(n0) * n1;
  const long q = n / 4;
  Extent e0, e1, e2, e3;
  for (long k = 0; k < q; ++k) {
    e0.add(points_host + 3 * k);
    e1.add(points_host + 3 * (q + k));
    e2.add(points_host + 3 * (2 * q + k));
    e3.add(points_host + 3 * (3 * q + k));
  }
  for (long k = 4 * q; k < n; ++k) e3.add(points_host + 3 * k);
  e0.merge(e1);
  e0.merge(e2);
  e0.merge(e3);
  const float x_min = e0.x_min, x_max = e0.x_max, z_min = e0.z_min, z_max = e0.z_max;
  s.image = image;
  s.pixels = pixels;
  s.n0 = n0;
  s.n1 = n1;
  s.width = width;
  s.height = height;
  s.cart = grid->type == USX_GRID_CARTESIAN;
  s.x_min = x_min;
  s.x_max = x_max;
  s.z_min = z_min;
  s.z_max = z_max;
  s.a0_first = grid->axis0[0];
  s.a0_last = grid->axis0[n0 - 1];
  s.a1_first = grid->axis1[0];
  s.a1_last = grid->axis1[n1 - 1];
  s.apex_x = grid->apex[0];
  s.apex_z = grid->apex[2];
  s.fill = fill;
  if (extent) {
    extent[0] = x_min;
    extent[1] = x_max;
    extent[2] = z_min;
    extent[3] = z_max;
  }
  const dim3 tiles(ceil_div(width, kScanTile), ceil_div(height, kScanTile));
  prof_begin(ctx, "scan_convert_kernel");
  scan_convert_kernel<<<tiles, 256, 0, ctx->stream>>>(s);
  prof_end(ctx);
  USX_CHECK_LAUNCH("scan_convert_kernel");
  return USX_OK;
}

}  // extern "C"
