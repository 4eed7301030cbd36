// gemm_tc5.cu — the network's inference GEMMs on the fifth-generation tensor
// cores: C[M x N] = act(A[M x K] W[K x N] + b), BF16 operands, FP32
// accumulation in tensor memory (TMEM), for N = 128 or 256 and K a multiple
// of 64 (the learned-MV network: K = 256).
//
// One CTA of four warps per SM, persistent over 128-row tiles of A:
//   * the weights W^T ([N][K], K contiguous) are copied into shared memory
//     once per CTA, the A tile (128 x K) once per tile, both with cp.async in
//     the 128-byte-swizzled K-major layout the tensor core reads (rows of 64
//     BF16 = 128 bytes, the 16-byte chunk j of row r stored at chunk j ^ (r & 7),
//     1024-byte atoms of 8 rows);
//   * one thread issues K / 16 tcgen05.mma (M = 128, N, K = 16 each) into a
//     TMEM accumulator of N columns and commits them to an mbarrier;
//   * every warp reads its 32 TMEM lanes (rows) back with tcgen05.ld, adds the
//     bias, applies the ReLU and stores BF16 (hidden layers) or FP32 (output).
// All waits are bounded: on a timeout the kernel records it in the context's
// status word, skips the tile and still releases its TMEM.
#include <cuda_bf16.h>

#include <algorithm>

#include "tc5.cuh"
#include "usx_internal.cuh"

namespace usxcu {
namespace {

constexpr int kTcM = 128;          // rows per tile (one MMA's M)
constexpr int kTcThreads = 128;    // four warps: TMEM lanes 0..127
constexpr int kAtomK = 64;         // BF16 per 128-byte swizzled row

struct Tc5Args {
  const __nv_bfloat16* A;   // [M][K]
  const __nv_bfloat16* Bt;  // [N][K]
  const float* bias;        // [N]
  __nv_bfloat16* C16;       // [M][N] or null
  float* C32;               // [M][N] or null
  int M, K, relu;
  int* status;
};

__device__ __forceinline__ void cp16(void* smem, const void* g) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(su32(smem)), "l"(g));
}

// Copy rows [0, rows) x K of a K-contiguous BF16 matrix into the swizzled
// layout: K / 64 blocks of rows x 128 bytes.
__device__ __forceinline__ void load_swizzled(char* dst, const __nv_bfloat16* src, int rows, int K, long ld) {
  const int chunks_per_row = K / 8;        // 16-byte chunks
  const int total = rows * chunks_per_row;
  for (int c = threadIdx.x; c < total; c += kTcThreads) {
    const int r = c / chunks_per_row, q = c - r * chunks_per_row;
    const int blk = q >> 3, j = q & 7;      // K block of 64, chunk in the 128-byte row
    char* d = dst + static_cast<long>(blk) * rows * 128 + r * 128 + ((j ^ (r & 7)) << 4);
    cp16(d, src + r * ld + q * 8);
  }
  asm volatile("cp.async.commit_group;\n" ::);
}

template <int N>
__global__ void __launch_bounds__(kTcThreads, 1) gemm_tc5_kernel(const Tc5Args g) {
  extern __shared__ __align__(1024) char tc5_raw[];
  // 1024-byte alignment of the operand blocks (the swizzle atom).
  char* base = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(tc5_raw) + 1023) & ~uintptr_t(1023));
  char* sB = base;                                            // N x K
  char* sA = base + static_cast<long>(N) * g.K * 2;           // 128 x K
  uint64_t* bar = reinterpret_cast<uint64_t*>(sA + static_cast<long>(kTcM) * g.K * 2);
  unsigned* tmem_slot = reinterpret_cast<unsigned*>(bar + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(su32(tmem_slot)),
                 "r"(N));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::);
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(su32(bar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  load_swizzled(sB, g.Bt, N, g.K, g.K);
  const int n_tiles = g.M / kTcM;
  int tile = blockIdx.x;
  if (tile < n_tiles) load_swizzled(sA, g.A + static_cast<long>(tile) * kTcM * g.K, kTcM, g.K, g.K);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const unsigned tmem = *tmem_slot;
  const uint32_t idesc = instr_desc(kTcM, N);
  unsigned phase = 0;

  for (; tile < n_tiles; tile += gridDim.x) {
    const long m0 = static_cast<long>(tile) * kTcM;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    // Make this thread's shared-memory writes visible to the tensor core.
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const unsigned a0 = su32(sA), b0 = su32(sB);
      int step = 0;
      for (int kb = 0; kb < g.K / kAtomK; ++kb) {
        for (int j = 0; j < kAtomK / 16; ++j, ++step) {
          const uint64_t ad = smem_desc(a0 + kb * kTcM * 128 + j * 32);
          const uint64_t bd = smem_desc(b0 + kb * N * 128 + j * 32);
          const unsigned acc = step > 0 ? 1u : 0u;
          asm volatile(
              "{\n .reg .pred p;\n setp.ne.u32 p, %4, 0;\n"
              " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
              "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
        }
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(su32(bar))
                   : "memory");
    }
    const bool ok = mbar_wait(su32(bar), phase);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0 && g.status) atomicExch(g.status, 1);
      break;
    }
    phase ^= 1u;
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    // The MMAs have read the A tile: fetch the next one behind the epilogue.
    const int next = tile + static_cast<int>(gridDim.x);
    if (next < n_tiles) load_swizzled(sA, g.A + static_cast<long>(next) * kTcM * g.K, kTcM, g.K, g.K);
    // Epilogue: warp w owns TMEM lanes (rows) 32 w .. 32 w + 31.
    const long row = m0 + warp * 32 + lane;
    const unsigned lane_base = tmem + (static_cast<unsigned>(warp * 32) << 16);
#pragma unroll 1
    for (int c0 = 0; c0 < N; c0 += 32) {
      uint32_t r[32];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
          "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
            "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]),
            "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
            "=r"(r[30]), "=r"(r[31])
          : "r"(lane_base + c0));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      float v[32];
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        float x = __uint_as_float(r[i]) + (g.bias ? __ldg(g.bias + c0 + i) : 0.0f);
        if (g.relu) x = fmaxf(x, 0.0f);
        v[i] = x;
      }
      if (row < g.M) {
        if (g.C32) {
          float4* dst = reinterpret_cast<float4*>(g.C32 + row * N + c0);
#pragma unroll
          for (int i = 0; i < 8; ++i) dst[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        }
        if (g.C16) {
          uint4* dst = reinterpret_cast<uint4*>(g.C16 + row * N + c0);
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            __nv_bfloat162 h0 = __floats2bfloat162_rn(v[8 * i], v[8 * i + 1]);
            __nv_bfloat162 h1 = __floats2bfloat162_rn(v[8 * i + 2], v[8 * i + 3]);
            __nv_bfloat162 h2 = __floats2bfloat162_rn(v[8 * i + 4], v[8 * i + 5]);
            __nv_bfloat162 h3 = __floats2bfloat162_rn(v[8 * i + 6], v[8 * i + 7]);
            dst[i] = make_uint4(*reinterpret_cast<uint32_t*>(&h0), *reinterpret_cast<uint32_t*>(&h1),
                                *reinterpret_cast<uint32_t*>(&h2), *reinterpret_cast<uint32_t*>(&h3));
          }
        }
      }
    }
    // The accumulator is reused by the next tile.
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(N));
}

__global__ void transpose_bf16_kernel(const __nv_bfloat16* w, int K, int N, __nv_bfloat16* wt) {
  const long i = blockIdx.x * static_cast<long>(blockDim.x) + threadIdx.x;
  if (i >= static_cast<long>(K) * N) return;
  const int k = static_cast<int>(i / N), n = static_cast<int>(i - static_cast<long>(k) * N);
  wt[static_cast<long>(n) * K + k] = w[i];
}

}  // namespace

size_t gemm_tc5_smem(int N, int K) { return static_cast<size_t>(N + kTcM) * K * 2 + 1024 + 64; }

bool gemm_tc5_supported(int M, int N, int K) {
  return (N == 128 || N == 256) && K % kAtomK == 0 && K >= kAtomK && M % kTcM == 0 &&
         gemm_tc5_smem(N, K) <= 227 * 1024;
}

int transpose_bf16(cudaStream_t st, const void* w, int K, int N, void* wt) {
  const long n = static_cast<long>(K) * N;
  transpose_bf16_kernel<<<static_cast<unsigned>(ceil_div(n, 256)), 256, 0, st>>>(
      static_cast<const __nv_bfloat16*>(w), K, N, static_cast<__nv_bfloat16*>(wt));
  USX_CHECK_LAUNCH("transpose_bf16_kernel");
  return USX_OK;
}

int launch_gemm_tc5(usx_ctx* ctx, const void* A, const void* Bt, const float* bias, bool relu, void* C16, float* C32,
                    int M, int N, int K) {
  if (!gemm_tc5_supported(M, N, K)) return fail(USX_ERR_UNSUPPORTED, "gemm_tc5: unsupported shape");
  Tc5Args g;
  g.A = static_cast<const __nv_bfloat16*>(A);
  g.Bt = static_cast<const __nv_bfloat16*>(Bt);
  g.bias = bias;
  g.C16 = static_cast<__nv_bfloat16*>(C16);
  g.C32 = C32;
  g.M = M;
  g.K = K;
  g.relu = relu ? 1 : 0;
  g.status = ctx->d_status + 13;
  const size_t smem = gemm_tc5_smem(N, K);
  const int tiles = M / kTcM;
  const unsigned grid = static_cast<unsigned>(std::max(1, std::min(tiles, ctx->sm_count)));
  if (N == 256) {
    if (int rc = smem_limit(reinterpret_cast<const void*>(gemm_tc5_kernel<256>), smem)) return rc;
    gemm_tc5_kernel<256><<<grid, kTcThreads, smem, ctx->stream>>>(g);
  } else {
    if (int rc = smem_limit(reinterpret_cast<const void*>(gemm_tc5_kernel<128>), smem)) return rc;
    gemm_tc5_kernel<128><<<grid, kTcThreads, smem, ctx->stream>>>(g);
  }
  USX_CHECK_LAUNCH("gemm_tc5_kernel");
  return USX_OK;
}

}  // namespace usxcu
