// shl_mlp.cu -- the warm-start surrogate: a multilayer perceptron trained and
// evaluated on the GPU with this file's own kernels (no counterpart in the
// reference, which always starts from the undeformed state).
//
// Network: x (n_in) -> [Linear -> GELU] x n_hidden -> Linear -> y (n_out).
// Weights are kept as FP32 master copies and as BF16 copies W (out x in) and
// W^T (in x out) for the tensor-core GEMMs; every GEMM multiplies BF16
// operands with FP32 accumulation.  One GEMM form serves all three products
// of a layer, C[M,N] = A[M,K] . B[N,K]^T with both operands K-contiguous:
//   forward        Z  = H_prev . W^T        (A = H_prev,  B = W)
//   input grad     dH = dZ . W              (A = dZ,      B = W^T)
//   weight grad    dW = dZ^T . H_prev       (A = dZ^T,    B = H_prev^T)
// The GEMM (k_gemm_tc) runs on the tcgen05 tensor cores: a persistent,
// warp-specialised kernel with TMA loads into a four-stage shared-memory ring,
// tcgen05.mma into two tensor-memory accumulators and a tcgen05.ld epilogue
// that overlaps the next tile's products.  Split-K writes
// FP32 partials that one fixed-order kernel sums, so every result is
// deterministic.
//
// GELU is the erf form 0.5 x (1 + erf(x / sqrt 2)); the loss is the mean
// squared error over the real (unpadded) outputs; the optimiser is Adam with
// bias correction.  Feature dimensions are padded to multiples of 32 and the
// batch to a multiple of 128; padded weights, inputs and targets are zero.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <random>
#include <string>
#include <vector>

#include "../../include/shl.h"
#include "shl_setup.h"

namespace {

// ---- the BF16 GEMM on the fifth-generation tensor cores ----
// C[M,N] = A[M,K] . B[N,K]^T, both operands K-contiguous, 128 x 256 output
// tiles.  A persistent grid (one CTA per SM) takes the tiles in turn; each CTA
// has six warps with fixed roles:
//   warp 0     one thread streams 128 x 64 tiles of A and 256 x 64 tiles of B
//              into a four-stage shared-memory ring with TMA (128-byte swizzle,
//              zero fill past the matrix edges);
//   warp 1     owns the tensor memory (two 256-column FP32 accumulators) and one
//              thread issues tcgen05.mma (M 128, N 256, K 16; BF16 operands read
//              from shared memory through matrix descriptors), releasing each
//              stage with tcgen05.commit and signalling a finished accumulator;
//   warps 2-5  the epilogue: each reads its 32 accumulator lanes (rows) with
//              tcgen05.ld, adds the bias (and GELU), stores, and hands the
//              accumulator back, so the next tile's products overlap it.
// Every wait on an mbarrier is bounded in time: on expiry the kernel records an
// error, stops its loops, waits (bounded) for its copies and products in flight,
// frees its tensor memory and returns.
constexpr int kBM = 128, kBN = 256, kBK = 64;  // kBK bf16 = 128 bytes: one swizzle row
constexpr int kStages = 4;
constexpr int kGemmThreads = 192;
constexpr int kTileA = kBM * kBK * 2;          // 16 KB
constexpr int kTileB = kBN * kBK * 2;          // 32 KB
constexpr int kStageBytes = kTileA + kTileB;
constexpr int kGemmSmem = kStages * kStageBytes + 1024;
constexpr uint32_t kTmemCols = 512;            // two FP32 accumulators of 128 lanes x 256 columns
constexpr uint64_t kWaitNs = 2000000000ull;    // a wait gives up after 2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ bool mbar_test(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// wait for the phase of the given parity to complete; false after kWaitNs or
// once *abort is set by another thread of the CTA
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile int* abort) {
  const uint64_t t0 = globaltimer();
  for (uint32_t it = 0;; ++it) {
    if (mbar_test(bar, parity)) return true;
    if ((it & 63u) == 63u && (*abort || globaltimer() - t0 > kWaitNs)) return false;
  }
}

// bounded wait that ignores the abort flag (the drain after an abort)
__device__ __forceinline__ void mbar_drain(uint32_t bar, uint32_t parity) {
  const uint64_t t0 = globaltimer();
  while (!mbar_test(bar, parity) && globaltimer() - t0 < kWaitNs) {
  }
}

__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// 2-D tiled TMA load of the box at (x = K element, y = row) into shared memory
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int x, int y, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
      ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// shared-memory matrix descriptor of a K-major operand tile written by TMA with
// the 128-byte swizzle: rows of 128 bytes, 8-row groups 1024 bytes apart
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
  uint64_t d = (uint64_t)((addr >> 4) & 0x3FFFu);  // start address
  d |= (uint64_t)1 << 16;                          // leading byte offset (not used by swizzled K-major)
  d |= (uint64_t)(1024 >> 4) << 32;                // stride byte offset between 8-row groups
  d |= (uint64_t)1 << 46;                          // descriptor version of sm_100
  d |= (uint64_t)2 << 61;                          // 128-byte swizzle
  return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M 128, N 256
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kBN >> 3) << 17) |
                            ((uint32_t)(kBM >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 16 consecutive FP32 columns of this thread's accumulator lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

// epilogue modes
enum { EPI_PARTIAL = 0, EPI_BIAS = 1, EPI_BIAS_GELU = 2 };

struct GemmArgs {
  int M, N, K;
  int kb_per_split;        // K blocks (kBK wide) per split-K slice
  int gx, gy, splits;      // tiles along N, along M, K slices
  int mode;
  const float* bias;       // N (EPI_BIAS*)
  float* C;                // M x N fp32 (ldc) ; EPI_PARTIAL: split z writes C + z*M*ldc
  int ldc;
  __nv_bfloat16* Cb;       // optional bf16 copy of the activation (ldc)
  int* error;              // set to 1 when a wait gave up
};

// tile t of the persistent schedule: N block fastest, then M block, then K slice
struct TileCoord {
  int m0, n0, kb0, nkb, z;
};
__device__ __forceinline__ TileCoord tile_coord(const GemmArgs& g, int t) {
  TileCoord c;
  const int per_z = g.gx * g.gy;
  c.z = t / per_z;
  const int r = t - c.z * per_z;
  c.m0 = (r / g.gx) * kBM;
  c.n0 = (r % g.gx) * kBN;
  const int kb_total = (g.K + kBK - 1) / kBK;
  c.kb0 = c.z * g.kb_per_split;
  c.nkb = max(0, min(g.kb_per_split, kb_total - c.kb0));
  return c;
}

__global__ void __launch_bounds__(kGemmThreads, 1)
    k_gemm_tc(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, GemmArgs g) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages], tfull_bar[2], tempty_bar[2], done_bar;
  __shared__ uint32_t tmem_base;
  __shared__ int abort_flag;
  __shared__ int loads_issued;  // stage loads issued by the producer (for the drain after an abort)
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;  // swizzled tiles start on 1024 bytes
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n_tiles = g.gx * g.gy * g.splits;
  volatile int* abort = &abort_flag;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&tfull_bar[b]), 1);
      mbar_init(smem_u32(&tempty_bar[b]), 4);  // one arrival per epilogue warp
    }
    mbar_init(smem_u32(&done_bar), 1);
    abort_flag = 0;
    loads_issued = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int it = 0;
      for (int t = blockIdx.x; t < n_tiles && !*abort; t += gridDim.x) {
        const TileCoord c = tile_coord(g, t);
        for (int kb = 0; kb < c.nkb; ++kb, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)(it / kStages) & 1u;
          if (!mbar_wait(smem_u32(&empty_bar[s]), ph ^ 1u, abort)) {
            *abort = 1;
            break;
          }
          const uint32_t fb = smem_u32(&full_bar[s]);
          mbar_expect_tx(fb, kStageBytes);
          const int kx = (c.kb0 + kb) * kBK;
          tma_load_2d(base + (uint32_t)s * kStageBytes, &map_a, kx, c.m0, fb);
          tma_load_2d(base + (uint32_t)s * kStageBytes + kTileA, &map_b, kx, c.n0, fb);
          loads_issued = it + 1;
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      int it = 0, tl = 0;
      for (int t = blockIdx.x; t < n_tiles && !*abort; t += gridDim.x, ++tl) {
        const TileCoord c = tile_coord(g, t);
        const int acc = tl & 1;
        const uint32_t aph = (uint32_t)(tl >> 1) & 1u;
        if (!mbar_wait(smem_u32(&tempty_bar[acc]), aph ^ 1u, abort)) {
          *abort = 1;
          break;
        }
        tc_fence_after();
        const uint32_t d = tmem + (uint32_t)(acc * kBN);
        bool ok = true;
        for (int kb = 0; kb < c.nkb; ++kb, ++it) {
          const int s = it % kStages;
          const uint32_t ph = (uint32_t)(it / kStages) & 1u;
          if (!mbar_wait(smem_u32(&full_bar[s]), ph, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t a_addr = base + (uint32_t)s * kStageBytes, b_addr = a_addr + kTileA;
#pragma unroll
          for (int k = 0; k < kBK / 16; ++k)  // K 16 per product: 32 bytes further along the swizzled rows
            tc_mma(d, smem_desc_sw128(a_addr + 32u * k), smem_desc_sw128(b_addr + 32u * k),
                   (kb | k) != 0 ? 1u : 0u);
          tc_commit(smem_u32(&empty_bar[s]));
        }
        if (!ok) {
          *abort = 1;
          break;
        }
        if (c.nkb > 0)
          tc_commit(smem_u32(&tfull_bar[acc]));  // arrives once the tile's products are complete
        else
          mbar_arrive(smem_u32(&tfull_bar[acc]));  // an empty K range: the epilogue writes zeros
      }
      tc_commit(smem_u32(&done_bar));  // every product this thread issued has completed
    }
  } else {  // epilogue warps 2-5: accumulator lanes 32 (warp % 4) .. + 31
    const int q = warp & 3;
    int tl = 0;
    for (int t = blockIdx.x; t < n_tiles && !*abort; t += gridDim.x, ++tl) {
      const TileCoord c = tile_coord(g, t);
      const int acc = tl & 1;
      const uint32_t aph = (uint32_t)(tl >> 1) & 1u;
      if (!mbar_wait(smem_u32(&tfull_bar[acc]), aph, abort)) {
        *abort = 1;
        break;
      }
      tc_fence_after();
      const int row = c.m0 + q * 32 + lane;
      float* C = g.C + (g.mode == EPI_PARTIAL ? (size_t)c.z * g.M * g.ldc : 0);
      const bool vec = (g.ldc & 3) == 0;
#pragma unroll 1
      for (int col0 = 0; col0 < kBN; col0 += 16) {
        if (c.n0 + col0 >= g.N) break;  // warp-uniform
        float v[16];
        if (c.nkb > 0) {
          tc_ld16(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(acc * kBN + col0), v);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = 0.f;
        }
        if (row >= g.M) continue;
        const int cb = c.n0 + col0;
        if (g.mode != EPI_PARTIAL) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cb + i < g.N) v[i] += g.bias[cb + i];
        }
        const size_t o = (size_t)row * g.ldc + cb;
        if (vec && cb + 16 <= g.N) {
#pragma unroll
          for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(C + o + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        } else {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cb + i < g.N) C[o + i] = v[i];
        }
        if (g.Cb) {
#pragma unroll
          for (int i = 0; i < 16; ++i)
            if (cb + i < g.N) g.Cb[o + i] = __float2bfloat16_rn(g.mode == EPI_BIAS_GELU ? gelu(v[i]) : v[i]);
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(smem_u32(&tempty_bar[acc]));
    }
  }
  __syncwarp();
  if (threadIdx.x == 32) mbar_drain(smem_u32(&done_bar), 0u);  // no product in flight past this point
  tc_fence_before();
  __syncthreads();
  if (*abort && threadIdx.x == 0) {
    atomicExch(g.error, 1);
    // every load issued lands before the CTA's shared memory is released
    const int n = loads_issued;
    for (int it = max(0, n - kStages); it < n; ++it)
      mbar_drain(smem_u32(&full_bar[it % kStages]), (uint32_t)(it / kStages) & 1u);
  }
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

// pseudo-random bf16 values in [-1, 1) (hash of the index), operands of the GEMM timing
__global__ void k_fill_bf16(__nv_bfloat16* p, size_t n, uint32_t seed) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    uint32_t h = (uint32_t)i * 2654435761u ^ seed;
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    p[i] = __float2bfloat16_rn((float)(h >> 8) * (2.0f / 16777216.0f) - 1.0f);
  }
}

// out[m, n] = sum over splits of part[s, m, n] (fixed order), optional bf16 copy
__global__ void k_splitk_reduce(const float* part, int splits, size_t mn, float* out, __nv_bfloat16* outb) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < mn; i += (size_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int z = 0; z < splits; ++z) s += part[(size_t)z * mn + i];
    if (out) out[i] = s;
    if (outb) outb[i] = __float2bfloat16_rn(s);
  }
}

// rows of the dataset into a padded bf16 input batch and an fp32 target batch
__global__ void k_gather_batch(const float* X, const float* T, const uint32_t* idx, int n, int in_real, int in_pad,
                               int out_real, int out_pad, int batch_pad, __nv_bfloat16* Xb, float* Tb) {
  const int r = blockIdx.x;
  if (r >= batch_pad) return;
  const bool real = r < n;
  const size_t src = real ? idx[r] : 0;
  for (int c = threadIdx.x; c < in_pad; c += blockDim.x)
    Xb[(size_t)r * in_pad + c] = __float2bfloat16_rn(real && c < in_real ? X[src * in_real + c] : 0.f);
  if (Tb)
    for (int c = threadIdx.x; c < out_pad; c += blockDim.x)
      Tb[(size_t)r * out_pad + c] = real && c < out_real ? T[src * out_real + c] : 0.f;
}

// loss = mean over the n x out_real block of (y - t)^2; dY = 2 (y - t) / (n out_real) as bf16;
// per-block partial sums of the squared error
__global__ void k_mse(const float* Y, const float* Tb, int n, int out_real, int out_pad, int batch_pad,
                      __nv_bfloat16* dY, double* partial) {
  __shared__ double sh[32];
  const size_t total = (size_t)batch_pad * out_pad;
  const float scale = 2.0f / ((float)n * (float)out_real);
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / out_pad), c = (int)(i % out_pad);
    float d = 0.f;
    if (r < n && c < out_real) d = Y[i] - Tb[i];
    s += (double)d * d;
    dY[i] = __float2bfloat16_rn(scale * d);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
  }
}

// dZ = dH * gelu'(Z), padded rows and columns forced to zero; bf16 out
__global__ void k_gelu_back(const float* dH, const float* Z, size_t mn, int cols, int n_rows, int real_cols,
                            __nv_bfloat16* dZ) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < mn; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const float v = (r < n_rows && c < real_cols) ? dH[i] * gelu_grad(Z[i]) : 0.f;
    dZ[i] = __float2bfloat16_rn(v);
  }
}

// out (cols x rows) = in (rows x cols)^T, bf16, 32x32 tiles
__global__ void k_transpose(const __nv_bfloat16* in, int rows, int cols, __nv_bfloat16* out) {
  __shared__ __nv_bfloat16 t[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int r = by + j, c = bx + threadIdx.x;
    t[j][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * cols + c] : __float2bfloat16_rn(0.f);
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const int c = bx + j, r = by + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * rows + r] = t[threadIdx.x][j];
  }
}

// db[n] = sum over the batch rows of dZ[r, n] (fixed order)
__global__ void k_bias_grad(const __nv_bfloat16* dZ, int rows, int cols, float* db) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (int r = 0; r < rows; ++r) s += __bfloat162float(dZ[(size_t)r * cols + c]);
  db[c] = s;
}

struct AdamArgs {
  float lr, b1, b2, eps, c1, c2;  // c1 = 1/(1-b1^t), c2 = 1/(1-b2^t)
};

// Adam on the real (unpadded) block; refreshes W (out x in), W^T (in x out) bf16 copies
__global__ void k_adam_w(float* W, float* m, float* v, const float* g, int out_real, int in_real, int out_pad,
                         int in_pad, AdamArgs a, __nv_bfloat16* Wb, __nv_bfloat16* WTb) {
  const size_t total = (size_t)out_pad * in_pad;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int r = (int)(i / in_pad), c = (int)(i % in_pad);
    if (r < out_real && c < in_real) {
      const float gi = g[i];
      const float mi = a.b1 * m[i] + (1.f - a.b1) * gi;
      const float vi = a.b2 * v[i] + (1.f - a.b2) * gi * gi;
      m[i] = mi;
      v[i] = vi;
      W[i] -= a.lr * (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
    }
    const __nv_bfloat16 wb = __float2bfloat16_rn(W[i]);
    Wb[i] = wb;
    WTb[(size_t)c * out_pad + r] = wb;
  }
}

__global__ void k_adam_b(float* b, float* m, float* v, const float* g, int n_real, AdamArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_real) return;
  const float mi = a.b1 * m[i] + (1.f - a.b1) * g[i];
  const float vi = a.b2 * v[i] + (1.f - a.b2) * g[i] * g[i];
  m[i] = mi;
  v[i] = vi;
  b[i] -= a.lr * (mi * a.c1) / (sqrtf(vi * a.c2) + a.eps);
}

int pad_to(int x, int m) { return (x + m - 1) / m * m; }

}  // namespace

struct shl_mlp {
  int n_layers = 0;                  // linear layers
  std::vector<int> dim, pad;         // real and padded widths, n_layers + 1
  int max_batch = 0, batch_pad = 0;  // rows
  cudaStream_t stream = nullptr;
  std::vector<void*> allocs;
  // per layer (out x in)
  std::vector<float*> W, b, mW, vW, mb, vb, gW, gb;
  std::vector<__nv_bfloat16*> Wb, WTb;
  // activations per layer boundary (batch_pad x pad[l])
  std::vector<float*> Z;             // pre-activation of layer l output (l = 1..n)
  std::vector<__nv_bfloat16*> H;     // bf16 activation (H[0] = input)
  std::vector<__nv_bfloat16*> HT;    // transposes for the weight-gradient GEMM
  float* dH = nullptr;               // fp32 input grad scratch (max width)
  __nv_bfloat16* dZ = nullptr;       // bf16 grads (max width)
  __nv_bfloat16* dZT = nullptr;
  float* part = nullptr;             // split-K partials
  int* gemm_err = nullptr;           // set by a GEMM whose wait gave up
  size_t part_elems = 0;
  float* Tb = nullptr;
  double* loss_part = nullptr;
  uint32_t* idx = nullptr;
  float* dX = nullptr;               // dataset inputs (n x in_real)
  float* dT = nullptr;               // dataset targets (n x out_real)
  size_t n_data = 0;
  int step = 0;
};

namespace {

thread_local std::string g_mlp_err;

#define MLP_TRY(expr)                                                            \
  do {                                                                           \
    cudaError_t e_ = (expr);                                                     \
    if (e_ != cudaSuccess) {                                                     \
      shl::set_error(std::string(#expr) + ": " + cudaGetErrorString(e_));        \
      return e_ == cudaErrorMemoryAllocation ? SHL_ERR_OOM : SHL_ERR_CUDA;       \
    }                                                                            \
  } while (0)

template <class T>
shl_status mlp_alloc(shl_mlp* m, T** p, size_t n) {
  void* q = nullptr;
  MLP_TRY(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
  MLP_TRY(cudaMemsetAsync(q, 0, std::max<size_t>(n, 1) * sizeof(T), m->stream));
  m->allocs.push_back(q);
  *p = (T*)q;
  return SHL_OK;
}

#define MLP_CHECK(expr)                  \
  do {                                   \
    shl_status s_ = (expr);              \
    if (s_ != SHL_OK) return s_;         \
  } while (0)

// cuTensorMapEncodeTiled from the driver (no link-time dependency on libcuda)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

// TMA map of a K-contiguous BF16 operand (rows x K, row stride ld elements):
// 64 x box_rows boxes with the 128-byte swizzle, zeros past the edges
shl_status operand_map(CUtensorMap* map, const __nv_bfloat16* ptr, int rows, int K, int ld, int box_rows) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) {
    shl::set_error("cuTensorMapEncodeTiled is not available from the driver");
    return SHL_ERR_CUDA;
  }
  if ((reinterpret_cast<uintptr_t>(ptr) & 15u) || (ld * 2) % 16 || rows < 1 || K < 1) {
    shl::set_error("GEMM operand: 16-byte aligned base and row stride, non-empty extents");
    return SHL_ERR_ARG;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
  const cuuint32_t es[2] = {1, 1};
  const CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<__nv_bfloat16*>(ptr), dims, strides, box,
                         es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    shl::set_error("cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return SHL_ERR_CUDA;
  }
  return SHL_OK;
}

cudaError_t gemm_kernel_attributes() {
  static cudaError_t e = cudaFuncSetAttribute((const void*)k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              kGemmSmem);
  return e;
}

// C[M,N] = A[M,K] . B[N,K]^T with the chosen epilogue.  Products without an
// epilogue split K when the output tiles alone would leave SMs idle.
shl_status gemm(shl_mlp* m, const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K,
                int mode, const float* bias, float* C, __nv_bfloat16* Cb) {
  MLP_TRY(gemm_kernel_attributes());
  int dev = 0, sms = 0;
  MLP_TRY(cudaGetDevice(&dev));
  MLP_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  CUtensorMap ma, mb;
  MLP_CHECK(operand_map(&ma, A, M, K, lda, kBM));
  MLP_CHECK(operand_map(&mb, B, N, K, ldb, kBN));
  const int gx = (N + kBN - 1) / kBN, gy = (M + kBM - 1) / kBM;
  const int k_blocks = (K + kBK - 1) / kBK;
  int splits = 1;
  if (mode == EPI_PARTIAL)
    while (gx * gy * splits < sms && k_blocks / (splits * 2) >= 4 && (size_t)(splits * 2) * M * N <= m->part_elems)
      splits *= 2;
  const int per = (k_blocks + splits - 1) / splits;
  splits = std::max(1, (k_blocks + per - 1) / per);
  GemmArgs g{M, N, K, per, gx, gy, splits, mode, bias, C, N, Cb, m->gemm_err};
  if (splits > 1) {
    g.C = m->part;
    g.Cb = nullptr;
  }
  const int tiles = gx * gy * splits;
  k_gemm_tc<<<std::min(tiles, sms), kGemmThreads, kGemmSmem, m->stream>>>(ma, mb, g);
  if (splits > 1) k_splitk_reduce<<<592, 256, 0, m->stream>>>(m->part, splits, (size_t)M * N, C, Cb);
  return SHL_OK;
}

// SHL_ERR_TIMEOUT when a GEMM gave up waiting (the flag is cleared)
shl_status gemm_status(shl_mlp* m) {
  int e = 0;
  MLP_TRY(cudaMemcpyAsync(&e, m->gemm_err, sizeof(int), cudaMemcpyDeviceToHost, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  if (e) {
    MLP_TRY(cudaMemsetAsync(m->gemm_err, 0, sizeof(int), m->stream));
    shl::set_error("tensor-core GEMM: a pipeline wait gave up");
    return SHL_ERR_TIMEOUT;
  }
  return SHL_OK;
}

// forward pass of `rows` (padded) inputs already in H[0]
shl_status forward(shl_mlp* m) {
  const int R = m->batch_pad;
  for (int l = 0; l < m->n_layers; ++l) {
    const bool last = l == m->n_layers - 1;
    MLP_CHECK(gemm(m, m->H[l], m->pad[l], m->Wb[l], m->pad[l], R, m->pad[l + 1], m->pad[l], last ? EPI_BIAS : EPI_BIAS_GELU,
                   m->b[l], m->Z[l + 1], last ? nullptr : m->H[l + 1]));
  }
  return SHL_OK;
}

shl_status backward(shl_mlp* m, int n_rows) {
  const int R = m->batch_pad;
  // dZ of the output layer is in m->dZ (bf16, R x pad[n])
  for (int l = m->n_layers - 1; l >= 0; --l) {
    const int out = m->pad[l + 1], in = m->pad[l];
    // transposes for dW = dZ^T . H_l
    k_transpose<<<dim3((out + 31) / 32, (R + 31) / 32), dim3(32, 8), 0, m->stream>>>(m->dZ, R, out, m->dZT);
    k_transpose<<<dim3((in + 31) / 32, (R + 31) / 32), dim3(32, 8), 0, m->stream>>>(m->H[l], R, in, m->HT[l]);
    MLP_CHECK(gemm(m, m->dZT, R, m->HT[l], R, out, in, R, EPI_PARTIAL, nullptr, m->gW[l], nullptr));
    k_bias_grad<<<(out + 127) / 128, 128, 0, m->stream>>>(m->dZ, R, out, m->gb[l]);
    if (l == 0) break;
    // dH_l = dZ . W  (B operand W^T: in x out)
    MLP_CHECK(gemm(m, m->dZ, out, m->WTb[l], out, R, in, out, EPI_PARTIAL, nullptr, m->dH, nullptr));
    k_gelu_back<<<592, 256, 0, m->stream>>>(m->dH, m->Z[l], (size_t)R * in, in, n_rows, m->dim[l], m->dZ);
  }
  return SHL_OK;
}

shl_status load_batch(shl_mlp* m, const uint32_t* idx_host, int n) {
  MLP_TRY(cudaMemcpyAsync(m->idx, idx_host, n * sizeof(uint32_t), cudaMemcpyHostToDevice, m->stream));
  k_gather_batch<<<m->batch_pad, 256, 0, m->stream>>>(m->dX, m->dT, m->idx, n, m->dim[0], m->pad[0],
                                                      m->dim[m->n_layers], m->pad[m->n_layers], m->batch_pad,
                                                      m->H[0], m->Tb);
  return SHL_OK;
}

shl_status loss_and_grad(shl_mlp* m, int n, double* loss_out) {
  const int L = m->n_layers;
  k_mse<<<592, 256, 0, m->stream>>>(m->Z[L], m->Tb, n, m->dim[L], m->pad[L], m->batch_pad, m->dZ, m->loss_part);
  if (loss_out) {
    std::vector<double> p(592);
    MLP_TRY(cudaMemcpyAsync(p.data(), m->loss_part, 592 * sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    MLP_TRY(cudaStreamSynchronize(m->stream));
    double s = 0;
    for (double x : p) s += x;
    *loss_out = s / ((double)n * m->dim[L]);
  }
  return SHL_OK;
}

shl_status adam(shl_mlp* m, float lr) {
  ++m->step;
  AdamArgs a{lr, 0.9f, 0.999f, 1e-8f, 0.f, 0.f};
  a.c1 = 1.f / (1.f - std::pow(a.b1, (float)m->step));
  a.c2 = 1.f / (1.f - std::pow(a.b2, (float)m->step));
  for (int l = 0; l < m->n_layers; ++l) {
    k_adam_w<<<592, 256, 0, m->stream>>>(m->W[l], m->mW[l], m->vW[l], m->gW[l], m->dim[l + 1], m->dim[l],
                                          m->pad[l + 1], m->pad[l], a, m->Wb[l], m->WTb[l]);
    k_adam_b<<<(m->dim[l + 1] + 255) / 256, 256, 0, m->stream>>>(m->b[l], m->mb[l], m->vb[l], m->gb[l],
                                                                 m->dim[l + 1], a);
  }
  return SHL_OK;
}

// refresh bf16 copies after host-set weights
shl_status refresh_copies(shl_mlp* m) {
  for (int l = 0; l < m->n_layers; ++l) {
    AdamArgs a{0.f, 0.f, 0.f, 1.f, 0.f, 0.f};
    // lr = 0: the Adam kernel only rewrites the bf16 copies (m, v unchanged since g is not read for lr 0)
    k_adam_w<<<592, 256, 0, m->stream>>>(m->W[l], m->mW[l], m->vW[l], m->gW[l], 0, 0, m->pad[l + 1], m->pad[l], a,
                                          m->Wb[l], m->WTb[l]);
  }
  return SHL_OK;
}

}  // namespace

extern "C" {

shl_status shl_mlp_create(const uint32_t* dims, uint32_t n_dims, uint32_t max_batch, uint64_t seed, shl_mlp** out) {
  if (!dims || n_dims < 2 || !out || max_batch == 0) return SHL_ERR_ARG;
  shl_mlp* m = new shl_mlp();
  m->n_layers = (int)n_dims - 1;
  for (uint32_t i = 0; i < n_dims; ++i) {
    if (dims[i] == 0) {
      delete m;
      return SHL_ERR_ARG;
    }
    m->dim.push_back((int)dims[i]);
    m->pad.push_back(pad_to((int)dims[i], 32));
  }
  m->max_batch = (int)max_batch;
  m->batch_pad = pad_to((int)max_batch, kBM);
  cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete m;
    shl::set_error(std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    return SHL_ERR_CUDA;
  }
  auto fail = [&](shl_status s) {
    shl_mlp_destroy(m);
    return s;
  };
  const int L = m->n_layers, R = m->batch_pad;
  int maxw = 0;
  for (int w : m->pad) maxw = std::max(maxw, w);
  m->W.resize(L); m->b.resize(L); m->mW.resize(L); m->vW.resize(L); m->mb.resize(L); m->vb.resize(L);
  m->gW.resize(L); m->gb.resize(L); m->Wb.resize(L); m->WTb.resize(L);
  m->Z.assign(L + 1, nullptr); m->H.assign(L + 1, nullptr); m->HT.assign(L + 1, nullptr);
  std::mt19937_64 rng(seed);
  size_t max_wgrad = 0;
  for (int l = 0; l < L; ++l) {
    const size_t n = (size_t)m->pad[l + 1] * m->pad[l];
    max_wgrad = std::max(max_wgrad, n);
    shl_status s;
    if ((s = mlp_alloc(m, &m->W[l], n)) || (s = mlp_alloc(m, &m->mW[l], n)) || (s = mlp_alloc(m, &m->vW[l], n)) ||
        (s = mlp_alloc(m, &m->gW[l], n)) || (s = mlp_alloc(m, &m->Wb[l], n)) || (s = mlp_alloc(m, &m->WTb[l], n)) ||
        (s = mlp_alloc(m, &m->b[l], m->pad[l + 1])) || (s = mlp_alloc(m, &m->mb[l], m->pad[l + 1])) ||
        (s = mlp_alloc(m, &m->vb[l], m->pad[l + 1])) || (s = mlp_alloc(m, &m->gb[l], m->pad[l + 1])))
      return fail(s);
    // He-normal weights for the GELU layers, Glorot-normal for the output layer; zero bias
    const double sd = (l < L - 1) ? std::sqrt(2.0 / m->dim[l]) : std::sqrt(2.0 / (m->dim[l] + m->dim[l + 1]));
    std::normal_distribution<double> nd(0.0, sd);
    std::vector<float> w(n, 0.f);
    for (int r = 0; r < m->dim[l + 1]; ++r)
      for (int c = 0; c < m->dim[l]; ++c) w[(size_t)r * m->pad[l] + c] = (float)nd(rng);
    if (cudaMemcpyAsync(m->W[l], w.data(), n * sizeof(float), cudaMemcpyHostToDevice, m->stream) != cudaSuccess)
      return fail(SHL_ERR_CUDA);
  }
  for (int l = 0; l <= L; ++l) {
    shl_status s;
    if ((s = mlp_alloc(m, &m->H[l], (size_t)R * m->pad[l])) || (s = mlp_alloc(m, &m->HT[l], (size_t)R * m->pad[l])) ||
        (s = mlp_alloc(m, &m->Z[l], (size_t)R * m->pad[l])))
      return fail(s);
  }
  m->part_elems = std::max((size_t)R * maxw, max_wgrad) * 2;
  shl_status s;
  if ((s = mlp_alloc(m, &m->dH, (size_t)R * maxw)) || (s = mlp_alloc(m, &m->dZ, (size_t)R * maxw)) ||
      (s = mlp_alloc(m, &m->dZT, (size_t)R * maxw)) || (s = mlp_alloc(m, &m->part, m->part_elems)) ||
      (s = mlp_alloc(m, &m->Tb, (size_t)R * m->pad[L])) || (s = mlp_alloc(m, &m->loss_part, 592)) ||
      (s = mlp_alloc(m, &m->idx, (size_t)R)) || (s = mlp_alloc(m, &m->gemm_err, 1)))
    return fail(s);
  if ((s = refresh_copies(m)) != SHL_OK) return fail(s);
  if (cudaStreamSynchronize(m->stream) != cudaSuccess) return fail(SHL_ERR_CUDA);
  *out = m;
  return SHL_OK;
}

void shl_mlp_destroy(shl_mlp* m) {
  if (!m) return;
  if (m->stream) cudaStreamSynchronize(m->stream);
  for (void* p : m->allocs) cudaFree(p);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
}

shl_status shl_mlp_set_params(shl_mlp* m, uint32_t layer, const float* W, const float* b) {
  if (!m || (int)layer >= m->n_layers) return SHL_ERR_ARG;
  const int l = (int)layer, out = m->dim[l + 1], in = m->dim[l];
  if (W) {
    std::vector<float> w((size_t)m->pad[l + 1] * m->pad[l], 0.f);
    for (int r = 0; r < out; ++r) std::memcpy(&w[(size_t)r * m->pad[l]], W + (size_t)r * in, in * sizeof(float));
    MLP_TRY(cudaMemcpyAsync(m->W[l], w.data(), w.size() * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  }
  if (b) MLP_TRY(cudaMemcpyAsync(m->b[l], b, out * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MLP_CHECK(refresh_copies(m));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return SHL_OK;
}

shl_status shl_mlp_get_params(shl_mlp* m, uint32_t layer, float* W, float* b) {
  if (!m || (int)layer >= m->n_layers) return SHL_ERR_ARG;
  const int l = (int)layer, out = m->dim[l + 1], in = m->dim[l];
  if (W) {
    std::vector<float> w((size_t)m->pad[l + 1] * m->pad[l]);
    MLP_TRY(cudaMemcpyAsync(w.data(), m->W[l], w.size() * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MLP_TRY(cudaStreamSynchronize(m->stream));
    for (int r = 0; r < out; ++r) std::memcpy(W + (size_t)r * in, &w[(size_t)r * m->pad[l]], in * sizeof(float));
  }
  if (b) {
    MLP_TRY(cudaMemcpyAsync(b, m->b[l], out * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MLP_TRY(cudaStreamSynchronize(m->stream));
  }
  return SHL_OK;
}

shl_status shl_mlp_set_dataset(shl_mlp* m, const float* X, const float* T, uint64_t n) {
  if (!m || !X || !T || n == 0) return SHL_ERR_ARG;
  if (m->dX) {
    // datasets are replaced by allocating anew (old ones stay until destroy)
  }
  const size_t in = (size_t)m->dim[0], out = (size_t)m->dim[m->n_layers];
  MLP_CHECK(mlp_alloc(m, &m->dX, n * in));
  MLP_CHECK(mlp_alloc(m, &m->dT, n * out));
  MLP_TRY(cudaMemcpyAsync(m->dX, X, n * in * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MLP_TRY(cudaMemcpyAsync(m->dT, T, n * out * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MLP_TRY(cudaStreamSynchronize(m->stream));
  m->n_data = n;
  return SHL_OK;
}

shl_status shl_mlp_train(shl_mlp* m, uint32_t iters, uint32_t batch, float lr0, float lr_final, uint64_t seed,
                         float* loss_curve, uint32_t curve_every) {
  if (!m || !m->dX || batch == 0 || (int)batch > m->max_batch) return SHL_ERR_ARG;
  std::mt19937_64 rng(seed);
  std::vector<uint32_t> perm(m->n_data);
  for (size_t i = 0; i < perm.size(); ++i) perm[i] = (uint32_t)i;
  size_t pos = perm.size();
  std::vector<uint32_t> idx(batch);
  for (uint32_t it = 0; it < iters; ++it) {
    for (uint32_t k = 0; k < batch; ++k) {
      if (pos == perm.size()) {
        std::shuffle(perm.begin(), perm.end(), rng);
        pos = 0;
      }
      idx[k] = perm[pos++];
    }
    MLP_CHECK(load_batch(m, idx.data(), (int)batch));
    MLP_CHECK(forward(m));
    const bool record = loss_curve && curve_every && it % curve_every == 0;
    double loss = 0;
    MLP_CHECK(loss_and_grad(m, (int)batch, record ? &loss : nullptr));
    if (record) loss_curve[it / curve_every] = (float)loss;
    MLP_CHECK(backward(m, (int)batch));
    // cosine decay from lr0 to lr_final
    const float lr = lr_final + 0.5f * (lr0 - lr_final) * (1.f + std::cos(3.14159265358979f * it / std::max(1u, iters)));
    MLP_CHECK(adam(m, lr));
  }
  MLP_TRY(cudaStreamSynchronize(m->stream));
  MLP_TRY(cudaGetLastError());
  return gemm_status(m);
}

shl_status shl_mlp_predict(shl_mlp* m, const float* X, uint32_t n, float* Y) {
  if (!m || !X || !Y) return SHL_ERR_ARG;
  const int in = m->dim[0], L = m->n_layers, out = m->dim[L];
  float* dXtmp = nullptr;
  // inputs through a temporary device copy, in chunks of the maximum batch
  MLP_TRY(cudaMallocAsync((void**)&dXtmp, (size_t)std::max<uint32_t>(n, 1) * in * sizeof(float), m->stream));
  MLP_TRY(cudaMemcpyAsync(dXtmp, X, (size_t)n * in * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  std::vector<uint32_t> idx(m->max_batch);
  std::vector<float> z((size_t)m->batch_pad * m->pad[L]);
  shl_status st = SHL_OK;
  for (uint32_t s = 0; s < n && st == SHL_OK; s += (uint32_t)m->max_batch) {
    const int rows = (int)std::min<uint32_t>(m->max_batch, n - s);
    for (int k = 0; k < rows; ++k) idx[k] = k;
    if (cudaMemcpyAsync(m->idx, idx.data(), rows * sizeof(uint32_t), cudaMemcpyHostToDevice, m->stream) != cudaSuccess) {
      st = SHL_ERR_CUDA;
      break;
    }
    k_gather_batch<<<m->batch_pad, 256, 0, m->stream>>>(dXtmp + (size_t)s * in, nullptr, m->idx, rows, in, m->pad[0],
                                                        out, m->pad[L], m->batch_pad, m->H[0], nullptr);
    st = forward(m);
    if (st != SHL_OK) break;
    if (cudaMemcpyAsync(z.data(), m->Z[L], z.size() * sizeof(float), cudaMemcpyDeviceToHost, m->stream) != cudaSuccess ||
        cudaStreamSynchronize(m->stream) != cudaSuccess) {
      st = SHL_ERR_CUDA;
      break;
    }
    for (int r = 0; r < rows; ++r)
      std::memcpy(Y + (size_t)(s + r) * out, &z[(size_t)r * m->pad[L]], out * sizeof(float));
  }
  cudaFreeAsync(dXtmp, m->stream);
  MLP_TRY(cudaStreamSynchronize(m->stream));
  if (st != SHL_OK) return st;
  return gemm_status(m);
}

shl_status shl_mlp_gradients(shl_mlp* m, const float* X, const float* T, uint32_t n, double* loss, float* const* dW,
                             float* const* db) {
  if (!m || !X || !T || n == 0 || (int)n > m->max_batch) return SHL_ERR_ARG;
  // the rows as a temporary dataset
  float *x = m->dX, *t = m->dT;
  const size_t nd = m->n_data;
  const int in = m->dim[0], L = m->n_layers, out = m->dim[L];
  MLP_TRY(cudaMallocAsync((void**)&m->dX, (size_t)n * in * sizeof(float), m->stream));
  MLP_TRY(cudaMallocAsync((void**)&m->dT, (size_t)n * out * sizeof(float), m->stream));
  MLP_TRY(cudaMemcpyAsync(m->dX, X, (size_t)n * in * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  MLP_TRY(cudaMemcpyAsync(m->dT, T, (size_t)n * out * sizeof(float), cudaMemcpyHostToDevice, m->stream));
  std::vector<uint32_t> idx(n);
  for (uint32_t k = 0; k < n; ++k) idx[k] = k;
  shl_status st = load_batch(m, idx.data(), (int)n);
  if (st == SHL_OK) st = forward(m);
  if (st == SHL_OK) st = loss_and_grad(m, (int)n, loss);
  if (st == SHL_OK) st = backward(m, (int)n);
  cudaFreeAsync(m->dX, m->stream);
  cudaFreeAsync(m->dT, m->stream);
  m->dX = x;
  m->dT = t;
  m->n_data = nd;
  if (st != SHL_OK) return st;
  MLP_CHECK(gemm_status(m));
  for (int l = 0; l < L; ++l) {
    const int o = m->dim[l + 1], i = m->dim[l];
    if (dW && dW[l]) {
      std::vector<float> w((size_t)m->pad[l + 1] * m->pad[l]);
      MLP_TRY(cudaMemcpyAsync(w.data(), m->gW[l], w.size() * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
      MLP_TRY(cudaStreamSynchronize(m->stream));
      for (int r = 0; r < o; ++r) std::memcpy(dW[l] + (size_t)r * i, &w[(size_t)r * m->pad[l]], i * sizeof(float));
    }
    if (db && db[l]) MLP_TRY(cudaMemcpyAsync(db[l], m->gb[l], o * sizeof(float), cudaMemcpyDeviceToHost, m->stream));
  }
  MLP_TRY(cudaStreamSynchronize(m->stream));
  return SHL_OK;
}

shl_status shl_gemm_bf16(const uint16_t* A, const uint16_t* B, uint32_t M, uint32_t N, uint32_t K, float* C) {
  // C = A . B^T for host bf16 bit patterns (A: M x K, B: N x K), K a multiple of 8; a test entry point
  if (!A || !B || !C || K % 8 != 0) return SHL_ERR_ARG;
  shl_mlp tmp;
  MLP_TRY(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float* dC = nullptr;
  tmp.part_elems = (size_t)M * N * 8;
  shl_status st = SHL_OK;
  if (mlp_alloc(&tmp, &dA, (size_t)M * K) || mlp_alloc(&tmp, &dB, (size_t)N * K) || mlp_alloc(&tmp, &dC, (size_t)M * N) ||
      mlp_alloc(&tmp, &tmp.part, tmp.part_elems) || mlp_alloc(&tmp, &tmp.gemm_err, 1))
    st = SHL_ERR_OOM;
  if (st == SHL_OK) {
    cudaMemcpyAsync(dA, A, (size_t)M * K * 2, cudaMemcpyHostToDevice, tmp.stream);
    cudaMemcpyAsync(dB, B, (size_t)N * K * 2, cudaMemcpyHostToDevice, tmp.stream);
    st = gemm(&tmp, dA, (int)K, dB, (int)K, (int)M, (int)N, (int)K, EPI_PARTIAL, nullptr, dC, nullptr);
    cudaMemcpyAsync(C, dC, (size_t)M * N * sizeof(float), cudaMemcpyDeviceToHost, tmp.stream);
    if (cudaStreamSynchronize(tmp.stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) st = SHL_ERR_CUDA;
    if (st == SHL_OK) st = gemm_status(&tmp);
  }
  for (void* p : tmp.allocs) cudaFree(p);
  cudaStreamDestroy(tmp.stream);
  return st;
}

shl_status shl_gemm_bf16_time(uint32_t M, uint32_t N, uint32_t K, int reps, double* avg_ms) {
  // average device time of C = A . B^T on device-resident operands (CUDA events, reps launches after one warm-up)
  if (!avg_ms || M == 0 || N == 0 || K == 0 || K % 8 != 0 || reps < 1) return SHL_ERR_ARG;
  shl_mlp tmp;
  MLP_TRY(cudaStreamCreateWithFlags(&tmp.stream, cudaStreamNonBlocking));
  __nv_bfloat16 *dA = nullptr, *dB = nullptr;
  float* dC = nullptr;
  tmp.part_elems = (size_t)M * N * 8;
  shl_status st = SHL_OK;
  if (mlp_alloc(&tmp, &dA, (size_t)M * K) || mlp_alloc(&tmp, &dB, (size_t)N * K) || mlp_alloc(&tmp, &dC, (size_t)M * N) ||
      mlp_alloc(&tmp, &tmp.part, tmp.part_elems) || mlp_alloc(&tmp, &tmp.gemm_err, 1))
    st = SHL_ERR_OOM;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (st == SHL_OK && (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)) st = SHL_ERR_CUDA;
  if (st == SHL_OK) {
    k_fill_bf16<<<592, 256, 0, tmp.stream>>>(dA, (size_t)M * K, 1u);
    k_fill_bf16<<<592, 256, 0, tmp.stream>>>(dB, (size_t)N * K, 2u);
  }
  if (st == SHL_OK) st = gemm(&tmp, dA, (int)K, dB, (int)K, (int)M, (int)N, (int)K, EPI_PARTIAL, nullptr, dC, nullptr);
  if (st == SHL_OK) {
    cudaEventRecord(e0, tmp.stream);
    for (int r = 0; r < reps && st == SHL_OK; ++r)
      st = gemm(&tmp, dA, (int)K, dB, (int)K, (int)M, (int)N, (int)K, EPI_PARTIAL, nullptr, dC, nullptr);
    cudaEventRecord(e1, tmp.stream);
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) st = SHL_ERR_CUDA;
    *avg_ms = ms / reps;
  }
  if (st == SHL_OK) st = gemm_status(&tmp);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  cudaStreamSynchronize(tmp.stream);
  for (void* q : tmp.allocs) cudaFree(q);
  cudaStreamDestroy(tmp.stream);
  return st;
}

}  // extern "C"
