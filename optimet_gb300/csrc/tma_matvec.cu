// Complex64 matrix-vector product with the matrix staged by the Tensor
// Memory Accelerator: the inner FP32 GMRES matvec of the precision form.
//
// Same decomposition as the plain kernels: tiles of 256 rows x `cols` columns
// taken from a counter by a capped grid, x chunk in shared memory, one row
// per thread, partial sums per column chunk. Here the tile's columns arrive
// in stages of 16 columns (256 x 16 complex64 = 32 KB, one 2-D TMA box of the
// column-major matrix) through a ring of shared-memory buffers, each
// with an mbarrier that the TMA completes by transaction bytes. Thread 0
// issues the copies; after all threads have consumed a buffer it refills it
// with the stage four ahead. The arithmetic and its order per thread are those
// of the plain kernel, so the results are bitwise the same.
//
// The same kernel serves the precision form's bf16 copy of the matrix
// (kBf16): 4-byte entries (real part in the low 16 bits, imaginary in the
// high), 32 columns per 32 KB stage, unpacked to FP32 by two bit operations and
// accumulated in FP32 in the same order. The first inner product of a solve
// runs on the complex64 matrix and writes that copy as it goes (`copy`: each
// entry rounded to nearest even, coalesced 4-byte stores), so the copy costs
// one extra write of 4 bytes per entry and no extra read.
//
// Waits are bounded: every thread polls the stage's barrier a bounded number
// of times and the CTA decides together (a barrier with an OR reduction)
// whether the stage arrived. If not, thread 0 records the failure in the
// error flag the solver reads back, waits (bounded again) for the stages it
// has already issued so that no copy lands in this CTA's shared memory after
// it exits, and the CTA stops taking tiles.
#include <cuda.h>

#include <mutex>
#include <type_traits>

#include "om_internal.h"
#include "om_krylov.cuh"

namespace om {

namespace {

constexpr int kTmaRows = 256;
constexpr uint32_t kStageBytes = 32768;  // 256 rows x 16 complex64 or 32 bf16 columns
// Stages in the ring: four for the complex64 matrix (one CTA per SM); two for
// the bf16 copy, whose product does twice the arithmetic per byte and
// measured 0.66 of the copy peak with four stages (one CTA of eight warps per
// SM) and 0.90 with two (three CTAs per SM) at n = 16,000.
template <bool kBf16> struct TmaEntry {
  typedef float2 T;
  static constexpr int kCols = 16;
  static constexpr int kStages = 4;
  static __device__ __forceinline__ float2 load(const T &v) { return v; }
};
template <> struct TmaEntry<true> {
  typedef Bf16c T;
  static constexpr int kCols = 32;
  static constexpr int kStages = 2;
  static __device__ __forceinline__ float2 load(const T &v) { return mv_entry<float2>(v); }
};

__device__ __forceinline__ uint32_t sa(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_load(void *dst, const CUtensorMap *tm, int row, int col,
                                         uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          sa(dst)),
      "l"(tm), "r"(row), "r"(col), "r"(sa(bar))
      : "memory");
}

__device__ __forceinline__ void arm(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes)
               : "memory");
}

// bounded wait for the given phase parity; false on time-out
__device__ __forceinline__ bool wait_phase(uint64_t *bar, uint32_t parity) {
  for(long it = 0; it < (1L << 26); ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(sa(bar)), "r"(parity)
        : "memory");
    if(ok)
      return true;
  }
  return false;
}

template <bool kBf16>
__global__ void __launch_bounds__(kTmaRows) k_matvec_tma(const __grid_constant__ CUtensorMap tm, long n,
                                                          const float2 *x, float2 *part, int row_tiles,
                                                          long tiles, unsigned long long *next, int cols,
                                                          int *err, Bf16c *copy, long ldc) {
  typedef typename TmaEntry<kBf16>::T E;
  constexpr int kTmaStageCols = TmaEntry<kBf16>::kCols;
  constexpr int kTmaStages = TmaEntry<kBf16>::kStages;
  extern __shared__ __align__(128) unsigned char tsm_[];
  E *stage = reinterpret_cast<E *>(tsm_);  // [kTmaStages][kTmaStageCols][kTmaRows]
  float2 *xs = reinterpret_cast<float2 *>(tsm_ + kTmaStages * kStageBytes);
  __shared__ __align__(8) uint64_t bar[kTmaStages];
  __shared__ long tile;
  __shared__ int fail;
  const int t = threadIdx.x;
  if(t == 0) {
    for(int s = 0; s < kTmaStages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(&bar[s])), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fail = 0;
  }
  __syncthreads();
  uint32_t parity = 0;  // bit s: parity of the next completion of bar[s]
  for(;;) {
    __syncthreads();
    if(t == 0)
      tile = (long)atomicAdd(next, 1ull);
    __syncthreads();
    const long tl = tile;
    if(tl >= tiles || fail)
      break;
    const long ct = tl / row_tiles, rt = tl - ct * row_tiles;
    const long i = rt * kTmaRows + t;
    const long j0 = ct * cols;
    const long j1 = min(n, j0 + cols);
    const int nst = (int)((j1 - j0 + kTmaStageCols - 1) / kTmaStageCols);
    if(t == 0) {
      for(int s = 0; s < kTmaStages && s < nst; ++s) {
        arm(&bar[s], kStageBytes);
        tma_load(stage + (size_t)s * kTmaStageCols * kTmaRows, &tm, (int)(rt * kTmaRows),
                 (int)(j0 + s * kTmaStageCols), &bar[s]);
      }
    }
    for(long j = j0 + t; j < j1; j += kTmaRows)
      xs[j - j0] = x[j];
    __syncthreads();
    // accumulators (the plain kernel's order: columns in groups of eight,
    // alternating accumulators, a tail of fewer than eight into acc0)
    float2 acc0 = make_float2(0.f, 0.f), acc1 = make_float2(0.f, 0.f);
    const long full8 = j0 + ((j1 - j0) / 8) * 8;
    for(int s = 0; s < nst; ++s) {
      const int slot = s % kTmaStages;
      const bool arrived = wait_phase(&bar[slot], (parity >> slot) & 1u);
      parity ^= 1u << slot;
      if(__syncthreads_or(!arrived)) {
        if(t == 0) {
          atomicExch(err, 1);
          for(int q = s + 1; q < nst && q < s + kTmaStages; ++q) {  // issued, not yet waited for
            const int sl = q % kTmaStages;
            wait_phase(&bar[sl], (parity >> sl) & 1u);
            parity ^= 1u << sl;
          }
          fail = 1;
        }
        break;
      }
      const E *sb = stage + (size_t)slot * kTmaStageCols * kTmaRows;
      const long cb = j0 + (long)s * kTmaStageCols;
      const int ccount = (int)min((long)kTmaStageCols, j1 - cb);
      if(i < n) {
        for(int c = 0; c < ccount; ++c) {
          const float2 a = TmaEntry<kBf16>::load(sb[c * kTmaRows + t]);
          if(!kBf16 && copy)
            copy[(cb + c) * ldc + i] = pack_bf16c(a);
          const long j = cb + c;
          const float2 xv = xs[j - j0];
          const bool alt = j < full8 && ((j - j0) & 1);
          float2 acc = alt ? acc1 : acc0;
          acc.x = fmaf(a.x, xv.x, acc.x);
          acc.x = fmaf(-a.y, xv.y, acc.x);
          acc.y = fmaf(a.x, xv.y, acc.y);
          acc.y = fmaf(a.y, xv.x, acc.y);
          if(alt)
            acc1 = acc;
          else
            acc0 = acc;
        }
      }
      __syncthreads();  // the buffer is free again
      if(t == 0 && s + kTmaStages < nst) {
        arm(&bar[slot], kStageBytes);
        tma_load(stage + (size_t)slot * kTmaStageCols * kTmaRows, &tm, (int)(rt * kTmaRows),
                 (int)(j0 + (long)(s + kTmaStages) * kTmaStageCols), &bar[slot]);
      }
    }
    __syncthreads();  // `fail` as thread 0 left it
    if(i < n && !fail) {
      acc0.x += acc1.x;
      acc0.y += acc1.y;
      part[ct * n + i] = acc0;
    }
  }
}

typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                             const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                             CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                             CUtensorMapFloatOOBfill);

EncodeFn encode_fn() {
  static EncodeFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
           cudaSuccess &&
       q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeFn>(p);
    cudaGetLastError();
  });
  return fn;
}

}  // namespace

void *tensor_map_encoder() { return reinterpret_cast<void *>(encode_fn()); }

// Launches the TMA matvec on the complex64 matrix S (ld n), writing its bf16
// copy into `copy` (ld ldc) when that is not null; false when the tensor map
// cannot be made (the caller then runs the plain kernel).
bool launch_matvec_tma(om_context *ctx, const float2 *S, long n, const float2 *x, float2 *part, int row_tiles,
                       long tiles, int cols, unsigned grid, void *copy, long ldc) {
  EncodeFn enc = encode_fn();
  if(!enc || (reinterpret_cast<uintptr_t>(S) & 15) || (n & 1))
    return false;
  alignas(64) CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)n * sizeof(float2)};
  const cuuint32_t box[2] = {kTmaRows, (cuuint32_t)TmaEntry<false>::kCols};
  const cuuint32_t estr[2] = {1, 1};
  if(enc(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, const_cast<float2 *>(S), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  const size_t smem = TmaEntry<false>::kStages * kStageBytes + (size_t)cols * sizeof(float2);
  cudaFuncSetAttribute(k_matvec_tma<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_matvec_tma<false><<<grid, kTmaRows, smem, ctx->stream>>>(tm, n, x, part, row_tiles, tiles,
                                                             ctx->d_tile_counter, cols, ctx->d_tma_err,
                                                             static_cast<Bf16c *>(copy), ldc);
  return true;
}

// The same product on the bf16 copy H (n x n, ld ldh, ldh a multiple of 4 so
// that its column stride is a multiple of 16 bytes); false when the tensor map
// cannot be made.
bool launch_matvec_bf16(om_context *ctx, const void *H, long n, long ldh, const float2 *x, float2 *part,
                        int row_tiles, long tiles, int cols, unsigned grid) {
  EncodeFn enc = encode_fn();
  if(!enc || (reinterpret_cast<uintptr_t>(H) & 15) || (ldh & 3))
    return false;
  alignas(64) CUtensorMap tm;
  const cuuint64_t dims[2] = {(cuuint64_t)n, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)ldh * sizeof(uint32_t)};
  const cuuint32_t box[2] = {kTmaRows, (cuuint32_t)TmaEntry<true>::kCols};
  const cuuint32_t estr[2] = {1, 1};
  if(enc(&tm, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void *>(H), dims, strides, box, estr,
         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  const size_t smem = TmaEntry<true>::kStages * kStageBytes + (size_t)cols * sizeof(float2);
  cudaFuncSetAttribute(k_matvec_tma<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  k_matvec_tma<true><<<grid, kTmaRows, smem, ctx->stream>>>(tm, n, x, part, row_tiles, tiles,
                                                            ctx->d_tile_counter, cols, ctx->d_tma_err, nullptr,
                                                            0);
  return true;
}

}  // namespace om
