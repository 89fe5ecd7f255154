// Complex64 rank-k update on the 5th-generation tensor cores (tcgen05):
//   C (m x n) -= A (m x k) B (k x n),  k <= 32, column-major complex64,
// the trailing update of the precision form's blocked LU (the role of the
// pzgesv trailing pzgemm, ScalapackSolver.cpp:54-130 / LinearSystemSolver.hpp:55-65).
//
// Each FP32 component x is split into bf16 x_hi + x_lo (x_lo = bf16(x - x_hi));
// a real product is x_hi y_hi + x_hi y_lo + x_lo y_hi (three bf16 MMAs with
// FP32 accumulation, about 17 significant bits), so
//   Re(AB) = Ar Br + Ai (-Bi),  Im(AB) = Ar Bi + Ai Br
// takes 12 MMAs of M = 128, N = 64, K = 16 per 16 columns of k (B's imaginary
// part is staged twice, with both signs; a sign flip is exact in bf16). One
// CTA of 128 threads owns a 128 x 64 tile of C: the operands are split and
// stored in shared memory in the canonical K-major layout without swizzle
// (8 x 16-byte core matrices), thread 0 issues the MMAs into two TMEM
// accumulators (Re, Im; 64 columns each: 128 TMEM columns, four CTAs per
// SM), commits them to an mbarrier, and the four warps read their 32 TMEM
// lanes back (tcgen05.ld 32x32b) and subtract from C, whose first 16 columns
// are loaded while the MMAs run. Waits are bounded: on time-out the kernel
// raises *err, still frees its TMEM and leaves C untouched.
#include <cuda_bf16.h>
#include <stdint.h>

#include "om_internal.h"

namespace om {

namespace {

constexpr int kTcM = 128, kTcN = 64, kTcK = 32;
constexpr uint32_t kTmemCols = 128;  // 2 x 64 accumulator columns
// shared-memory operand tiles (bf16): A parts 128 x 32, B parts 64 x 32
// (Ar, Ai, Br, Bi, -Bi: hi and lo each)
constexpr int kAPart = kTcM * kTcK * 2, kBPart = kTcN * kTcK * 2;
constexpr int kTcSmem = 4 * kAPart + 6 * kBPart + 64;

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading (K) and
// stride (M/N) byte offsets between core matrices, descriptor version 1, no
// swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
  d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
  d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major.
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                            ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdesc), "r"(acc));
}

// byte offset of element (row r, k index c) in a K-major no-swizzle tile with
// 32 columns of K: core matrices of 8 rows x 8 bf16, K-adjacent ones 128 B
// apart (LBO), row-adjacent ones 512 B apart (SBO)
__device__ __forceinline__ int kmajor_off(int r, int c) {
  return (r >> 3) * 512 + (c >> 3) * 128 + (r & 7) * 16 + (c & 7) * 2;
}

__device__ __forceinline__ void split_store(unsigned char *hi, unsigned char *lo, int off, float x) {
  const __nv_bfloat16 h = __float2bfloat16_rn(x);
  const __nv_bfloat16 l = __float2bfloat16_rn(x - __bfloat162float(h));
  *reinterpret_cast<__nv_bfloat16 *>(hi + off) = h;
  *reinterpret_cast<__nv_bfloat16 *>(lo + off) = l;
}

__global__ void __launch_bounds__(128) k_cgemm_sub_tc(const float2 *A, long lda, const float2 *B,
                                                      long ldb, float2 *C, long ldc, long m, long n,
                                                      int k, int *err) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  unsigned char *Arh = tsm, *Arl = tsm + kAPart, *Aih = tsm + 2 * kAPart, *Ail = tsm + 3 * kAPart;
  unsigned char *Brh = tsm + 4 * kAPart, *Brl = Brh + kBPart, *Bih = Brh + 2 * kBPart,
                *Bil = Brh + 3 * kBPart, *Bnh = Brh + 4 * kBPart, *Bnl = Brh + 5 * kBPart;
  uint64_t *mbar = reinterpret_cast<uint64_t *>(tsm + 4 * kAPart + 6 * kBPart);
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(tsm + 4 * kAPart + 6 * kBPart + 16);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long r0 = (long)blockIdx.x * kTcM, c0 = (long)blockIdx.y * kTcN;

  if(warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if(t == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mbar)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }

  // A tile: thread t owns row r0 + t (coalesced down each column); all of a
  // thread's loads are issued before the first split, so that they are in
  // flight together
  {
    const long r = r0 + t;
    float2 av[kTcK];
#pragma unroll
    for(int c = 0; c < kTcK; ++c)
      av[c] = (c < k && r < m) ? A[(long)c * lda + r] : make_float2(0.f, 0.f);
#pragma unroll
    for(int c = 0; c < kTcK; ++c) {
      const int off = kmajor_off(t, c);
      split_store(Arh, Arl, off, av[c].x);
      split_store(Aih, Ail, off, av[c].y);
    }
  }
  // B tile as N x K: thread t owns column c0 + t / 2, half of K (contiguous in memory)
  {
    const int j = t >> 1, cb = (t & 1) * 16;
    const long col = c0 + j;
    float2 bv[16];
#pragma unroll
    for(int c = 0; c < 16; ++c)
      bv[c] = (cb + c < k && col < n) ? B[col * ldb + cb + c] : make_float2(0.f, 0.f);
#pragma unroll
    for(int c = 0; c < 16; ++c) {
      const int off = kmajor_off(j, cb + c);
      split_store(Brh, Brl, off, bv[c].x);
      split_store(Bih, Bil, off, bv[c].y);
      split_store(Bnh, Bnl, off, -bv[c].y);
    }
  }
  // generic-proxy stores -> visible to the tensor core (async proxy)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t d_re = tmem, d_im = tmem + kTcN;

  if(t == 0) {
    for(int s = 0; s < kTcK / 16; ++s) {
      const uint32_t ko = s * 256;  // two core matrices along K per MMA
      auto da = [&](unsigned char *p) { return umma_desc(smem_addr(p) + ko, 128, 512); };
      const uint32_t acc = s > 0;  // the first K step overwrites the accumulators
      // Re: Ar Br + Ai (-Bi)
      mma_bf16(d_re, da(Arh), da(Brh), acc);
      mma_bf16(d_re, da(Arh), da(Brl), 1);
      mma_bf16(d_re, da(Arl), da(Brh), 1);
      mma_bf16(d_re, da(Aih), da(Bnh), 1);
      mma_bf16(d_re, da(Aih), da(Bnl), 1);
      mma_bf16(d_re, da(Ail), da(Bnh), 1);
      // Im: Ar Bi + Ai Br
      mma_bf16(d_im, da(Arh), da(Bih), acc);
      mma_bf16(d_im, da(Arh), da(Bil), 1);
      mma_bf16(d_im, da(Arl), da(Bih), 1);
      mma_bf16(d_im, da(Aih), da(Brh), 1);
      mma_bf16(d_im, da(Aih), da(Brl), 1);
      mma_bf16(d_im, da(Ail), da(Brh), 1);
    }
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_addr(mbar))
        : "memory");
  }
  // the first 16 columns of this thread's row of C, loaded while the MMAs run
  const long r = r0 + warp * 32 + lane;
  float2 cpre[16];
#pragma unroll
  for(int q = 0; q < 16; ++q) {
    const long col = c0 + q;
    cpre[q] = (r < m && col < n) ? C[col * ldc + r] : make_float2(0.f, 0.f);
  }
  // bounded wait for the MMAs (phase 0 of the mbarrier)
  uint32_t done = 0;
  for(long it = 0; it < (1L << 24) && !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(0u)
        : "memory");
  }
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  done = __syncthreads_and(done);  // one decision for the whole CTA
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if(!done) {
    if(t == 0)
      atomicExch(err, 1);
  } else {
    // warp w reads TMEM lanes 32 w .. 32 w + 31 = rows r0 + 32 w + lane
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    for(int cc = 0; cc < kTcN; cc += 16) {
      uint32_t a[16], b[16];
#define OM_TMEM_LD16(dst, addr)                                                                     \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
               : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]),  \
                 "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]),              \
                 "=r"(dst[11]), "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])           \
               : "r"(addr))
      OM_TMEM_LD16(a, d_re + lane_base + cc);
      OM_TMEM_LD16(b, d_im + lane_base + cc);
#undef OM_TMEM_LD16
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if(r < m) {
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const long col = c0 + cc + q;
          if(col < n) {
            float2 v = cc == 0 ? cpre[q] : C[col * ldc + r];
            v.x -= __uint_as_float(a[q]);
            v.y -= __uint_as_float(b[q]);
            C[col * ldc + r] = v;
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols));
  }
}

}  // namespace

void launch_cgemm_sub_tc(om_context *ctx, const float2 *A, long lda, const float2 *B, long ldb,
                         float2 *C, long ldc, long m, long n, int k, int *d_err) {
  cudaFuncSetAttribute(k_cgemm_sub_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
  dim3 grid((unsigned)((m + kTcM - 1) / kTcM), (unsigned)((n + kTcN - 1) / kTcN));
  k_cgemm_sub_tc<<<grid, 128, kTcSmem, ctx->stream>>>(A, lda, B, ldb, C, ldc, m, n, k, d_err);
  ctx->last_launches++;
}

}  // namespace om
