// Complex64 rank-k update on the 5th-generation tensor cores (tcgen05):
//   C (m x n) -= A (m x k) B (k x n),  any k >= 1, column-major complex64,
// the trailing update of the precision form's blocked LU (the role of the
// pzgesv trailing pzgemm, ScalapackSolver.cpp:54-130 / LinearSystemSolver.hpp:55-65).
//
// Each FP32 component x is split into bf16 x_hi + x_lo (x_lo = bf16(x - x_hi));
// a real product is x_hi y_hi + x_hi y_lo + x_lo y_hi (three bf16 MMAs with
// FP32 accumulation, about 17 significant bits), so
//   Re(AB) = Ar Br + Ai (-Bi),  Im(AB) = Ar Bi + Ai Br
// takes 12 MMAs of M = 128, N = 64, K = 16 per 16 columns of k (B's imaginary
// part is staged twice, with both signs; a sign flip is exact in bf16). One
// CTA of 128 threads owns a 128 x 64 tile of C. k runs in chunks of 32: each
// chunk's operands are split and stored in shared memory in the canonical
// K-major layout without swizzle (8 x 16-byte core matrices), thread 0 issues
// its MMAs into two TMEM accumulators (Re, Im; 64 columns each: 128 TMEM
// columns) and commits them to an mbarrier, and the next chunk's operands are
// loaded into registers while those MMAs run. After the last chunk the four
// warps read their 32 TMEM lanes back (tcgen05.ld 32x32b) and subtract from
// C, whose first 16 columns are loaded while the last MMAs run: C is read and
// written once for the whole rank-k update. Waits are bounded: on time-out
// the kernel raises *err, still frees its TMEM and leaves C untouched.
//
// From k = 64 (the LU's rank-128 updates) a second path splits the operands
// once and streams them by bulk copies (k_tc_split_a/b, k_cgemm_sub_tc2,
// below).
#include <algorithm>

#include <cuda.h>
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

// Two FP32 values split into bf16 hi and lo parts, packed as bf16x2
// (the first value in the low half): hi = bf16(x), lo = bf16(x - hi), both
// rounded to nearest.
__device__ __forceinline__ void split2(float a, float b, uint32_t &hi, uint32_t &lo) {
  const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
  const float2 hf = __bfloat1622float2(h);
  const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

__device__ __forceinline__ void st_shared_v4(unsigned char *p, uint32_t x, uint32_t y, uint32_t z,
                                             uint32_t w) {
  asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(smem_addr(p)), "r"(x), "r"(y), "r"(z),
               "r"(w)
               : "memory");
}

// Eight K-consecutive complex values of one row (v[0..7]) into one 16-byte
// core-matrix row of each part: the real parts' hi / lo, the imaginary parts'
// hi / lo, and (for B) the negated imaginary parts' hi / lo, whose bf16 values
// are those of the imaginary parts with the sign bit flipped (rounding to
// nearest is symmetric).
__device__ __forceinline__ void stage8(const float2 *v, int off, unsigned char *rh, unsigned char *rl,
                                       unsigned char *ih, unsigned char *il, unsigned char *nh,
                                       unsigned char *nl) {
  uint32_t a[4], b[4], c[4], d[4];
#pragma unroll
  for(int p = 0; p < 4; ++p) {
    split2(v[2 * p].x, v[2 * p + 1].x, a[p], b[p]);
    split2(v[2 * p].y, v[2 * p + 1].y, c[p], d[p]);
  }
  st_shared_v4(rh + off, a[0], a[1], a[2], a[3]);
  st_shared_v4(rl + off, b[0], b[1], b[2], b[3]);
  st_shared_v4(ih + off, c[0], c[1], c[2], c[3]);
  st_shared_v4(il + off, d[0], d[1], d[2], d[3]);
  if(nh) {
    constexpr uint32_t sgn = 0x80008000u;
    st_shared_v4(nh + off, c[0] ^ sgn, c[1] ^ sgn, c[2] ^ sgn, c[3] ^ sgn);
    st_shared_v4(nl + off, d[0] ^ sgn, d[1] ^ sgn, d[2] ^ sgn, d[3] ^ sgn);
  }
}

// Bounded wait for the completion of the mbarrier phase of the given parity;
// 1 when it completed, 0 on time-out.
__device__ __forceinline__ uint32_t wait_phase(uint64_t *mbar, uint32_t parity) {
  uint32_t done = 0;
  for(long it = 0; it < (1L << 24) && !done; ++it) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(parity)
        : "memory");
  }
  return done;
}

__global__ void __launch_bounds__(128, 3) k_cgemm_sub_tc(const float2 *A, long lda, const float2 *B,
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

  // K runs in chunks of kTcK columns through the one set of operand tiles.
  // Chunk q + 1 is loaded into registers while the MMAs of chunk q run, and
  // is stored to shared memory once those MMAs have completed (mbarrier
  // phase q). A tile: thread t owns row r0 + t (coalesced down each column);
  // B tile as N x K: thread t owns column c0 + t / 2, half of the chunk
  // (contiguous in memory).
  // the C tile's lines requested into L2 now, so that its DRAM reads overlap
  // the operand staging and the MMAs: thread t covers column t / 2, rows
  // (t & 1) 64 .. (t & 1) 64 + 63 (four 128-byte lines)
  {
    const long col = c0 + (t >> 1);
    if(col < n) {
#pragma unroll
      for(int i = 0; i < 4; ++i) {
        const long row = r0 + (t & 1) * 64 + 16 * i;
        if(row < m)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(C + col * ldc + row));
      }
    }
  }
  const int nq = (k + kTcK - 1) / kTcK;
  // B's chunks start at even offsets of 16-byte aligned columns when B is
  // 16-byte aligned and ldb is even
  const bool bvec = ((reinterpret_cast<uintptr_t>(B) & 15) == 0) && ((ldb & 1) == 0);
  const long ra = r0 + t;
  const int jb = t >> 1, cb = (t & 1) * 16;
  const long colb = c0 + jb;
  float2 av[kTcK], bv[16];
  auto load_chunk = [&](int q) {
    const int kq = q * kTcK;
#pragma unroll
    for(int c = 0; c < kTcK; ++c)
      av[c] = (kq + c < k && ra < m) ? A[(long)(kq + c) * lda + ra] : make_float2(0.f, 0.f);
    if(bvec && kq + cb + 16 <= k && colb < n) {  // 16-byte loads
      const float4 *src = reinterpret_cast<const float4 *>(B + colb * ldb + kq + cb);
#pragma unroll
      for(int c = 0; c < 8; ++c) {
        const float4 w = src[c];
        bv[2 * c] = make_float2(w.x, w.y);
        bv[2 * c + 1] = make_float2(w.z, w.w);
      }
    } else {
#pragma unroll
      for(int c = 0; c < 16; ++c)
        bv[c] = (kq + cb + c < k && colb < n) ? B[colb * ldb + kq + cb + c] : make_float2(0.f, 0.f);
    }
  };
  load_chunk(0);
  uint32_t tmem = 0;
  bool ok = true;
  for(int q = 0; q < nq; ++q) {
    uint32_t done = 1;
    if(q > 0)  // the MMAs of chunk q - 1 have read the tiles
      done = wait_phase(mbar, (uint32_t)(q - 1) & 1u);
#pragma unroll
    for(int g = 0; g < kTcK / 8; ++g)
      stage8(av + 8 * g, kmajor_off(t, 8 * g), Arh, Arl, Aih, Ail, nullptr, nullptr);
#pragma unroll
    for(int g = 0; g < 2; ++g)
      stage8(bv + 8 * g, kmajor_off(jb, cb + 8 * g), Brh, Brl, Bih, Bil, Bnh, Bnl);
    // generic-proxy stores -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    done = __syncthreads_and(done);  // one decision for the whole CTA
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    tmem = *tmem_slot;
    if(!done) {
      ok = false;
      break;
    }
    if(t == 0) {
      const uint32_t d_re = tmem, d_im = tmem + kTcN;
      for(int s = 0; s < kTcK / 16; ++s) {
        const uint32_t ko = s * 256;  // two core matrices along K per MMA
        auto da = [&](unsigned char *p) { return umma_desc(smem_addr(p) + ko, 128, 512); };
        const uint32_t acc = q > 0 || s > 0;  // the first K step overwrites the accumulators
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
    if(q + 1 < nq)
      load_chunk(q + 1);
  }
  const uint32_t d_re = tmem, d_im = tmem + kTcN;

  // columns 0 .. 31 of this thread's row of C, loaded while the last MMAs
  // run; columns 32 .. 47 and 48 .. 63 follow into the registers of the
  // 16 columns just done
  const long r = r0 + warp * 32 + lane;
  float2 cv[32];
#pragma unroll
  for(int q = 0; q < 32; ++q) {
    const long col = c0 + q;
    cv[q] = (r < m && col < n) ? C[col * ldc + r] : make_float2(0.f, 0.f);
  }
  // bounded wait for the last chunk's MMAs (phase nq - 1 of the mbarrier)
  uint32_t done = ok ? wait_phase(mbar, (uint32_t)(nq - 1) & 1u) : 0u;
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  done = __syncthreads_and(done);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if(!done) {
    if(t == 0)
      atomicExch(err, 1);
  } else {
    // warp w reads TMEM lanes 32 w .. 32 w + 31 = rows r0 + 32 w + lane
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
    for(int g = 0; g < kTcN / 16; ++g) {
      const int cc = 16 * g, base = (g & 1) * 16;
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
            float2 v = cv[base + q];
            v.x -= __uint_as_float(a[q]);
            v.y -= __uint_as_float(b[q]);
            C[col * ldc + r] = v;
          }
        }
      }
      if(g < 2) {
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const long col = c0 + cc + 32 + q;
          cv[base + q] = (r < m && col < n) ? C[col * ldc + r] : make_float2(0.f, 0.f);
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

// --- pre-split operands, streamed by bulk copies --------------------------
//
// For the LU's rank-128 trailing updates the operands are split once, before
// the update: L21 (m x k) and U12 (k x n) go to bf16 hi / lo parts laid out
// exactly as the shared-memory tiles above (per 128-row tile of A or 64-column
// tile of B and per 32-column chunk of k: the parts one after another, each
// in the K-major core-matrix layout). The update kernel then copies each
// chunk's tiles with one-dimensional bulk copies (cp.async.bulk, completion
// counted on an mbarrier) into one of two shared-memory stages, so that no
// thread converts or stores operands in the loop. The real part is kept as
// two accumulators (Ar Br and Ai Bi, subtracted in the epilogue) instead of
// staging -Bi, which leaves 48 KB a stage: two stages and two CTAs per SM.
constexpr int kStageA = 4 * kAPart, kStageB = 4 * kBPart, kStage = kStageA + kStageB;
constexpr int kTc2Smem = 2 * kStage + 128;
constexpr uint32_t kTmem2Cols = 256;  // three 64-column accumulators

// A (m x k, lda) -> per (row tile, chunk): Arh, Arl, Aih, Ail (8 KB each).
// One CTA of 512 threads per (row tile, chunk): thread t takes row t % 128
// and the chunk's K columns 8 (t / 128) .. 8 (t / 128) + 7.
__global__ void __launch_bounds__(512) k_tc_split_a(const float2 *A, long lda, long m, int k, int nq,
                                                    unsigned char *out) {
  const int t = threadIdx.x, r = t & 127, g = t >> 7;
  const long row = (long)blockIdx.x * kTcM + r;
  const int q = blockIdx.y, k0 = q * kTcK + 8 * g;
  float2 v[8];
#pragma unroll
  for(int j = 0; j < 8; ++j)
    v[j] = (row < m && k0 + j < k) ? A[(long)(k0 + j) * lda + row] : make_float2(0.f, 0.f);
  uint32_t a[4], b[4], c[4], d[4];
#pragma unroll
  for(int p = 0; p < 4; ++p) {
    split2(v[2 * p].x, v[2 * p + 1].x, a[p], b[p]);
    split2(v[2 * p].y, v[2 * p + 1].y, c[p], d[p]);
  }
  unsigned char *o = out + ((size_t)blockIdx.x * nq + q) * kStageA + kmajor_off(r, 8 * g);
  *reinterpret_cast<uint4 *>(o) = make_uint4(a[0], a[1], a[2], a[3]);
  *reinterpret_cast<uint4 *>(o + kAPart) = make_uint4(b[0], b[1], b[2], b[3]);
  *reinterpret_cast<uint4 *>(o + 2 * kAPart) = make_uint4(c[0], c[1], c[2], c[3]);
  *reinterpret_cast<uint4 *>(o + 3 * kAPart) = make_uint4(d[0], d[1], d[2], d[3]);
}

// B (k x n, ldb) -> per (column tile, chunk): Brh, Brl, Bih, Bil (4 KB each),
// as N x K. One CTA of 256 threads per (column tile, chunk): thread t takes
// column t % 64 and the chunk's K rows 8 (t / 64) .. 8 (t / 64) + 7.
__global__ void __launch_bounds__(256) k_tc_split_b(const float2 *B, long ldb, long n, int k, int nq,
                                                    unsigned char *out) {
  const int t = threadIdx.x, j = t & 63, g = t >> 6;
  const long col = (long)blockIdx.x * kTcN + j;
  const int q = blockIdx.y, k0 = q * kTcK + 8 * g;
  float2 v[8];
#pragma unroll
  for(int i = 0; i < 8; ++i)
    v[i] = (col < n && k0 + i < k) ? B[col * ldb + k0 + i] : make_float2(0.f, 0.f);
  uint32_t a[4], b[4], c[4], d[4];
#pragma unroll
  for(int p = 0; p < 4; ++p) {
    split2(v[2 * p].x, v[2 * p + 1].x, a[p], b[p]);
    split2(v[2 * p].y, v[2 * p + 1].y, c[p], d[p]);
  }
  unsigned char *o = out + ((size_t)blockIdx.x * nq + q) * kStageB + kmajor_off(j, 8 * g);
  *reinterpret_cast<uint4 *>(o) = make_uint4(a[0], a[1], a[2], a[3]);
  *reinterpret_cast<uint4 *>(o + kBPart) = make_uint4(b[0], b[1], b[2], b[3]);
  *reinterpret_cast<uint4 *>(o + 2 * kBPart) = make_uint4(c[0], c[1], c[2], c[3]);
  *reinterpret_cast<uint4 *>(o + 3 * kBPart) = make_uint4(d[0], d[1], d[2], d[3]);
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void arrive_expect(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

// C (m x n) -= A B from the pre-split tiles (nq chunks of 32 columns of k).
// Thread 0 issues the bulk copies (two stages ahead) and the MMAs; the copy
// of chunk q + 2 waits for the MMAs of chunk q (mbarrier `empty`), the MMAs of
// chunk q for its copy (mbarrier `full`). The other threads load their rows
// of C meanwhile; all wait for the last chunk's MMAs, then run the epilogue.
// Waits are bounded: on time-out the kernel raises *err, frees its TMEM and
// leaves C untouched.
__global__ void __launch_bounds__(128) k_cgemm_sub_tc2(const unsigned char *As, const unsigned char *Bs,
                                                       int nq, float2 *C, long ldc, long m, long n,
                                                       int *err) {
  extern __shared__ __align__(1024) unsigned char tsm[];
  uint64_t *full = reinterpret_cast<uint64_t *>(tsm + 2 * kStage);  // [2]
  uint64_t *empty = full + 2;                                        // [2]
  uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(full + 4);
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long r0 = (long)blockIdx.x * kTcM, c0 = (long)blockIdx.y * kTcN;
  const unsigned char *Ab = As + (size_t)blockIdx.x * nq * kStageA;
  const unsigned char *Bb = Bs + (size_t)blockIdx.y * nq * kStageB;

  if(warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(tmem_slot)),
                 "r"(kTmem2Cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if(t == 0) {
    for(int i = 0; i < 4; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(full + i)), "r"(1));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // the C tile's lines requested into L2 (as in k_cgemm_sub_tc)
  {
    const long col = c0 + (t >> 1);
    if(col < n) {
#pragma unroll
      for(int i = 0; i < 4; ++i) {
        const long row = r0 + (t & 1) * 64 + 16 * i;
        if(row < m)
          asm volatile("prefetch.global.L2 [%0];" ::"l"(C + col * ldc + row));
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  const uint32_t d_r1 = tmem, d_r2 = tmem + kTcN, d_im = tmem + 2 * kTcN;

  uint32_t ok = 1;
  if(t == 0) {
    int issued = 0, landed = 0, committed = 0;  // chunks copied in / waited for / with MMAs issued
    auto issue = [&](int q) {
      const int s = q & 1;
      arrive_expect(full + s, (uint32_t)kStage);
      bulk_load(tsm + s * kStage, Ab + (size_t)q * kStageA, (uint32_t)kStageA, full + s);
      bulk_load(tsm + s * kStage + kStageA, Bb + (size_t)q * kStageB, (uint32_t)kStageB, full + s);
      issued = q + 1;
    };
    issue(0);
    if(nq > 1)
      issue(1);
    for(int q = 0; q < nq; ++q) {
      const int s = q & 1;
      const uint32_t par = (uint32_t)(q >> 1) & 1u;
      if(!wait_phase(full + s, par)) {
        ok = 0;
        break;
      }
      landed = q + 1;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      unsigned char *Ar = tsm + s * kStage;
      unsigned char *Arh = Ar, *Arl = Ar + kAPart, *Aih = Ar + 2 * kAPart, *Ail = Ar + 3 * kAPart;
      unsigned char *Brh = Ar + kStageA, *Brl = Brh + kBPart, *Bih = Brh + 2 * kBPart,
                    *Bil = Brh + 3 * kBPart;
      for(int st = 0; st < kTcK / 16; ++st) {
        const uint32_t ko = st * 256;  // two core matrices along K per MMA
        auto da = [&](unsigned char *p) { return umma_desc(smem_addr(p) + ko, 128, 512); };
        const uint32_t acc = q > 0 || st > 0;
        // Ar Br
        mma_bf16(d_r1, da(Arh), da(Brh), acc);
        mma_bf16(d_r1, da(Arh), da(Brl), 1);
        mma_bf16(d_r1, da(Arl), da(Brh), 1);
        // Ai Bi
        mma_bf16(d_r2, da(Aih), da(Bih), acc);
        mma_bf16(d_r2, da(Aih), da(Bil), 1);
        mma_bf16(d_r2, da(Ail), da(Bih), 1);
        // Ar Bi + Ai Br
        mma_bf16(d_im, da(Arh), da(Bih), acc);
        mma_bf16(d_im, da(Arh), da(Bil), 1);
        mma_bf16(d_im, da(Arl), da(Bih), 1);
        mma_bf16(d_im, da(Aih), da(Brh), 1);
        mma_bf16(d_im, da(Aih), da(Brl), 1);
        mma_bf16(d_im, da(Ail), da(Brh), 1);
      }
      asm volatile(
          "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
              smem_addr(empty + s))
          : "memory");
      committed = q + 1;
      if(q + 2 < nq) {  // stage s is free once these MMAs have read it
        if(!wait_phase(empty + s, par)) {
          ok = 0;
          break;
        }
        issue(q + 2);
      }
    }
    if(!ok) {  // before leaving: the copies still in flight and the last MMAs (bounded)
      for(int q = landed; q < issued; ++q)
        wait_phase(full + (q & 1), (uint32_t)(q >> 1) & 1u);
      if(committed > 0)
        wait_phase(empty + ((committed - 1) & 1), (uint32_t)((committed - 1) >> 1) & 1u);
    }
  }
  // columns 0 .. 31 of this thread's row of C, loaded while the MMAs run
  const long r = r0 + warp * 32 + lane;
  float2 cv[32];
#pragma unroll
  for(int q = 0; q < 32; ++q) {
    const long col = c0 + q;
    cv[q] = (r < m && col < n) ? C[col * ldc + r] : make_float2(0.f, 0.f);
  }
  // bounded wait for the last chunk's MMAs (they complete after all earlier ones)
  const int last = nq - 1;
  uint32_t done = __syncthreads_and(ok);
  if(done)
    done = wait_phase(empty + (last & 1), (uint32_t)(last >> 1) & 1u);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  done = __syncthreads_and(done);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if(!done) {
    if(t == 0)
      atomicExch(err, 1);
  } else {
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
#pragma unroll
    for(int g = 0; g < kTcN / 16; ++g) {
      const int cc = 16 * g, base = (g & 1) * 16;
      uint32_t a[16], b[16], c[16];
#define OM_TMEM_LD16(dst, addr)                                                                     \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
               : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]),  \
                 "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]),              \
                 "=r"(dst[11]), "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])           \
               : "r"(addr))
      OM_TMEM_LD16(a, d_r1 + lane_base + cc);
      OM_TMEM_LD16(b, d_r2 + lane_base + cc);
      OM_TMEM_LD16(c, d_im + lane_base + cc);
#undef OM_TMEM_LD16
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if(r < m) {
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const long col = c0 + cc + q;
          if(col < n) {
            float2 v = cv[base + q];
            v.x -= __uint_as_float(a[q]) - __uint_as_float(b[q]);
            v.y -= __uint_as_float(c[q]);
            C[col * ldc + r] = v;
          }
        }
      }
      if(g < 2) {
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const long col = c0 + cc + 32 + q;
          cv[base + q] = (r < m && col < n) ? C[col * ldc + r] : make_float2(0.f, 0.f);
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmem2Cols));
  }
}

// ---------------------------------------------------------------------------
// Persistent form of the split-operand update, one CTA per SM. The CTA takes a
// contiguous range of the 128 x 64 tiles in row-tile-major order, so its A
// tiles (all nq <= 4 chunks: up to 128 KB) stay resident in shared memory
// while it walks the column tiles of a row tile; only B's chunks (16 KB) are
// streamed, through a ring of three stages. The roles are split by warp:
//   warps 0-3  epilogue: TMEM lanes 32 w .. 32 w + 31 (rows of the tile), C
//              read from a shared-memory ring, C - AB stored to global;
//   warp 4     operand copies (A when the row tile changes, B chunks);
//   warp 5     TMEM allocation and the MMAs (one elected thread);
//   warp 6     C copies: each tile's columns in groups of 16 (16 KB, one
//              two-dimensional tensor copy) through a ring of three slots.
// The accumulators (Ar Br, Ai Bi, Im: 3 x 64 TMEM columns) are double
// buffered, so the epilogue of one tile runs under the MMAs of the next, and
// the C ring keeps up to 48 KB of C reads in flight per SM. Every wait is
// bounded; a time-out raises *err and a shared abort flag that the other
// roles poll, after which each role waits (bounded) for its own copies and
// MMAs in flight, and the TMEM is freed.
constexpr int kPThreads = 224;
constexpr int kPMaxQ = 4;                      // k <= 128
constexpr int kPBStages = 3, kPCSlots = 3;
constexpr int kPCSlot = 16 * kTcM * 8;         // 16 columns of 128 complex64
constexpr int kPOffB = kPMaxQ * kStageA;       // 128 KB of resident A
constexpr int kPOffC = kPOffB + kPBStages * kStageB;
constexpr int kPOffBar = kPOffC + kPCSlots * kPCSlot;
constexpr int kPSmem = kPOffBar + 256;
constexpr uint32_t kPTmemCols = 512;           // two sets of three 64-column accumulators
static_assert(kPSmem <= 227 * 1024, "persistent update: shared memory");

struct PBars {
  uint64_t a_full, a_empty, drain;
  uint64_t b_full[kPBStages], b_empty[kPBStages];
  uint64_t c_full[kPCSlots], c_empty[kPCSlots];
  uint64_t t_full[2], t_empty[2];
  uint32_t tmem;
  int abort;
};
static_assert(sizeof(PBars) <= 256, "persistent update: barrier block");

__device__ __forceinline__ uint32_t try_phase(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done;
}

// Bounded wait that also gives up when another role has aborted; a time-out
// raises the abort flag and *err.
__device__ __forceinline__ uint32_t pwait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *err) {
  for(long it = 0; it < (1L << 24); ++it) {
    if(try_phase(bar, parity))
      return 1;
    if((it & 63) == 63 && *abort_flag)
      return 0;
  }
  *abort_flag = 1;
  atomicExch(err, 1);
  return 0;
}

__device__ __forceinline__ void arrive1(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                   smem_addr(bar))
               : "memory");
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *tm, int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(tm), "r"(x), "r"(y), "r"(smem_addr(bar))
      : "memory");
}

__global__ void __launch_bounds__(kPThreads, 1)
    k_cgemm_sub_tc3(const unsigned char *As, const unsigned char *Bs, int nq,
                    const __grid_constant__ CUtensorMap cmap, float2 *C, long ldc, long m, long n, int *err) {
  extern __shared__ __align__(1024) unsigned char psm[];
  PBars *bars = reinterpret_cast<PBars *>(psm + kPOffBar);
  volatile int *abort_flag = &bars->abort;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long mt = (m + kTcM - 1) / kTcM, nt = (n + kTcN - 1) / kTcN, T = mt * nt;
  const long t0 = T * blockIdx.x / gridDim.x, t1 = T * (blockIdx.x + 1) / gridDim.x;

  if(warp == 5) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_addr(&bars->tmem)),
                 "r"(kPTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if(t == 0) {
    auto init = [](uint64_t *b, int c) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(c));
    };
    init(&bars->a_full, 1);
    init(&bars->a_empty, 1);
    init(&bars->drain, 1);
    for(int i = 0; i < kPBStages; ++i) {
      init(bars->b_full + i, 1);
      init(bars->b_empty + i, 1);
    }
    for(int i = 0; i < kPCSlots; ++i) {
      init(bars->c_full + i, 1);
      init(bars->c_empty + i, 4);
    }
    for(int i = 0; i < 2; ++i) {
      init(bars->t_full + i, 1);
      init(bars->t_empty + i, 4);
    }
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t tmem = bars->tmem;

  if(warp == 4 && lane == 0) {
    // operand copies
    long prev_rt = -1, bq = 0;
    int a_loads = 0;
    for(long tile = t0; tile < t1 && !*abort_flag; ++tile) {
      const long rt = tile / nt, ct = tile - rt * nt;
      if(rt != prev_rt) {
        if(a_loads > 0 && !pwait(&bars->a_empty, (uint32_t)(a_loads - 1) & 1u, abort_flag, err))
          break;
        arrive_expect(&bars->a_full, (uint32_t)(nq * kStageA));
        for(int q = 0; q < nq; ++q)
          bulk_load(psm + q * kStageA, As + ((size_t)rt * nq + q) * kStageA, (uint32_t)kStageA,
                    &bars->a_full);
        ++a_loads;
        prev_rt = rt;
      }
      bool stop = false;
      for(int q = 0; q < nq; ++q, ++bq) {
        const int s = (int)(bq % kPBStages);
        if(bq >= kPBStages &&
           !pwait(bars->b_empty + s, (uint32_t)(bq / kPBStages - 1) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        arrive_expect(bars->b_full + s, (uint32_t)kStageB);
        bulk_load(psm + kPOffB + s * kStageB, Bs + ((size_t)ct * nq + q) * kStageB, (uint32_t)kStageB,
                  bars->b_full + s);
      }
      if(stop)
        break;
    }
    // the copies still in flight land before the CTA may exit (bounded)
    if(a_loads > 0)
      wait_phase(&bars->a_full, (uint32_t)(a_loads - 1) & 1u);
    for(long q = bq - 1; q >= 0 && q >= bq - kPBStages; --q)
      wait_phase(bars->b_full + q % kPBStages, (uint32_t)(q / kPBStages) & 1u);
  } else if(warp == 5 && lane == 0) {
    // MMAs
    long prev_rt = -1, bq = 0;
    int a_loaded = 0;
    for(long tile = t0, j = 0; tile < t1 && !*abort_flag; ++tile, ++j) {
      const long rt = tile / nt;
      if(rt != prev_rt) {
        if(prev_rt >= 0)
          mma_commit(&bars->a_empty);  // the previous row tile's MMAs have read A
        if(!pwait(&bars->a_full, (uint32_t)a_loaded & 1u, abort_flag, err))
          break;
        ++a_loaded;
        prev_rt = rt;
      }
      const int as = (int)(j & 1);
      if(j >= 2 && !pwait(bars->t_empty + as, (uint32_t)(j / 2 - 1) & 1u, abort_flag, err))
        break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d_r1 = tmem + as * 3 * kTcN, d_r2 = d_r1 + kTcN, d_im = d_r1 + 2 * kTcN;
      bool stop = false;
      for(int q = 0; q < nq; ++q, ++bq) {
        const int s = (int)(bq % kPBStages);
        if(!pwait(bars->b_full + s, (uint32_t)(bq / kPBStages) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        unsigned char *Aq = psm + q * kStageA;
        unsigned char *Arh = Aq, *Arl = Aq + kAPart, *Aih = Aq + 2 * kAPart, *Ail = Aq + 3 * kAPart;
        unsigned char *Brh = psm + kPOffB + s * kStageB, *Brl = Brh + kBPart, *Bih = Brh + 2 * kBPart,
                      *Bil = Brh + 3 * kBPart;
        for(int st = 0; st < kTcK / 16; ++st) {
          const uint32_t ko = st * 256;
          auto da = [&](unsigned char *p) { return umma_desc(smem_addr(p) + ko, 128, 512); };
          const uint32_t acc = q > 0 || st > 0;
          mma_bf16(d_r1, da(Arh), da(Brh), acc);
          mma_bf16(d_r1, da(Arh), da(Brl), 1);
          mma_bf16(d_r1, da(Arl), da(Brh), 1);
          mma_bf16(d_r2, da(Aih), da(Bih), acc);
          mma_bf16(d_r2, da(Aih), da(Bil), 1);
          mma_bf16(d_r2, da(Ail), da(Bih), 1);
          mma_bf16(d_im, da(Arh), da(Bih), acc);
          mma_bf16(d_im, da(Arh), da(Bil), 1);
          mma_bf16(d_im, da(Arl), da(Bih), 1);
          mma_bf16(d_im, da(Aih), da(Brh), 1);
          mma_bf16(d_im, da(Aih), da(Brl), 1);
          mma_bf16(d_im, da(Ail), da(Brh), 1);
        }
        mma_commit(bars->b_empty + s);
      }
      if(stop)
        break;
      mma_commit(bars->t_full + as);
    }
    // every MMA issued has completed before the TMEM is freed (bounded)
    mma_commit(&bars->drain);
    wait_phase(&bars->drain, 0u);
  } else if(warp == 6 && lane == 0) {
    // C copies: a 128 x 16 box per group (rows and columns past C's edge
    // read as zeros and are not used)
    long cq = 0;
    for(long tile = t0; tile < t1 && !*abort_flag; ++tile) {
      const long rt = tile / nt, ct = tile - rt * nt;
      const long r0 = rt * kTcM, c0 = ct * kTcN;
      bool stop = false;
      for(int g = 0; g < kTcN / 16; ++g, ++cq) {
        const int s = (int)(cq % kPCSlots);
        if(cq >= kPCSlots &&
           !pwait(bars->c_empty + s, (uint32_t)(cq / kPCSlots - 1) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        arrive_expect(bars->c_full + s, (uint32_t)kPCSlot);
        tma_load_2d(psm + kPOffC + s * kPCSlot, &cmap, (int)r0, (int)(c0 + 16 * g), bars->c_full + s);
      }
      if(stop)
        break;
    }
    for(long q = cq - 1; q >= 0 && q >= cq - kPCSlots; --q)
      wait_phase(bars->c_full + q % kPCSlots, (uint32_t)(q / kPCSlots) & 1u);
  } else if(warp < 4) {
    // epilogue: thread (warp, lane) owns row 32 warp + lane of each tile
    // (decisions are made per warp: tcgen05.ld needs the whole warp)
    long cq = 0;
    const uint32_t lane_base = (uint32_t)(warp * 32) << 16;
    for(long tile = t0, j = 0; tile < t1; ++tile, ++j) {
      if(__any_sync(0xffffffffu, *abort_flag))
        break;
      const long rt = tile / nt, ct = tile - rt * nt;
      const long r = rt * kTcM + warp * 32 + lane, c0 = ct * kTcN;
      const int as = (int)(j & 1);
      if(!__all_sync(0xffffffffu, pwait(bars->t_full + as, (uint32_t)(j / 2) & 1u, abort_flag, err)))
        break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d_r1 = tmem + lane_base + as * 3 * kTcN, d_r2 = d_r1 + kTcN, d_im = d_r1 + 2 * kTcN;
      bool stop = false;
      for(int g = 0; g < kTcN / 16; ++g, ++cq) {
        const int s = (int)(cq % kPCSlots);
        uint32_t a[16], b[16], c[16];
#define OM_TMEM_LD16(dst, addr)                                                                     \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
               : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]),  \
                 "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]),              \
                 "=r"(dst[11]), "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])           \
               : "r"(addr))
        OM_TMEM_LD16(a, d_r1 + 16 * g);
        OM_TMEM_LD16(b, d_r2 + 16 * g);
        OM_TMEM_LD16(c, d_im + 16 * g);
#undef OM_TMEM_LD16
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if(!__all_sync(0xffffffffu, pwait(bars->c_full + s, (uint32_t)(cq / kPCSlots) & 1u, abort_flag, err))) {
          stop = true;
          break;
        }
        const float2 *cs = reinterpret_cast<const float2 *>(psm + kPOffC + s * kPCSlot) + warp * 32 + lane;
        if(r < m) {
#pragma unroll
          for(int q = 0; q < 16; ++q) {
            const long col = c0 + 16 * g + q;
            if(col < n) {
              float2 v = cs[q * kTcM];
              v.x -= __uint_as_float(a[q]) - __uint_as_float(b[q]);
              v.y -= __uint_as_float(c[q]);
              C[col * ldc + r] = v;
            }
          }
        }
        __syncwarp();
        if(lane == 0)
          arrive1(bars->c_empty + s);
      }
      if(stop)
        break;
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncwarp();
      if(lane == 0)
        arrive1(bars->t_empty + as);
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if(warp == 5) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPTmemCols));
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

size_t cgemm_sub_tc_split_bytes(long m, long n, int k) {
  const size_t nq = (size_t)((k + kTcK - 1) / kTcK);
  return (size_t)((m + kTcM - 1) / kTcM) * nq * kStageA + (size_t)((n + kTcN - 1) / kTcN) * nq * kStageB;
}

void launch_cgemm_sub_tc_split(om_context *ctx, const float2 *A, long lda, const float2 *B, long ldb,
                               float2 *C, long ldc, long m, long n, int k, void *scratch, int *d_err) {
  const int nq = (k + kTcK - 1) / kTcK;
  const unsigned mt = (unsigned)((m + kTcM - 1) / kTcM), nt = (unsigned)((n + kTcN - 1) / kTcN);
  unsigned char *As = static_cast<unsigned char *>(scratch);
  unsigned char *Bs = As + (size_t)mt * nq * kStageA;
  k_tc_split_a<<<dim3(mt, (unsigned)nq), 512, 0, ctx->stream>>>(A, lda, m, k, nq, As);
  k_tc_split_b<<<dim3(nt, (unsigned)nq), 256, 0, ctx->stream>>>(B, ldb, n, k, nq, Bs);
  // the persistent form reads C by tensor copies: a 16-byte aligned base and
  // an even leading dimension (column stride a multiple of 16 bytes)
  alignas(64) CUtensorMap cmap;
  bool persistent = ctx->lu_tc == 1 && nq <= kPMaxQ && (reinterpret_cast<uintptr_t>(C) & 15) == 0 &&
                    (ldc & 1) == 0;
  if(persistent) {
    typedef CUresult (*EncodeFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                 CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                 CUtensorMapFloatOOBfill);
    EncodeFn enc = reinterpret_cast<EncodeFn>(tensor_map_encoder());
    const cuuint64_t dims[2] = {(cuuint64_t)m, (cuuint64_t)n};
    const cuuint64_t strides[1] = {(cuuint64_t)ldc * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)kTcM, 16};
    const cuuint32_t estr[2] = {1, 1};
    persistent = enc && enc(&cmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, C, dims, strides, box, estr,
                            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  if(persistent) {
    cudaFuncSetAttribute(k_cgemm_sub_tc3, cudaFuncAttributeMaxDynamicSharedMemorySize, kPSmem);
    const long tiles = (long)mt * nt;
    const unsigned grid = (unsigned)std::min<long>(tiles, ctx->sm_count);
    k_cgemm_sub_tc3<<<grid, kPThreads, kPSmem, ctx->stream>>>(As, Bs, nq, cmap, C, ldc, m, n, d_err);
  } else {
    cudaFuncSetAttribute(k_cgemm_sub_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, kTc2Smem);
    k_cgemm_sub_tc2<<<dim3(mt, nt), 128, kTc2Smem, ctx->stream>>>(As, Bs, nq, C, ldc, m, n, d_err);
  }
  ctx->last_launches += 3;
}

}  // namespace om
