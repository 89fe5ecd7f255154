// Complex64 rank-k update on the 5th-generation tensor cores (tcgen05):
//   C (m x n) -= A (m x k) B (k x n),  any k >= 1, column-major complex64,
// the trailing updates of the precision form's blocked LU (the role of the
// pzgesv trailing pzgemm, ScalapackSolver.cpp:54-130 / LinearSystemSolver.hpp:55-65).
//
// The operands are split once into fp16 hi / lo parts of power-of-two scaled
// rows (A) and columns (B) (k_tc_split_a/b), laid out as the tensor cores'
// shared-memory operand tiles: K-major, no swizzle, 8 x 16-byte core
// matrices. A real product is hi hi + hi lo + lo hi (FP32 accumulation in
// TMEM), and B's tile holds its parts in the order -Bi, Br, Bi (hi, then lo),
// so that [Br | Bi] and [-Bi | Br] are each one 128-row operand: with
//   Re + i Im = Ar [Br | Bi] + Ai [-Bi | Br]
// the 128 x 64 tile of C takes 6 MMAs of M = 128, N = 128, K = 16 per 16
// columns of k into one 128-column accumulator (Re, Im side by side): half
// the MMAs, and a third less shared-memory operand traffic, than separate
// 64-column products. Two update kernels share the layout and the epilogue
// arithmetic, so they give the same bits: k_cgemm_sub_tc2, one CTA per
// 128 x 64 tile of C, and k_cgemm_sub_tc3, one persistent CTA per SM with its
// row tile's A resident and the roles split by warp.
#include <algorithm>

#include <cuda.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "om_internal.h"

namespace om {

namespace {

constexpr int kTcM = 128, kTcN = 64, kTcK = 32;
// shared-memory operand tiles (fp16): A parts 128 x 32 (Ar, Ai: hi and lo),
// B parts 64 x 32 (-Bi, Br, Bi: hi, then lo)
constexpr int kAPart = kTcM * kTcK * 2, kBPart = kTcN * kTcK * 2;

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

// Instruction descriptor, kind::f16: D F32, A and B F16, both K-major (the
// pre-split operands below).
constexpr uint32_t kIdescF16 = (1u << 4) | ((uint32_t)((2 * kTcN) >> 3) << 17) | ((uint32_t)(kTcM >> 4) << 24);

__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(adesc), "l"(bdesc), "r"(kIdescF16), "r"(acc));
}

// The 12 MMAs (N = 128) of one 32-column chunk of k (two K-steps of 16) into
// the accumulator d (Re: columns 0-63, Im: 64-127), from the chunk's operand
// tiles at shared addresses a (Arh, Arl, Aih, Ail, kAPart bytes apart) and b
// (-Bih, Brh, Bih, -Bil, Brl, Bil, kBPart apart). A descriptor is a fixed
// template plus the address / 16: the address field takes the low 14 bits and
// cannot carry into the next field below 256 KB, so the issuing thread spends
// one add per operand.
constexpr int kAPartB = kTcM * kTcK * 2, kBPartB = kTcN * kTcK * 2;  // (= kAPart, kBPart)
__device__ __forceinline__ void mma_chunk(uint32_t d, uint32_t a, uint32_t b, bool first) {
  const uint64_t tmpl = umma_desc(0, 128, 512);
  constexpr uint32_t dA = kAPartB >> 4, dB = kBPartB >> 4;
#pragma unroll
  for(int st = 0; st < kTcK / 16; ++st) {
    const uint64_t A0 = tmpl + ((a >> 4) + 16u * st), B0 = tmpl + ((b >> 4) + 16u * st);
    const uint64_t Arh = A0, Arl = A0 + dA, Aih = A0 + 2 * dA, Ail = A0 + 3 * dA;
    const uint64_t NBh = B0, BRh = B0 + dB, NBl = B0 + 3 * dB, BRl = B0 + 4 * dB;  // [-Bi | Br], [Br | Bi]
    const uint32_t acc = !first || st > 0;
    mma_f16(d, Arh, BRh, acc);  // Ar [Br | Bi]
    mma_f16(d, Arh, BRl, 1);
    mma_f16(d, Arl, BRh, 1);
    mma_f16(d, Aih, NBh, 1);    // Ai [-Bi | Br]
    mma_f16(d, Aih, NBl, 1);
    mma_f16(d, Ail, NBh, 1);
  }
}

// byte offset of element (row r, k index c) in a K-major no-swizzle tile with
// 32 columns of K: core matrices of 8 rows x 8 fp16, K-adjacent ones 128 B
// apart (LBO), row-adjacent ones 512 B apart (SBO)
__device__ __forceinline__ int kmajor_off(int r, int c) {
  return (r >> 3) * 512 + (c >> 3) * 128 + (r & 7) * 16 + (c & 7) * 2;
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

// --- pre-split operands, streamed by bulk copies --------------------------
//
// For the LU's trailing updates the operands are split once, before the
// update, into fp16 hi / lo parts of power-of-two scaled values: each row of
// L21 (m x k) is scaled by sa = 2^e so that its largest component lies in
// [2^14, 2^15), each column of U12 (k x n) likewise by sb, and x sa = hi + lo
// with hi = fp16(x sa), lo = fp16(x sa - hi). The scaled values keep 22
// significant bits (11 in each part); lo stays a normal fp16 number for every
// entry within 2^-17 of its row's (column's) largest, and below that its
// absolute error is under 2^-39 of the largest. A real product is
// hi hi + hi lo + lo hi (three MMAs, FP32 accumulation), so the update carries
// about 21 significant bits relative to the rows' and columns' magnitudes,
// against about 17 for bf16 parts without scaling. The epilogue takes the
// accumulators times 1 / (sa sb), exactly (powers of two). The parts are laid
// out exactly as the shared-memory tiles above (per 128-row tile of A or
// 64-column tile of B and per 32-column chunk of k: the parts one after
// another, each in the K-major core-matrix layout), followed by the inverse
// scales (float per row of A, then per column of B). The update kernels copy
// each chunk's tiles with one-dimensional bulk copies (cp.async.bulk,
// completion counted on an mbarrier), so that no thread converts or stores
// operands in the loop. The real part is kept as two accumulators (Ar Br and
// Ai Bi, subtracted in the epilogue) instead of staging -Bi.
constexpr int kStageA = 4 * kAPart, kStageB = 6 * kBPart, kStage = kStageA + kStageB;
constexpr int kTc2Smem = 2 * kStage + 128;
constexpr uint32_t kTmem2Cols = 128;  // one 128-column accumulator (Re, Im)

// Two scaled FP32 values split into fp16 hi and lo parts, packed as half2
// (the first value in the low half).
__device__ __forceinline__ void split2_f16(float a, float b, uint32_t &hi, uint32_t &lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 hf = __half22float2(h);
  const __half2 l = __floats2half2_rn(a - hf.x, b - hf.y);
  hi = *reinterpret_cast<const uint32_t *>(&h);
  lo = *reinterpret_cast<const uint32_t *>(&l);
}

// 2^e with max |x| 2^e in [2^14, 2^15) (1 for a zero row or column)
__device__ __forceinline__ float split_scale(float amax) {
  if(!(amax > 0.f))
    return 1.f;
  int e;
  frexpf(amax, &e);  // amax = f 2^e, f in [0.5, 1)
  return ldexpf(1.f, 15 - e);
}

// A (m x k, lda) -> per (row tile, chunk): Arh, Arl, Aih, Ail (8 KB each),
// and 1 / sa per row (inv_a). One CTA of 512 threads per row tile: thread t
// takes row t % 128 and, in every chunk, the K columns 8 (t / 128) ..
// 8 (t / 128) + 7; a first pass finds the row's largest component.
__global__ void __launch_bounds__(512) k_tc_split_a(const float2 *A, long lda, long m, int k, int nq,
                                                    unsigned char *out, float *inv_a) {
  __shared__ float part_max[4][kTcM];
  __shared__ float scale_s[kTcM];
  const int t = threadIdx.x, r = t & 127, g = t >> 7;
  const long row = (long)blockIdx.x * kTcM + r;
  float amax = 0.f;
  for(int q = 0; q < nq; ++q) {
    const int k0 = q * kTcK + 8 * g;
#pragma unroll
    for(int j = 0; j < 8; ++j)
      if(row < m && k0 + j < k) {
        const float2 v = A[(long)(k0 + j) * lda + row];
        amax = fmaxf(amax, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
  }
  part_max[g][r] = amax;
  __syncthreads();
  if(g == 0) {
    const float sc = split_scale(fmaxf(fmaxf(part_max[0][r], part_max[1][r]), fmaxf(part_max[2][r], part_max[3][r])));
    scale_s[r] = sc;
    if(row < m)
      inv_a[row] = 1.f / sc;
  }
  __syncthreads();
  const float sc = scale_s[r];
  for(int q = 0; q < nq; ++q) {
    const int k0 = q * kTcK + 8 * g;
    float2 v[8];
#pragma unroll
    for(int j = 0; j < 8; ++j) {
      v[j] = (row < m && k0 + j < k) ? A[(long)(k0 + j) * lda + row] : make_float2(0.f, 0.f);
      v[j].x *= sc;
      v[j].y *= sc;
    }
    uint32_t a[4], b[4], c[4], d[4];
#pragma unroll
    for(int p = 0; p < 4; ++p) {
      split2_f16(v[2 * p].x, v[2 * p + 1].x, a[p], b[p]);
      split2_f16(v[2 * p].y, v[2 * p + 1].y, c[p], d[p]);
    }
    unsigned char *o = out + ((size_t)blockIdx.x * nq + q) * kStageA + kmajor_off(r, 8 * g);
    *reinterpret_cast<uint4 *>(o) = make_uint4(a[0], a[1], a[2], a[3]);
    *reinterpret_cast<uint4 *>(o + kAPart) = make_uint4(b[0], b[1], b[2], b[3]);
    *reinterpret_cast<uint4 *>(o + 2 * kAPart) = make_uint4(c[0], c[1], c[2], c[3]);
    *reinterpret_cast<uint4 *>(o + 3 * kAPart) = make_uint4(d[0], d[1], d[2], d[3]);
  }
}

// B (k x n, ldb) -> per (column tile, chunk): Brh, Brl, Bih, Bil (4 KB each),
// as N x K, and 1 / sb per column (inv_b). One CTA of 256 threads per column
// tile: thread t takes column t % 64 and, in every chunk, the K rows
// 8 (t / 64) .. 8 (t / 64) + 7.
__global__ void __launch_bounds__(256) k_tc_split_b(const float2 *B, long ldb, long n, int k, int nq,
                                                    unsigned char *out, float *inv_b) {
  __shared__ float part_max[4][kTcN];
  __shared__ float scale_s[kTcN];
  const int t = threadIdx.x, j = t & 63, g = t >> 6;
  const long col = (long)blockIdx.x * kTcN + j;
  float amax = 0.f;
  for(int q = 0; q < nq; ++q) {
    const int k0 = q * kTcK + 8 * g;
#pragma unroll
    for(int i = 0; i < 8; ++i)
      if(col < n && k0 + i < k) {
        const float2 v = B[col * ldb + k0 + i];
        amax = fmaxf(amax, fmaxf(fabsf(v.x), fabsf(v.y)));
      }
  }
  part_max[g][j] = amax;
  __syncthreads();
  if(g == 0) {
    const float sc = split_scale(fmaxf(fmaxf(part_max[0][j], part_max[1][j]), fmaxf(part_max[2][j], part_max[3][j])));
    scale_s[j] = sc;
    if(col < n)
      inv_b[col] = 1.f / sc;
  }
  __syncthreads();
  const float sc = scale_s[j];
  for(int q = 0; q < nq; ++q) {
    const int k0 = q * kTcK + 8 * g;
    float2 v[8];
#pragma unroll
    for(int i = 0; i < 8; ++i) {
      v[i] = (col < n && k0 + i < k) ? B[col * ldb + k0 + i] : make_float2(0.f, 0.f);
      v[i].x *= sc;
      v[i].y *= sc;
    }
    uint32_t a[4], b[4], c[4], d[4];
#pragma unroll
    for(int p = 0; p < 4; ++p) {
      split2_f16(v[2 * p].x, v[2 * p + 1].x, a[p], b[p]);
      split2_f16(v[2 * p].y, v[2 * p + 1].y, c[p], d[p]);
    }
    // parts -Bih, Brh, Bih, -Bil, Brl, Bil (a sign flip is exact in fp16)
    constexpr uint32_t sgn = 0x80008000u;
    unsigned char *o = out + ((size_t)blockIdx.x * nq + q) * kStageB + kmajor_off(j, 8 * g);
    *reinterpret_cast<uint4 *>(o) = make_uint4(c[0] ^ sgn, c[1] ^ sgn, c[2] ^ sgn, c[3] ^ sgn);
    *reinterpret_cast<uint4 *>(o + kBPart) = make_uint4(a[0], a[1], a[2], a[3]);
    *reinterpret_cast<uint4 *>(o + 2 * kBPart) = make_uint4(c[0], c[1], c[2], c[3]);
    *reinterpret_cast<uint4 *>(o + 3 * kBPart) = make_uint4(d[0] ^ sgn, d[1] ^ sgn, d[2] ^ sgn, d[3] ^ sgn);
    *reinterpret_cast<uint4 *>(o + 4 * kBPart) = make_uint4(b[0], b[1], b[2], b[3]);
    *reinterpret_cast<uint4 *>(o + 5 * kBPart) = make_uint4(d[0], d[1], d[2], d[3]);
  }
}

// C entry minus the unscaled accumulators (re, im) / (sa sb), with the
// inverse scales applied one after the other (each product exact unless the
// result itself leaves FP32's range) and every operation written out, so that
// both update kernels round alike.
__device__ __forceinline__ float2 unscale_sub(float2 v, uint32_t re, uint32_t im, float sa, float sb) {
  const float rv = __fmul_rn(__fmul_rn(__uint_as_float(re), sa), sb);
  const float iv = __fmul_rn(__fmul_rn(__uint_as_float(im), sa), sb);
  return make_float2(__fsub_rn(v.x, rv), __fsub_rn(v.y, iv));
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
                                                       const float *inv_a, const float *inv_b, int nq,
                                                       float2 *C, long ldc, long m, long n, int *err) {
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
  const uint32_t d_re = tmem, d_im = tmem + kTcN;

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
      mma_chunk(d_re, smem_addr(tsm + s * kStage), smem_addr(tsm + s * kStage + kStageA), q == 0);
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
  const float sa = r < m ? inv_a[r] : 0.f;
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
      uint32_t a[16], c[16];
#define OM_TMEM_LD16(dst, addr)                                                                     \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
               : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]),  \
                 "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]),              \
                 "=r"(dst[11]), "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])           \
               : "r"(addr))
      OM_TMEM_LD16(a, d_re + lane_base + cc);
      OM_TMEM_LD16(c, d_im + lane_base + cc);
#undef OM_TMEM_LD16
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      {
        const long lcol = c0 + cc + (lane & 15);
        const float sbl = lcol < n ? inv_b[lcol] : 0.f;
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const float sb = __shfl_sync(0xffffffffu, sbl, q);
          const long col = c0 + cc + q;
          if(r < m && col < n)
            C[col * ldc + r] = unscale_sub(cv[base + q], a[q], c[q], sa, sb);
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
// while it walks the column tiles of a row tile; only B's chunks (24 KB) are
// streamed, through a ring of two stages. The roles are split by warp:
//   warps 0-3  epilogue: TMEM lanes 32 w .. 32 w + 31 (rows of the tile), C
//              read from a shared-memory ring, C - AB stored to global (one
//              consumer group, so that the ring's slots are consumed in the
//              order they are filled: a second group working ahead on other
//              columns could see a slot's previous fill as its own, since an
//              mbarrier's phase parity only tells two phases apart);
//   warp 4     operand copies (A when the row tile changes, B chunks);
//   warp 5     TMEM allocation and the MMAs (one elected thread);
//   warp 6     C copies: each tile's columns in groups of 16 (16 KB, one
//              two-dimensional tensor copy) through a ring of three slots.
// The accumulator (Re, Im: 2 x 64 TMEM columns) is double
// buffered, so the epilogue of one tile runs under the MMAs of the next, and
// the C ring keeps up to 48 KB of C reads in flight per SM. Every wait is
// bounded; a time-out raises *err and a shared abort flag that the other
// roles poll, after which each role waits (bounded) for its own copies and
// MMAs in flight, and the TMEM is freed.
constexpr int kPThreads = 224;
constexpr int kPProd = 4, kPMma = 5, kPCLoad = 6;  // the warps' roles (0-3: epilogue)
constexpr int kPMaxQ = 4;                      // k <= 128 with A resident
constexpr int kPBStages = 3, kPCSlots = 3;     // (stages: 2 with A resident, 3 streaming A)
constexpr int kPCAhead = 2;                    // C tiles requested into L2 ahead of the ring
constexpr int kPCSlot = 16 * kTcM * 8;         // 16 columns of 128 complex64
// Shared-memory layout: with A resident (k <= 128), 128 KB of A, then two
// stages of B chunks (24 KB); for larger k, three stages of an A chunk and a
// B chunk (56 KB) each. Then the C ring and the barriers.
template <bool kResA> struct PLayout {
  static constexpr int stages = kResA ? 2 : 3;
  static constexpr int offB = kResA ? kPMaxQ * kStageA : 0;
  static constexpr int stage = kResA ? kStageB : kStageA + kStageB;
  static constexpr int offC = offB + stages * stage;
  static constexpr int offBar = offC + kPCSlots * kPCSlot;
  static constexpr int smem = offBar + 256;
};
static_assert(PLayout<true>::smem <= 227 * 1024 && PLayout<false>::smem <= 227 * 1024,
              "persistent update: shared memory");
constexpr uint32_t kPTmemCols = 256;           // two 128-column accumulators (Re, Im)

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

__device__ __forceinline__ void tma_prefetch_l2(const CUtensorMap *tm, int x, int y) {
  asm volatile("cp.async.bulk.prefetch.tensor.2d.L2.global.tile [%0, {%1, %2}];" ::"l"(tm), "r"(x), "r"(y)
               : "memory");
}

template <bool kResA>
__global__ void __launch_bounds__(kPThreads, 1)
    k_cgemm_sub_tc3(const unsigned char *As, const unsigned char *Bs, const float *inv_a, const float *inv_b,
                    int nq, const __grid_constant__ CUtensorMap cmap, float2 *C, long ldc, long m, long n,
                    int *err) {
  extern __shared__ __align__(1024) unsigned char psm[];
  typedef PLayout<kResA> L;
  PBars *bars = reinterpret_cast<PBars *>(psm + L::offBar);
  volatile int *abort_flag = &bars->abort;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const long mt = (m + kTcM - 1) / kTcM, nt = (n + kTcN - 1) / kTcN, T = mt * nt;
  const long t0 = T * blockIdx.x / gridDim.x, t1 = T * (blockIdx.x + 1) / gridDim.x;

  if(warp == kPMma) {
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
    for(int i = 0; i < L::stages; ++i) {
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

  if(warp == kPProd && lane == 0) {
    // operand copies
    long prev_rt = -1, bq = 0;
    int a_loads = 0;
    for(long tile = t0; tile < t1 && !*abort_flag; ++tile) {
      const long rt = tile / nt, ct = tile - rt * nt;
      if(kResA && rt != prev_rt) {
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
        const int s = (int)(bq % L::stages);
        if(bq >= L::stages &&
           !pwait(bars->b_empty + s, (uint32_t)(bq / L::stages - 1) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        unsigned char *dst = psm + L::offB + s * L::stage;
        if(kResA) {
          arrive_expect(bars->b_full + s, (uint32_t)kStageB);
        } else {  // the A chunk too, ahead of B in the stage
          arrive_expect(bars->b_full + s, (uint32_t)(kStageA + kStageB));
          bulk_load(dst, As + ((size_t)rt * nq + q) * kStageA, (uint32_t)kStageA, bars->b_full + s);
          dst += kStageA;
        }
        bulk_load(dst, Bs + ((size_t)ct * nq + q) * kStageB, (uint32_t)kStageB, bars->b_full + s);
      }
      if(stop)
        break;
    }
    // the copies still in flight land before the CTA may exit (bounded)
    if(a_loads > 0)
      wait_phase(&bars->a_full, (uint32_t)(a_loads - 1) & 1u);
    for(long q = bq - 1; q >= 0 && q >= bq - L::stages; --q)
      wait_phase(bars->b_full + q % L::stages, (uint32_t)(q / L::stages) & 1u);
  } else if(warp == kPMma && lane == 0) {
    // MMAs
    long prev_rt = -1, bq = 0;
    int a_loaded = 0;
    for(long tile = t0, j = 0; tile < t1 && !*abort_flag; ++tile, ++j) {
      const long rt = tile / nt;
      if(kResA && rt != prev_rt) {
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
      const uint32_t d_acc = tmem + as * 2 * kTcN;
      bool stop = false;
      for(int q = 0; q < nq; ++q, ++bq) {
        const int s = (int)(bq % L::stages);
        if(!pwait(bars->b_full + s, (uint32_t)(bq / L::stages) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t stg = smem_addr(psm + L::offB + s * L::stage);
        if(kResA)
          mma_chunk(d_acc, smem_addr(psm + q * kStageA), stg, q == 0);
        else
          mma_chunk(d_acc, stg, stg + kStageA, q == 0);
        mma_commit(bars->b_empty + s);
      }
      if(stop)
        break;
      mma_commit(bars->t_full + as);
    }
    // every MMA issued has completed before the TMEM is freed (bounded)
    mma_commit(&bars->drain);
    wait_phase(&bars->drain, 0u);
  } else if(warp == kPCLoad && lane == 0) {
    // C copies: a 128 x 16 box per group (rows and columns past C's edge
    // read as zeros and are not used). The tiles kPCAhead ahead are requested
    // into L2 first, so that the shared-memory ring (three quarters of a
    // tile) refills from L2 and the DRAM reads run ahead of the epilogue.
    long cq = 0;
    auto prefetch_tile = [&](long tile) {
      const long rt = tile / nt, ct = tile - rt * nt;
      for(int g = 0; g < kTcN / 16; ++g)
        if(ct * kTcN + 16 * g < n)
          tma_prefetch_l2(&cmap, (int)(rt * kTcM), (int)(ct * kTcN + 16 * g));
    };
    for(long tile = t0; tile < t1 && tile < t0 + kPCAhead; ++tile)
      prefetch_tile(tile);
    for(long tile = t0; tile < t1 && !*abort_flag; ++tile) {
      const long rt = tile / nt, ct = tile - rt * nt;
      const long r0 = rt * kTcM, c0 = ct * kTcN;
      if(tile + kPCAhead < t1)
        prefetch_tile(tile + kPCAhead);
      bool stop = false;
      for(int g = 0; g < kTcN / 16; ++g, ++cq) {
        const int s = (int)(cq % kPCSlots);
        if(cq >= kPCSlots &&
           !pwait(bars->c_empty + s, (uint32_t)(cq / kPCSlots - 1) & 1u, abort_flag, err)) {
          stop = true;
          break;
        }
        arrive_expect(bars->c_full + s, (uint32_t)kPCSlot);
        tma_load_2d(psm + L::offC + s * kPCSlot, &cmap, (int)r0, (int)(c0 + 16 * g), bars->c_full + s);
      }
      if(stop)
        break;
    }
    for(long q = cq - 1; q >= 0 && q >= cq - kPCSlots; --q)
      wait_phase(bars->c_full + q % kPCSlots, (uint32_t)(q / kPCSlots) & 1u);
  } else if(warp < 4) {
    // epilogue: thread (warp, lane) owns row 32 warp + lane of each tile
    // (decisions are made per warp: tcgen05.ld needs the whole warp)
    const int quarter = warp;
    const uint32_t lane_base = (uint32_t)(quarter * 32) << 16;
    for(long tile = t0, j = 0; tile < t1; ++tile, ++j) {
      if(__any_sync(0xffffffffu, *abort_flag))
        break;
      const long rt = tile / nt, ct = tile - rt * nt;
      const long r = rt * kTcM + quarter * 32 + lane, c0 = ct * kTcN;
      const int as = (int)(j & 1);
      if(!__all_sync(0xffffffffu, pwait(bars->t_full + as, (uint32_t)(j / 2) & 1u, abort_flag, err)))
        break;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t d_re = tmem + lane_base + as * 2 * kTcN, d_im = d_re + kTcN;
      const float sa = r < m ? inv_a[r] : 0.f;
      bool stop = false;
      for(int g = 0; g < kTcN / 16; ++g) {
        const long cq = 4 * j + g;  // the C loader's group counter
        const int s = (int)(cq % kPCSlots);
        uint32_t a[16], c[16];
#define OM_TMEM_LD16(dst, addr)                                                                     \
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];" \
               : "=r"(dst[0]), "=r"(dst[1]), "=r"(dst[2]), "=r"(dst[3]), "=r"(dst[4]), "=r"(dst[5]),  \
                 "=r"(dst[6]), "=r"(dst[7]), "=r"(dst[8]), "=r"(dst[9]), "=r"(dst[10]),              \
                 "=r"(dst[11]), "=r"(dst[12]), "=r"(dst[13]), "=r"(dst[14]), "=r"(dst[15])           \
               : "r"(addr))
        OM_TMEM_LD16(a, d_re + 16 * g);
        OM_TMEM_LD16(c, d_im + 16 * g);
#undef OM_TMEM_LD16
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if(!__all_sync(0xffffffffu, pwait(bars->c_full + s, (uint32_t)(cq / kPCSlots) & 1u, abort_flag, err))) {
          stop = true;
          break;
        }
        const float2 *cs = reinterpret_cast<const float2 *>(psm + L::offC + s * kPCSlot) + quarter * 32 + lane;
        // the group's 16 column scales: lane q % 16 loads column q's, shuffled
        const long lcol = c0 + 16 * g + (lane & 15);
        const float sbl = lcol < n ? inv_b[lcol] : 0.f;
#pragma unroll
        for(int q = 0; q < 16; ++q) {
          const float sb = __shfl_sync(0xffffffffu, sbl, q);
          const long col = c0 + 16 * g + q;
          if(r < m && col < n)
            C[col * ldc + r] = unscale_sub(cs[q * kTcM], a[q], c[q], sa, sb);
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
  if(warp == kPMma) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kPTmemCols));
  }
}

}  // namespace

size_t cgemm_sub_tc_split_bytes(long m, long n, int k) {
  const size_t nq = (size_t)((k + kTcK - 1) / kTcK);
  const size_t mt = (size_t)((m + kTcM - 1) / kTcM), nt = (size_t)((n + kTcN - 1) / kTcN);
  return mt * nq * kStageA + nt * nq * kStageB + sizeof(float) * (mt * kTcM + nt * kTcN);
}

void launch_cgemm_sub_tc_split(om_context *ctx, const float2 *A, long lda, const float2 *B, long ldb,
                               float2 *C, long ldc, long m, long n, int k, void *scratch, int *d_err) {
  const int nq = (k + kTcK - 1) / kTcK;
  const unsigned mt = (unsigned)((m + kTcM - 1) / kTcM), nt = (unsigned)((n + kTcN - 1) / kTcN);
  unsigned char *As = static_cast<unsigned char *>(scratch);
  unsigned char *Bs = As + (size_t)mt * nq * kStageA;
  float *inv_a = reinterpret_cast<float *>(Bs + (size_t)nt * nq * kStageB);
  float *inv_b = inv_a + (size_t)mt * kTcM;
  k_tc_split_a<<<mt, 512, 0, ctx->stream>>>(A, lda, m, k, nq, As, inv_a);
  k_tc_split_b<<<nt, 256, 0, ctx->stream>>>(B, ldb, n, k, nq, Bs, inv_b);
  // the persistent form reads C by tensor copies: a 16-byte aligned base and
  // an even leading dimension (column stride a multiple of 16 bytes)
  alignas(64) CUtensorMap cmap;
  // (lu_tc 3: the one-CTA-per-tile kernel for the rank-32 in-block and U12
  // updates, whose few MMA steps per tile leave the persistent kernel waiting
  // on its C ring; the same bits either way)
  bool persistent = (ctx->lu_tc == 1 || (ctx->lu_tc == 3 && k > 64)) &&
                    (reinterpret_cast<uintptr_t>(C) & 15) == 0 && (ldc & 1) == 0;
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
    const long tiles = (long)mt * nt;
    const unsigned grid = (unsigned)std::min<long>(tiles, ctx->sm_count);
    if(nq <= kPMaxQ) {  // A resident
      cudaFuncSetAttribute(k_cgemm_sub_tc3<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           PLayout<true>::smem);
      k_cgemm_sub_tc3<true><<<grid, kPThreads, PLayout<true>::smem, ctx->stream>>>(As, Bs, inv_a, inv_b, nq,
                                                                                   cmap, C, ldc, m, n, d_err);
    } else {  // A streamed with B
      cudaFuncSetAttribute(k_cgemm_sub_tc3<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           PLayout<false>::smem);
      k_cgemm_sub_tc3<false><<<grid, kPThreads, PLayout<false>::smem, ctx->stream>>>(
          As, Bs, inv_a, inv_b, nq, cmap, C, ldc, m, n, d_err);
    }
  } else {
    cudaFuncSetAttribute(k_cgemm_sub_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize, kTc2Smem);
    k_cgemm_sub_tc2<<<dim3(mt, nt), 128, kTc2Smem, ctx->stream>>>(As, Bs, inv_a, inv_b, nq, C, ldc, m, n,
                                                                  d_err);
  }
  ctx->last_launches += 3;
}

}  // namespace om
