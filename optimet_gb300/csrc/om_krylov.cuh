// Complex arithmetic and the per-row matrix-vector sums shared by the Krylov
// solvers (solve.cu) and the batched solvers (batch.cu). Both call the same
// inline functions, so a row's sum is formed in the same order, and rounds the
// same, whichever solver runs it.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace om {

// An entry of the precision form's bf16 copy of a complex64 matrix (the inner
// FP32 GMRES reads it): the real part rounded to bf16 in the low 16 bits, the
// imaginary part in the high 16 bits. bf16 is the high half of an FP32 word,
// so each part unpacks by one bit operation.
struct Bf16c {
  unsigned v;
};
__device__ __forceinline__ Bf16c pack_bf16c(float2 a) {  // round to nearest even
  const unsigned re = __bfloat16_as_ushort(__float2bfloat16_rn(a.x));
  const unsigned im = __bfloat16_as_ushort(__float2bfloat16_rn(a.y));
  return Bf16c{re | (im << 16)};
}

// An entry of the batching form's fp16 copy of a complex64 matrix: both parts
// as fp16 after the entry's column in its 256-row block was scaled by a power
// of two (the block column's largest part lands in [2^14, 2^15)); the
// products take x times that scale's inverse, so that h (x d) = (h d) x with d
// exact.
struct F16c {
  __half2 v;
};

// a matrix entry as the vector type of a product
template <typename V, typename M> __device__ __forceinline__ V mv_entry(const M &s) {
  V a;
  a.x = s.x;
  a.y = s.y;
  return a;
}
template <> __device__ __forceinline__ float2 mv_entry<float2, F16c>(const F16c &s) {
  return __half22float2(s.v);
}
template <> __device__ __forceinline__ float2 mv_entry<float2, Bf16c>(const Bf16c &s) {
  return make_float2(__uint_as_float(s.v << 16), __uint_as_float(s.v & 0xffff0000u));
}

template <typename V> __device__ __forceinline__ V cfma(V a, V b, V c) {  // c + a*b
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(-a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(a.y, b.x, c.y);
  return c;
}
template <typename V> __device__ __forceinline__ V cfma_conj(V a, V b, V c) {  // c + conj(a)*b
  c.x = fma(a.x, b.x, c.x);
  c.x = fma(a.y, b.y, c.x);
  c.y = fma(a.x, b.y, c.y);
  c.y = fma(-a.y, b.x, c.y);
  return c;
}

// sum_{j0 <= j < j1} S[(j - j0) ld] xs[j - j0] for the row that `col` points
// into (xs: the column chunk j0 .. j1 - 1 staged in shared memory). Eight
// columns' loads are issued before their FMAs; two accumulators take
// alternate columns.
template <typename M, typename V>
__device__ __forceinline__ V mv_row(const M *col, long ld, const V *xs, long j0, long j1) {
  V acc0, acc1;
  acc0.x = acc0.y = acc1.x = acc1.y = 0;
  long j = j0;
  for(; j + 7 < j1; j += 8) {
    M s[8];
#pragma unroll
    for(int u = 0; u < 8; ++u)
      s[u] = col[u * ld];
#pragma unroll
    for(int u = 0; u < 8; u += 2) {
      const V a0 = mv_entry<V>(s[u]), a1 = mv_entry<V>(s[u + 1]);
      acc0 = cfma(a0, xs[j - j0 + u], acc0);
      acc1 = cfma(a1, xs[j - j0 + u + 1], acc1);
    }
    col += 8 * ld;
  }
  for(; j < j1; ++j) {
    const V a0 = mv_entry<V>(col[0]);
    acc0 = cfma(a0, xs[j - j0], acc0);
    col += ld;
  }
  acc0.x += acc1.x;
  acc0.y += acc1.y;
  return acc0;
}

// mv_row on a complex64 row that also writes the row's entries into the bf16
// copy (`copy` points at this row's entry of column j0, ld ldc)
__device__ __forceinline__ float2 mv_row_copy(const float2 *col, long ld, const float2 *xs, long j0, long j1,
                                              Bf16c *copy, long ldc) {
  float2 acc0 = make_float2(0.f, 0.f), acc1 = acc0;
  long j = j0;
  for(; j + 7 < j1; j += 8) {
    float2 s[8];
#pragma unroll
    for(int u = 0; u < 8; ++u)
      s[u] = col[u * ld];
#pragma unroll
    for(int u = 0; u < 8; ++u)
      copy[u * ldc] = pack_bf16c(s[u]);
#pragma unroll
    for(int u = 0; u < 8; u += 2) {
      acc0 = cfma(s[u], xs[j - j0 + u], acc0);
      acc1 = cfma(s[u + 1], xs[j - j0 + u + 1], acc1);
    }
    col += 8 * ld;
    copy += 8 * ldc;
  }
  for(; j < j1; ++j) {
    const float2 a0 = col[0];
    copy[0] = pack_bf16c(a0);
    acc0 = cfma(a0, xs[j - j0], acc0);
    col += ld;
    copy += ldc;
  }
  acc0.x += acc1.x;
  acc0.y += acc1.y;
  return acc0;
}

// Packed FP32 pairs (add / sub / mul / fma .rn.f32x2, sm_100 and later): one
// instruction updates the real and the imaginary lane, each rounded exactly as
// the scalar operation would be.
__device__ __forceinline__ unsigned long long pk_u(float2 a) { return *reinterpret_cast<unsigned long long *>(&a); }
__device__ __forceinline__ float2 pk_f(unsigned long long a) { return *reinterpret_cast<float2 *>(&a); }
__device__ __forceinline__ float2 pk_add(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_u(a)), "l"(pk_u(b)));
  return pk_f(d);
}
__device__ __forceinline__ float2 pk_sub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_u(a)), "l"(pk_u(b)));
  return pk_f(d);
}
__device__ __forceinline__ float2 pk_mul(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(pk_u(a)), "l"(pk_u(b)));
  return pk_f(d);
}
__device__ __forceinline__ float2 pk_fma(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(pk_u(a)), "l"(pk_u(b)), "l"(pk_u(c)));
  return pk_f(d);
}

// Float-float accumulation (TwoSum, Knuth) of a (re, im) pair of products:
// hi + lo gains p exactly.
__device__ __forceinline__ void df_add2(float2 &hi, float2 &lo, float2 p) {
  const float2 s = pk_add(hi, p);
  const float2 bb = pk_sub(s, hi);
  lo = pk_add(lo, pk_add(pk_sub(hi, pk_sub(s, bb)), pk_sub(p, bb)));
  hi = s;
}

// x staged for the compensated product: x = x_hi + x_lo in floats, each
// component duplicated into both lanes of a pair:
// h = (hi.re, hi.re, hi.im, hi.im), l = (lo.re, lo.re, lo.im, lo.im).
struct DFX {
  float4 h, l;
};
__device__ __forceinline__ DFX df_split(double2 v) {
  const float hr = (float)v.x, hi = (float)v.y;
  const float lr = (float)(v.x - (double)hr), li = (float)(v.y - (double)hi);
  return DFX{make_float4(hr, hr, hi, hi), make_float4(lr, lr, li, li)};
}

// Complex64 row times a complex128 vector with FP64-accurate results from
// FP32 arithmetic. With a = s_j and x_j = x_hi + x_lo, the products of
// a x_hi, P1 = hi.re (a.re, a.im) and P2 = hi.im (-a.im, a.re) (the real and
// imaginary lanes of the complex product), are made error-free with FMA
// (TwoProduct) and summed in a float-float accumulator; their rounding errors
// and a x_lo go to a separate float pair; the parts are combined in FP64.
// Eight columns' loads are in flight at a time. Per entry that is 44 FP32
// lane operations, so at n = 64,000 the FP32 pipe alone needs about 4.5 ms,
// as long as reading the matrix.
__device__ __forceinline__ double2 mv_row_df(const float2 *col, long ld, const DFX *xs, long j0, long j1) {
  float2 hi = make_float2(0.f, 0.f), lo = hi, e = hi;
  for(long j = j0; j < j1; j += 8) {
    float2 av[8];
    const int cnt = (int)min(8L, j1 - j);
#pragma unroll
    for(int u = 0; u < 8; ++u)
      av[u] = u < cnt ? col[u * ld] : make_float2(0.f, 0.f);
#pragma unroll
    for(int u = 0; u < 8; ++u) {
      if(u >= cnt)
        break;
      const float2 a = av[u];
      const float2 as = make_float2(-a.y, a.x), na = make_float2(-a.x, -a.y), nas = make_float2(a.y, -a.x);
      const DFX X = xs[j - j0 + u];
      const float2 x1 = make_float2(X.h.x, X.h.y), x2 = make_float2(X.h.z, X.h.w);
      const float2 l1 = make_float2(X.l.x, X.l.y), l2 = make_float2(X.l.z, X.l.w);
      const float2 P1 = pk_mul(x1, a), P2 = pk_mul(x2, as);
      // P - x a = -(rounding error of P), exact
      e = pk_sub(e, pk_fma(x1, na, P1));
      e = pk_sub(e, pk_fma(x2, nas, P2));
      e = pk_fma(l1, a, e);
      e = pk_fma(l2, as, e);
      df_add2(hi, lo, P1);
      df_add2(hi, lo, P2);
    }
    col += 8 * ld;
  }
  return make_double2((double)hi.x + ((double)lo.x + (double)e.x), (double)hi.y + ((double)lo.y + (double)e.y));
}

}  // namespace om
