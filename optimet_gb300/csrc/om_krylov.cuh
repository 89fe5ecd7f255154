// Complex arithmetic and the per-row matrix-vector sums shared by the Krylov
// solvers (solve.cu) and the batched solvers (batch.cu). Both call the same
// inline functions, so a row's sum is formed in the same order, and rounds the
// same, whichever solver runs it.
#pragma once

#include <cuda_runtime.h>

namespace om {

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
      V a0, a1;
      a0.x = s[u].x; a0.y = s[u].y; a1.x = s[u + 1].x; a1.y = s[u + 1].y;
      acc0 = cfma(a0, xs[j - j0 + u], acc0);
      acc1 = cfma(a1, xs[j - j0 + u + 1], acc1);
    }
    col += 8 * ld;
  }
  for(; j < j1; ++j) {
    M s0 = col[0];
    V a0;
    a0.x = s0.x;
    a0.y = s0.y;
    acc0 = cfma(a0, xs[j - j0], acc0);
    col += ld;
  }
  acc0.x += acc1.x;
  acc0.y += acc1.y;
  return acc0;
}

// Float-float accumulator (TwoSum, Knuth) of the compensated products.
struct DF {
  float hi, lo;
};
__device__ __forceinline__ void df_add(DF &a, float p) {
  const float s = a.hi + p;
  const float bb = s - a.hi;
  a.lo += (a.hi - (s - bb)) + (p - bb);
  a.hi = s;
}

// x split for the compensated product: (hi.re, hi.im, lo.re, lo.im) in floats
__device__ __forceinline__ float4 df_split(double2 v) {
  const float hr = (float)v.x, hi = (float)v.y;
  return make_float4(hr, hi, (float)(v.x - (double)hr), (float)(v.y - (double)hi));
}

// Complex64 row times a complex128 vector with FP64-accurate results from
// FP32 arithmetic: the products s * x_hi are made error-free with FMA
// (TwoProduct) and summed in a float-float accumulator; the small terms
// (product errors and s * x_lo) go to a separate float sum; the parts are
// combined in FP64. Four columns' loads are in flight at a time.
__device__ __forceinline__ double2 mv_row_df(const float2 *col, long ld, const float4 *xs, long j0,
                                             long j1) {
  DF re{0.f, 0.f}, im{0.f, 0.f};
  float er = 0.f, ei = 0.f;
  for(long j = j0; j < j1; j += 4) {
    float2 av[4];
    const int cnt = (int)min(4L, j1 - j);
#pragma unroll
    for(int u = 0; u < 4; ++u)
      av[u] = u < cnt ? col[u * ld] : make_float2(0.f, 0.f);
#pragma unroll
    for(int u = 0; u < 4; ++u) {
      if(u >= cnt)
        break;
      const float2 a = av[u];
      const float4 v = xs[j - j0 + u];
      // __fmul_rn keeps the products out of FMA contraction so that the
      // TwoProduct error terms below are exact
      float p = __fmul_rn(a.x, v.x);
      er += fmaf(a.x, v.x, -p);
      df_add(re, p);
      p = __fmul_rn(-a.y, v.y);
      er += fmaf(-a.y, v.y, -p);
      df_add(re, p);
      er = fmaf(a.x, v.z, er);
      er = fmaf(-a.y, v.w, er);
      p = __fmul_rn(a.x, v.y);
      ei += fmaf(a.x, v.y, -p);
      df_add(im, p);
      p = __fmul_rn(a.y, v.x);
      ei += fmaf(a.y, v.x, -p);
      df_add(im, p);
      ei = fmaf(a.x, v.w, ei);
      ei = fmaf(a.y, v.z, ei);
    }
    col += 4 * ld;
  }
  return make_double2((double)re.hi + ((double)re.lo + (double)er),
                      (double)im.hi + ((double)im.lo + (double)ei));
}

}  // namespace om
