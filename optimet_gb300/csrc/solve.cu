// Dense solves of the OPTIMET scattering system on the device.
//
//  * LU with partial pivoting (the ScalapackSolver / pzgesv role,
//    ScalapackSolver.cpp:54-130): right-looking, panels of kNb columns; the
//    complex64 LU with tensor cores in blocks of kTcBlock columns with one
//    rank-kTcBlock trailing update per block.
//  * Restarted GMRES (the MatrixBelosSolver / Gmres_Zcomp role,
//    MatrixBelosSolver.cpp:26-104, PreconditionedMatrix.cpp:892-985): classical
//    Gram-Schmidt with one re-orthogonalisation pass, Givens rotations of
//    det_approx (:1087-1133) on the host, residual |g_{k+1}| / ||b||.
//  * Mixed precision form: FP64 outer flexible GMRES (Saad 1993) whose
//    preconditioner is a fixed-length FP32 GMRES on the complex64 copy of S.
// Reductions write per-block partial sums and add them in a fixed order, so
// every solve is bitwise reproducible for a given problem.
#include <type_traits>
#include <algorithm>
#include <chrono>
#include <cmath>
#include <complex>
#include <mutex>
#include <string>
#include <vector>

#include "om_internal.h"
#include "om_krylov.cuh"

namespace om {

namespace {

template <typename R> struct C2;
template <> struct C2<double> {
  typedef double2 T;
};
template <> struct C2<float> {
  typedef float2 T;
};

constexpr int kMvThreads = 256;
constexpr int kMvCols = 1024;  // largest split-K chunk (x staged in shared memory)

// Columns per split-K chunk: 1024, halved (down to 128) while the tile grid
// would leave the GPU short of work (fewer than 4 tiles per SM).
inline int mv_cols(const om_context *ctx, long n) {
  int cols = kMvCols;
  const long rows = (n + kMvThreads - 1) / kMvThreads;
  while(cols > 128 && rows * ((n + cols - 1) / cols) < 4L * ctx->sm_count)
    cols >>= 1;
  return cols;
}
inline int mv_nsplit(const om_context *ctx, long n) {
  const int c = mv_cols(ctx, n);
  return (int)((n + c - 1) / c);
}

// Partial y over chunks of columns: part[s * n + i] = sum_{j in chunk s} S[j ld + i] x[j].
// A tile is kMvThreads rows x kMvCols columns; the grid is capped (a few CTAs
// per SM) and the CTAs take tiles from a counter (*next, zeroed before the
// launch) in column-chunk-major order, so the kernel leaves room on every SM
// for the assembly kernel of another slot and still balances its load. Eight columns'
// loads are issued before their FMAs; the two accumulators take alternate
// columns.
template <typename M, typename V>
__global__ void __launch_bounds__(kMvThreads) k_matvec_part(const M *S, long ld, long n, const V *x,
                                                           V *part, int row_tiles, long tiles,
                                                           unsigned long long *next, int cols) {
  __shared__ V xs[kMvCols];
  __shared__ long tile;
  for(;;) {
    __syncthreads();
    if(threadIdx.x == 0)
      tile = (long)atomicAdd(next, 1ull);
    __syncthreads();
    const long t = tile;
    if(t >= tiles)
      break;
    const long ct = t / row_tiles, rt = t - ct * row_tiles;
    const long i = rt * kMvThreads + threadIdx.x;
    const long j0 = ct * cols;
    const long j1 = min(n, j0 + cols);
    for(long j = j0 + threadIdx.x; j < j1; j += kMvThreads)
      xs[j - j0] = x[j];
    __syncthreads();
    if(i >= n)
      continue;
    part[ct * n + i] = mv_row<M, V>(S + j0 * ld + i, ld, xs, j0, j1);
  }
}

// k_matvec_part<float2, float2> that also writes the bf16 copy of S (ld ldc)
__global__ void __launch_bounds__(kMvThreads) k_matvec_part_copy(const float2 *S, long ld, long n,
                                                                const float2 *x, float2 *part, int row_tiles,
                                                                long tiles, unsigned long long *next, int cols,
                                                                Bf16c *copy, long ldc) {
  __shared__ float2 xs[kMvCols];
  __shared__ long tile;
  for(;;) {
    __syncthreads();
    if(threadIdx.x == 0)
      tile = (long)atomicAdd(next, 1ull);
    __syncthreads();
    const long t = tile;
    if(t >= tiles)
      break;
    const long ct = t / row_tiles, rt = t - ct * row_tiles;
    const long i = rt * kMvThreads + threadIdx.x;
    const long j0 = ct * cols;
    const long j1 = min(n, j0 + cols);
    for(long j = j0 + threadIdx.x; j < j1; j += kMvThreads)
      xs[j - j0] = x[j];
    __syncthreads();
    if(i >= n)
      continue;
    part[ct * n + i] = mv_row_copy(S + j0 * ld + i, ld, xs, j0, j1, copy + j0 * ldc + i, ldc);
  }
}

// Complex64 matrix times a complex128 vector with FP64-accurate results from
// FP32 arithmetic (the precision form's refinement residuals): x is split as
// x_hi + x_lo (floats); the products s * x_hi are made error-free with FMA
// (TwoProduct) and summed in a float-float accumulator (TwoSum, Knuth); the
// small terms (product errors and s * x_lo) go to a separate float sum. Each
// CTA sums kMvCols columns, so the per-thread sums are short; partials are
// combined in FP64.
__global__ void __launch_bounds__(kMvThreads) k_matvec_part_df(const float2 *S, long ld, long n,
                                                               const double2 *x, double2 *part,
                                                               int row_tiles, long tiles,
                                                               unsigned long long *next, int cols) {
  __shared__ DFX xs[kMvCols];
  __shared__ long tile;
  for(;;) {
    __syncthreads();
    if(threadIdx.x == 0)
      tile = (long)atomicAdd(next, 1ull);
    __syncthreads();
    const long t = tile;
    if(t >= tiles)
      break;
    const long ct = t / row_tiles, rt = t - ct * row_tiles;
    const long i = rt * kMvThreads + threadIdx.x;
    const long j0 = ct * cols;
    const long j1 = min(n, j0 + cols);
    for(long j = j0 + threadIdx.x; j < j1; j += kMvThreads)
      xs[j - j0] = df_split(x[j]);
    __syncthreads();
    if(i >= n)
      continue;
    part[ct * n + i] = mv_row_df(S + j0 * ld + i, ld, xs, j0, j1);
  }
}

// y = sum of partials (fixed order); if b given: y = b - sum.
template <typename V>
__global__ void k_matvec_reduce(const V *part, int nsplit, long n, const V *b, V *y) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  V acc = part[i];
  for(int s = 1; s < nsplit; ++s) {
    V v = part[s * n + i];
    acc.x += v.x;
    acc.y += v.y;
  }
  if(b) {
    acc.x = b[i].x - acc.x;
    acc.y = b[i].y - acc.y;
  }
  y[i] = acc;
}

constexpr int kDotThreads = 256;
constexpr int kDotRows = 2048;  // rows per block of the multi-dot

// part[b * (k+1) + t] = sum_{rows of block b} conj(V[:, t]) w   (t < k), and
// part[b * (k+1) + k] = sum |w|^2 over the block.
template <typename V>
__global__ void __launch_bounds__(kDotThreads) k_multidot(const V *Vb, long ldv, int k, const V *w,
                                                         long n, V *part) {
  __shared__ V red[kDotThreads];
  const long r0 = blockIdx.x * (long)kDotRows;
  const long r1 = min(n, r0 + kDotRows);
  for(int t = 0; t <= k; ++t) {
    V acc;
    acc.x = acc.y = 0;
    if(t < k) {
      const V *v = Vb + t * ldv;
      for(long i = r0 + threadIdx.x; i < r1; i += kDotThreads)
        acc = cfma_conj(v[i], w[i], acc);
    } else {
      for(long i = r0 + threadIdx.x; i < r1; i += kDotThreads) {
        V a = w[i];
        acc.x = fma(a.x, a.x, acc.x);
        acc.x = fma(a.y, a.y, acc.x);
      }
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for(int s = kDotThreads / 2; s > 0; s >>= 1) {
      if(threadIdx.x < s) {
        red[threadIdx.x].x += red[threadIdx.x + s].x;
        red[threadIdx.x].y += red[threadIdx.x + s].y;
      }
      __syncthreads();
    }
    if(threadIdx.x == 0)
      part[blockIdx.x * (k + 1) + t] = red[0];
    __syncthreads();
  }
}

template <typename V> __global__ void k_sum_parts(const V *part, int nblk, int k1, V *out) {
  const int t = threadIdx.x;
  if(t >= k1)
    return;
  V acc = part[t];
  for(int b = 1; b < nblk; ++b) {
    acc.x += part[b * k1 + t].x;
    acc.y += part[b * k1 + t].y;
  }
  out[t] = acc;
}

// w -= V[:, 0..k) h ; h read from device
template <typename V>
__global__ void k_sub_basis(const V *Vb, long ldv, int k, const V *h, V *w, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  V acc = w[i];
  for(int t = 0; t < k; ++t) {
    V c = h[t];
    c.x = -c.x;
    c.y = -c.y;
    acc = cfma(Vb[t * ldv + i], c, acc);
  }
  w[i] = acc;
}

// dst = src * s (real scale) with conversion
template <typename A, typename B> __global__ void k_scale_copy(const A *src, double s, B *dst, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  dst[i].x = src[i].x * s;
  dst[i].y = src[i].y * s;
}

// x += sum_t y_t Z[:, t]
template <typename V, typename Z>
__global__ void k_add_combo(const Z *Zb, long ldz, int k, const double2 *y, V *x, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  double2 acc = make_double2(x[i].x, x[i].y);
  for(int t = 0; t < k; ++t) {
    Z z = Zb[t * ldz + i];
    double2 zz = make_double2(z.x, z.y);
    acc = cfma(zz, y[t], acc);
  }
  x[i].x = acc.x;
  x[i].y = acc.y;
}

// ---------------------------------------------------------------------------
// Krylov workspace and helpers
// ---------------------------------------------------------------------------
struct Work {
  om_context *ctx = nullptr;
  long n = 0;
  void *buf = nullptr;
  size_t bytes = 0;
  ~Work() {
    if(buf)
      dev_release(ctx, buf, bytes);
  }
  template <typename T> T *take(size_t count, size_t &off) {
    T *p = reinterpret_cast<T *>(reinterpret_cast<char *>(buf) + off);
    off += ((count * sizeof(T) + 255) / 256) * 256;
    return p;
  }
};

int alloc_work(om_context *ctx, Work &w, size_t bytes) {
  int rc = dev_malloc(ctx, &w.buf, bytes);
  if(rc)
    return rc;
  w.bytes = bytes;
  return OM_OK;
}

template <typename M, typename V>
void matvec(om_context *ctx, const M *S, long n, const V *x, V *part, V *y, const V *b) {
  const int nsplit = mv_nsplit(ctx, n);
  const int row_tiles = (int)((n + kMvThreads - 1) / kMvThreads);
  const long tiles = (long)row_tiles * nsplit;
  constexpr bool df = sizeof(M) == sizeof(float2) && sizeof(V) == sizeof(double2);
  const long cap = (long)ctx->sm_count * (df ? ctx->mv_ctas_df : ctx->mv_ctas);
  const unsigned grid = (unsigned)std::max(1L, std::min(tiles, cap));
  auto &ev = sizeof(M) == sizeof(double2) ? ctx->ev_mv64 : (df ? ctx->ev_mvdf : ctx->ev_mv32);
  if(ctx->carve_mv >= 0) {
    if constexpr(df)
      cudaFuncSetAttribute(k_matvec_part_df, cudaFuncAttributePreferredSharedMemoryCarveout,
                           ctx->carve_mv);
    else
      cudaFuncSetAttribute(k_matvec_part<M, V>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           ctx->carve_mv);
  }
  timer_begin(ctx, ev);
  cudaMemsetAsync(ctx->d_tile_counter, 0, sizeof(unsigned long long), ctx->stream);
  // the inner FP32 matvec streams its tiles through TMA; the compensated one
  // (FP32-ALU heavy) keeps the register-prefetching kernel, which measured
  // faster (6.98 ms against 9.12 ms at n = 64,000)
  bool done = false;
  if constexpr(sizeof(M) == sizeof(float2) && !df)
    if(ctx->mv_tma)
      done = launch_matvec_tma(ctx, (const float2 *)S, n, (const float2 *)x, (float2 *)part, row_tiles, tiles,
                               mv_cols(ctx, n), grid, nullptr, 0);
  if(done) {
  } else if constexpr(df)
    k_matvec_part_df<<<grid, kMvThreads, 0, ctx->stream>>>((const float2 *)S, n, n,
                                                           (const double2 *)x, (double2 *)part,
                                                           row_tiles, tiles, ctx->d_tile_counter,
                                                           mv_cols(ctx, n));
  else
    k_matvec_part<M, V><<<grid, kMvThreads, 0, ctx->stream>>>(S, n, n, x, part, row_tiles, tiles,
                                                              ctx->d_tile_counter, mv_cols(ctx, n));
  timer_end(ctx, ev);
  k_matvec_reduce<V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(part, nsplit, n, b, y);
  ctx->last_launches += 2;
}

// The bf16 copy of a complex64 matrix for the inner FP32 GMRES (ld a
// multiple of 4, so that a column starts on a 16-byte boundary).
struct Bf16Copy {
  Bf16c *H = nullptr;
  long ld = 0;
  bool ready = false;  // written by an earlier product of this solve
};

// y = S x for the inner FP32 GMRES of the precision form. With a copy: the
// first product runs on the complex64 matrix and writes the copy as it reads
// S; the later ones read the copy (4 bytes per entry instead of 8). TMA-staged
// kernels where the context uses them, else the register-prefetching ones.
void matvec_inner(om_context *ctx, const float2 *S, long n, Bf16Copy *hc, const float2 *x, float2 *part,
                  float2 *y) {
  if(!hc || !hc->H) {
    matvec<float2, float2>(ctx, S, n, x, part, y, nullptr);
    return;
  }
  const int nsplit = mv_nsplit(ctx, n);
  const int row_tiles = (int)((n + kMvThreads - 1) / kMvThreads);
  const long tiles = (long)row_tiles * nsplit;
  const unsigned grid = (unsigned)std::max(1L, std::min(tiles, (long)ctx->sm_count * ctx->mv_ctas));
  const int cols = mv_cols(ctx, n);
  const bool first = !hc->ready;
  auto &ev = first ? ctx->ev_mvcp : ctx->ev_mv16;
  timer_begin(ctx, ev);
  cudaMemsetAsync(ctx->d_tile_counter, 0, sizeof(unsigned long long), ctx->stream);
  bool done = false;
  if(first) {
    if(ctx->mv_tma)
      done = launch_matvec_tma(ctx, S, n, x, part, row_tiles, tiles, cols, grid, hc->H, hc->ld);
    if(!done)
      k_matvec_part_copy<<<grid, kMvThreads, 0, ctx->stream>>>(S, n, n, x, part, row_tiles, tiles,
                                                               ctx->d_tile_counter, cols, hc->H, hc->ld);
    hc->ready = true;
  } else {
    if(ctx->mv_tma)
      done = launch_matvec_bf16(ctx, hc->H, n, hc->ld, x, part, row_tiles, tiles, cols, grid);
    if(!done)
      k_matvec_part<Bf16c, float2><<<grid, kMvThreads, 0, ctx->stream>>>(hc->H, hc->ld, n, x, part, row_tiles,
                                                                        tiles, ctx->d_tile_counter, cols);
  }
  timer_end(ctx, ev);
  k_matvec_reduce<float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(part, nsplit, n, nullptr, y);
  ctx->last_launches += 2;
}

// h[0..k) = V^H w, h[k] = |w|^2, returned on the host (synchronous).
template <typename V>
void multidot(om_context *ctx, const V *Vb, long n, int k, const V *w, V *part, V *hd,
              std::vector<std::complex<double>> &hh) {
  const int nblk = (int)((n + kDotRows - 1) / kDotRows);
  k_multidot<V><<<nblk, kDotThreads, 0, ctx->stream>>>(Vb, n, k, w, n, part);
  k_sum_parts<V><<<1, 256 * ((k + 256) / 256), 0, ctx->stream>>>(part, nblk, k + 1, hd);
  ctx->last_launches += 2;
  std::vector<V> tmp(k + 1);
  cudaMemcpyAsync(tmp.data(), hd, sizeof(V) * (k + 1), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  hh.resize(k + 1);
  for(int t = 0; t <= k; ++t)
    hh[t] = std::complex<double>(tmp[t].x, tmp[t].y);
}

// the same sums left on the device (hd[0..k]), no host copy
template <typename V>
void multidot_dev(om_context *ctx, const V *Vb, long n, int k, const V *w, V *part, V *hd) {
  const int nblk = (int)((n + kDotRows - 1) / kDotRows);
  k_multidot<V><<<nblk, kDotThreads, 0, ctx->stream>>>(Vb, n, k, w, n, part);
  k_sum_parts<V><<<1, 256 * ((k + 256) / 256), 0, ctx->stream>>>(part, nblk, k + 1, hd);
  ctx->last_launches += 2;
}


// Givens rotation of det_approx (PreconditionedMatrix.cpp:1102-1118)
void givens(std::complex<double> hi1, std::complex<double> hi2, std::complex<double> &c,
            std::complex<double> &s) {
  if(std::abs(hi2) > std::abs(hi1)) {
    std::complex<double> t = hi1 / hi2;
    s = 1.0 / std::sqrt(1.0 + std::pow(std::abs(t), 2));
    c = -t * s;
  } else {
    std::complex<double> t = hi2 / hi1;
    c = 1.0 / std::sqrt(1.0 + std::pow(std::abs(t), 2));
    s = -t * c;
  }
}

// One Arnoldi step with CGS2: w <- w - V h (twice), returns h (k+1 entries incl. norm).
template <typename V>
void arnoldi_orth(om_context *ctx, const V *Vb, long n, int k, V *w, V *part, V *hd,
                  std::vector<std::complex<double>> &h) {
  // hd holds (2 k + 3 entries): the projections of the two passes, then
  // |w|^2 after both; the passes subtract with the device copies and the host
  // reads all three once
  V *h1 = hd, *h2 = hd + (k + 1), *h3 = hd + 2 * (k + 1);
  multidot_dev(ctx, Vb, n, k, w, part, h1);
  k_sub_basis<V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(Vb, n, k, h1, w, n);
  multidot_dev(ctx, Vb, n, k, w, part, h2);
  k_sub_basis<V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(Vb, n, k, h2, w, n);
  multidot_dev(ctx, Vb, n, 0, w, part, h3);
  ctx->last_launches += 2;
  std::vector<V> tmp(2 * (k + 1) + 1);
  cudaMemcpyAsync(tmp.data(), hd, sizeof(V) * tmp.size(), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  h.assign(k + 1, 0.0);
  for(int t = 0; t < k; ++t)
    h[t] = std::complex<double>(tmp[t].x, tmp[t].y) +
           std::complex<double>(tmp[k + 1 + t].x, tmp[k + 1 + t].y);
  h[k] = std::sqrt((double)tmp[2 * (k + 1)].x);
}

double vec_norm(om_context *ctx, const double2 *w, long n, double2 *part, double2 *hd) {
  std::vector<std::complex<double>> h;
  multidot<double2>(ctx, nullptr, n, 0, w, part, hd, h);
  return std::sqrt(h[0].real());
}

// Restarted GMRES (right-hand side b, solution x; both FP64 device vectors).
// Preconditioner hook: if `precond` is set, the flexible variant is used and
// Z[:, k] = precond(V[:, k]) is stored (FGMRES).
struct PrecondFn {
  virtual void apply(const double2 *v, double2 *z) = 0;
  virtual ~PrecondFn() {}
};

// y = S x (b null) or y = b - S x for the operators GMRES runs on: a dense
// complex128 / complex64 matrix or the ACA-compressed operator
template <typename M>
void op_apply(om_context *ctx, const M *S, long n, const double2 *x, double2 *part, double2 *y,
              const double2 *b) {
  matvec<M, double2>(ctx, S, n, x, part, y, b);
}
inline void op_apply(om_context *ctx, const AcaOp *S, long, const double2 *x, double2 *, double2 *y,
                     const double2 *b) {
  aca_matvec(ctx, *S, x, y, b);
}

template <typename M>
int gmres64(om_context *ctx, const M *S, long n, const double2 *b, double2 *x, double tol, int m,
            int restarts, PrecondFn *pc, int *iters, double *relres) {
  Work w;
  w.ctx = ctx;
  const int nsplit = mv_nsplit(ctx, n);
  const int nblk = (int)((n + kDotRows - 1) / kDotRows);
  size_t bytes = sizeof(double2) * ((size_t)(m + 1) * n + (pc ? (size_t)m * n : 0) + n +
                                    (size_t)nsplit * n + (size_t)nblk * (m + 2) + 3 * (m + 2)) +
                 64 * 256;
  int rc = alloc_work(ctx, w, bytes);
  if(rc)
    return rc;
  size_t off = 0;
  double2 *Vb = w.take<double2>((size_t)(m + 1) * n, off);
  double2 *Zb = pc ? w.take<double2>((size_t)m * n, off) : nullptr;
  double2 *r = w.take<double2>(n, off);
  double2 *part = w.take<double2>((size_t)std::max<long>((long)nsplit * n, (long)nblk * (m + 2)), off);
  double2 *hd = w.take<double2>(2 * (m + 2), off);
  double2 *yd = w.take<double2>(m + 2, off);

  cudaMemsetAsync(x, 0, sizeof(double2) * n, ctx->stream);
  const double bnorm = vec_norm(ctx, b, n, part, hd);
  *iters = 0;
  if(bnorm == 0.0) {
    *relres = 0.0;
    return OM_OK;
  }
  double err = 1.0;
  int total = 0;
  for(int rest = 0; rest < restarts && err > tol; ++rest) {
    // r = b - S x (x = 0 on the first cycle)
    double beta;
    if(rest == 0) {
      cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->stream);
      beta = bnorm;
    } else {
      op_apply(ctx, S, n, x, part, r, b);
      beta = vec_norm(ctx, r, n, part, hd);
      err = beta / bnorm;
      if(err <= tol)
        break;
    }
    if(beta == 0.0) {
      err = 0.0;
      break;
    }
    k_scale_copy<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(r, 1.0 / beta, Vb, n);
    ctx->last_launches++;
    std::vector<std::vector<std::complex<double>>> H;
    std::vector<std::complex<double>> cs, sn, g(1, beta);
    int k = 0;
    double cur = beta / bnorm;
    while(k < m && cur > tol) {
      const double2 *vin = Vb + (size_t)k * n;
      const double2 *op_in = vin;
      if(pc) {
        pc->apply(vin, Zb + (size_t)k * n);
        op_in = Zb + (size_t)k * n;
      }
      double2 *wv = Vb + (size_t)(k + 1) * n;
      op_apply(ctx, S, n, op_in, part, wv, nullptr);
      std::vector<std::complex<double>> h;
      arnoldi_orth<double2>(ctx, Vb, n, k + 1, wv, part, hd, h);
      const double hn = h[k + 1].real();
      if(hn > 0.0) {
        k_scale_copy<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(wv, 1.0 / hn, wv, n);
        ctx->last_launches++;
      }
      for(int i = 0; i < k; ++i) {
        std::complex<double> a = h[i], bb = h[i + 1];
        h[i] = std::conj(cs[i]) * a + std::conj(-sn[i]) * bb;
        h[i + 1] = sn[i] * a + cs[i] * bb;
      }
      std::complex<double> c, s;
      givens(h[k], h[k + 1], c, s);
      cs.push_back(c);
      sn.push_back(s);
      std::complex<double> hk = h[k], hk1 = h[k + 1];
      h[k] = std::conj(c) * hk + std::conj(-s) * hk1;
      h[k + 1] = s * hk + c * hk1;
      g.push_back(0.0);
      std::complex<double> g0 = g[k], g1 = g[k + 1];
      g[k] = std::conj(c) * g0 + std::conj(-s) * g1;
      g[k + 1] = s * g0 + c * g1;
      H.push_back(h);
      cur = std::abs(g[k + 1]) / bnorm;
      ++k;
      ++total;
      if(hn == 0.0)
        break;
    }
    // back substitution and update
    std::vector<std::complex<double>> y(k);
    for(int j = k - 1; j >= 0; --j) {
      std::complex<double> v = g[j];
      for(int q = j + 1; q < k; ++q)
        v -= H[q][j] * y[q];
      y[j] = v / H[j][j];
    }
    std::vector<double2> yh(k);
    for(int j = 0; j < k; ++j)
      yh[j] = make_double2(y[j].real(), y[j].imag());
    cudaMemcpyAsync(yd, yh.data(), sizeof(double2) * k, cudaMemcpyHostToDevice, ctx->stream);
    k_add_combo<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(pc ? Zb : Vb, n, k,
                                                                               yd, x, n);
    ctx->last_launches++;
    // the stopping test of Gmres_Zcomp (PreconditionedMatrix.cpp:916-919,
    // 962-964): the residual estimate |g_{k+1}| / ||b||; a further cycle starts
    // from the true residual. The estimate assumes that y solves the small
    // least-squares problem exactly; with a flexible preconditioner the basis
    // Z can be ill-conditioned (an inaccurate LU), and so can R. Then the
    // true residual decides (R's diagonal ratio, a lower bound on its
    // condition number, above 1e6).
    err = cur;
    if(pc && err <= tol && k > 0) {
      double dmax = 0.0, dmin = 1e300;
      for(int j = 0; j < k; ++j) {
        dmax = std::max(dmax, std::abs(H[j][j]));
        dmin = std::min(dmin, std::abs(H[j][j]));
      }
      if(!(dmax <= 1e6 * dmin)) {
        op_apply(ctx, S, n, x, part, r, b);
        err = vec_norm(ctx, r, n, part, hd) / bnorm;
      }
    }
  }
  *iters = total;
  *relres = err;
  return err <= tol ? OM_OK : OM_ERR_NOT_CONVERGED;
}

// FP32 GMRES of fixed maximum length on the complex64 matrix, used as the
// flexible preconditioner: z ~= S^{-1} v (no restart, x0 = 0).
struct InnerGmres32 : PrecondFn {
  om_context *ctx;
  const float2 *S;
  long n;
  int m;
  double tol;
  Work w;
  float2 *Vb, *r, *part, *hd, *yd, *xz;
  int total = 0;
  Work hw;       // the bf16 copy of S (inner_half), made by the first product
  Bf16Copy hc;
  InnerGmres32(om_context *c, const float2 *S_, long n_, int m_, double tol_)
      : ctx(c), S(S_), n(n_), m(m_), tol(tol_) {
    w.ctx = c;
    hw.ctx = c;
  }
  int init() {
    if(ctx->inner_half) {
      // within the budget, else the products stay on the complex64 matrix
      const long ld = (n + 3) / 4 * 4;
      if(alloc_work(ctx, hw, sizeof(Bf16c) * (size_t)ld * n + 256) == OM_OK) {
        hc.H = static_cast<Bf16c *>(hw.buf);
        hc.ld = ld;
      } else {
        ctx->err.clear();
      }
    }
    const int nsplit = mv_nsplit(ctx, n);
    const int nblk = (int)((n + kDotRows - 1) / kDotRows);
    size_t bytes = sizeof(float2) * ((size_t)(m + 1) * n + 2 * n +
                                     (size_t)std::max<long>((long)nsplit * n, (long)nblk * (m + 2)) +
                                     3 * (m + 2)) +
                   16 * 256;
    int rc = alloc_work(ctx, w, bytes);
    if(rc)
      return rc;
    size_t off = 0;
    Vb = w.take<float2>((size_t)(m + 1) * n, off);
    r = w.take<float2>(n, off);
    xz = w.take<float2>(n, off);
    part = w.take<float2>((size_t)std::max<long>((long)nsplit * n, (long)nblk * (m + 2)), off);
    hd = w.take<float2>(2 * (m + 2), off);
    yd = w.take<float2>(m + 2, off);
    return OM_OK;
  }
  void apply(const double2 *v, double2 *z) override {
    // v has unit norm (an Arnoldi vector): start from r0 = v
    k_scale_copy<double2, float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(v, 1.0, Vb, n);
    ctx->last_launches++;
    std::vector<std::vector<std::complex<double>>> H;
    std::vector<std::complex<double>> cs, sn, g(1, 1.0);
    int k = 0;
    double cur = 1.0;
    while(k < m && cur > tol) {
      float2 *wv = Vb + (size_t)(k + 1) * n;
      matvec_inner(ctx, S, n, &hc, Vb + (size_t)k * n, part, wv);
      std::vector<std::complex<double>> h;
      arnoldi_orth<float2>(ctx, Vb, n, k + 1, wv, part, hd, h);
      const double hn = h[k + 1].real();
      if(hn > 0.0) {
        k_scale_copy<float2, float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(wv, 1.0 / hn, wv, n);
        ctx->last_launches++;
      }
      for(int i = 0; i < k; ++i) {
        std::complex<double> a = h[i], bb = h[i + 1];
        h[i] = std::conj(cs[i]) * a + std::conj(-sn[i]) * bb;
        h[i + 1] = sn[i] * a + cs[i] * bb;
      }
      std::complex<double> c, s;
      givens(h[k], h[k + 1], c, s);
      cs.push_back(c);
      sn.push_back(s);
      std::complex<double> hk = h[k], hk1 = h[k + 1];
      h[k] = std::conj(c) * hk + std::conj(-s) * hk1;
      h[k + 1] = s * hk + c * hk1;
      g.push_back(0.0);
      std::complex<double> g0 = g[k], g1 = g[k + 1];
      g[k] = std::conj(c) * g0 + std::conj(-s) * g1;
      g[k + 1] = s * g0 + c * g1;
      H.push_back(h);
      cur = std::abs(g[k + 1]);
      ++k;
      ++total;
      if(hn == 0.0)
        break;
    }
    std::vector<std::complex<double>> y(k);
    for(int j = k - 1; j >= 0; --j) {
      std::complex<double> vv = g[j];
      for(int q = j + 1; q < k; ++q)
        vv -= H[q][j] * y[q];
      y[j] = vv / H[j][j];
    }
    std::vector<double2> yh(k);
    for(int j = 0; j < k; ++j)
      yh[j] = make_double2(y[j].real(), y[j].imag());
    cudaMemsetAsync(z, 0, sizeof(double2) * n, ctx->stream);
    upload_y_and_combine(yh, k, z);
  }
  Work ybuf;
  double2 *ydev = nullptr;
  void upload_y_and_combine(const std::vector<double2> &yh, int k, double2 *z) {
    if(!ydev) {
      ybuf.ctx = ctx;
      alloc_work(ctx, ybuf, sizeof(double2) * (m + 2));
      ydev = reinterpret_cast<double2 *>(ybuf.buf);
    }
    cudaMemcpyAsync(ydev, yh.data(), sizeof(double2) * k, cudaMemcpyHostToDevice, ctx->stream);
    k_add_combo<double2, float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(Vb, n, k, ydev, z, n);
    ctx->last_launches++;
    cudaStreamSynchronize(ctx->stream);
  }
};

// ---------------------------------------------------------------------------
// LU with partial pivoting
// ---------------------------------------------------------------------------
constexpr int kNb = 32;

// The LU's complex products are written with explicit fused and unfused
// operations, so that every kernel that forms the same entry rounds it the
// same way (an expression such as a b - c d leaves the compiler free to fuse
// either product, and it may choose differently in different kernels).
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <typename V> __device__ __forceinline__ double mag2(V a) {
  return fma((double)a.x, (double)a.x, __dmul_rn((double)a.y, (double)a.y));
}
template <typename V> __device__ __forceinline__ V cmul(V a, V b) {
  V r;
  r.x = fma(a.x, b.x, -mul_rn(a.y, b.y));
  r.y = fma(a.x, b.y, mul_rn(a.y, b.x));
  return r;
}
template <typename V> __device__ __forceinline__ V make_neg(V a) {
  a.x = -a.x;
  a.y = -a.y;
  return a;
}
template <typename V> __device__ __forceinline__ V crecip(V a) {
  const double d = mag2(a);
  V r;
  r.x = a.x / d;
  r.y = -a.y / d;
  return r;
}

// Row i of the panel's columns c + 1 .. nb - 1 minus l times the pivot row u:
// eight columns' loads are issued before their stores (the loads of a group
// cannot move above the previous group's stores, which may alias them).
template <typename V>
__device__ __forceinline__ void panel_row_update(V *A, long ld, long k, long i, int c, int nb, V l,
                                                 const V *u) {
  for(int j0 = c + 1; j0 < nb; j0 += 8) {
    V a[8];
#pragma unroll
    for(int q = 0; q < 8; ++q)
      if(j0 + q < nb)
        a[q] = A[(k + j0 + q) * ld + i];
#pragma unroll
    for(int q = 0; q < 8; ++q)
      if(j0 + q < nb) {
        const V uu = u[j0 + q];
        a[q].x = sub_rn(a[q].x, fma(l.x, uu.x, -mul_rn(l.y, uu.y)));
        a[q].y = sub_rn(a[q].y, fma(l.x, uu.y, mul_rn(l.y, uu.x)));
        A[(k + j0 + q) * ld + i] = a[q];
      }
  }
}

// Unblocked LU of the panel A[k:n, k:k+nb) (one CTA); pivots to piv[k..k+nb).
template <typename V>
__global__ void __launch_bounds__(1024) k_lu_panel(V *A, long ld, long n, long k, int nb, int *piv,
                                                   int *info) {
  __shared__ double bestv[1024];
  __shared__ long besti[1024];
  __shared__ V pivrow[kNb];
  const int t = threadIdx.x;
  for(int c = 0; c < nb; ++c) {
    const long col = k + c;
    double bv = -1.0;
    long bi = col;
    for(long i = col + t; i < n; i += blockDim.x) {
      double v = mag2(A[col * ld + i]);
      if(v > bv) {
        bv = v;
        bi = i;
      }
    }
    bestv[t] = bv;
    besti[t] = bi;
    __syncthreads();
    for(int s = blockDim.x / 2; s > 0; s >>= 1) {
      if(t < s) {
        if(bestv[t + s] > bestv[t] || (bestv[t + s] == bestv[t] && besti[t + s] < besti[t])) {
          bestv[t] = bestv[t + s];
          besti[t] = besti[t + s];
        }
      }
      __syncthreads();
    }
    const long p = besti[0];
    if(t == 0) {
      piv[col] = (int)p;
      if(bestv[0] <= 0.0 && *info == 0)
        *info = (int)col + 1;
    }
    // swap rows col and p inside the panel
    if(t < nb && p != col) {
      V a = A[(k + t) * ld + col];
      A[(k + t) * ld + col] = A[(k + t) * ld + p];
      A[(k + t) * ld + p] = a;
    }
    __syncthreads();
    if(t < nb)
      pivrow[t] = A[(k + t) * ld + col];
    __syncthreads();
    if(bestv[0] > 0.0) {
      const V inv = crecip(pivrow[c]);
      for(long i = col + 1 + t; i < n; i += blockDim.x) {
        V l = cmul(A[col * ld + i], inv);
        A[col * ld + i] = l;
        panel_row_update(A, ld, k, i, c, nb, l, pivrow);
      }
    }
    __syncthreads();
  }
}

// Tall panels on many CTAs (rows >= kTallPanel). Per column c: a one-CTA
// kernel takes the pivot from the per-CTA partial maxima (block order; the
// larger magnitude, then the smaller row index, as k_lu_panel), swaps the two
// rows inside the panel and publishes the pivot row; then a multi-CTA kernel
// scales column c below the pivot, applies the rank-1 update to the panel's
// later columns, and leaves the partial maxima of column c + 1. Each entry
// takes the same operations as in k_lu_panel, so the factors are the same.
constexpr long kTallPanel = 8192;
constexpr long kCoopPanel = 512;  // the shared-memory cooperative panel from here
constexpr int kPanThreads = 256;

struct PanelScratch {
  double *bestv;  // per CTA
  long *besti;
  long *bestr;    // per CTA: the physical row of the partial maximum (shared-memory panel)
  void *prow;     // kNb entries of the element type: the pivot row
  int nblk;
};

// partial maxima of |A[col, i]|^2, i >= col, one per CTA
template <typename V>
__global__ void __launch_bounds__(kPanThreads) k_pan_max(const V *A, long ld, long n, long col,
                                                         PanelScratch ps) {
  __shared__ double bv_s[kPanThreads];
  __shared__ long bi_s[kPanThreads];
  double bv = -1.0;
  long bi = col;
  for(long i = col + blockIdx.x * (long)kPanThreads + threadIdx.x; i < n;
      i += (long)gridDim.x * kPanThreads) {
    const double v = mag2(A[col * ld + i]);
    if(v > bv) {
      bv = v;
      bi = i;
    }
  }
  bv_s[threadIdx.x] = bv;
  bi_s[threadIdx.x] = bi;
  __syncthreads();
  for(int h = kPanThreads / 2; h > 0; h >>= 1) {
    if(threadIdx.x < h && (bv_s[threadIdx.x + h] > bv_s[threadIdx.x] ||
                           (bv_s[threadIdx.x + h] == bv_s[threadIdx.x] &&
                            bi_s[threadIdx.x + h] < bi_s[threadIdx.x]))) {
      bv_s[threadIdx.x] = bv_s[threadIdx.x + h];
      bi_s[threadIdx.x] = bi_s[threadIdx.x + h];
    }
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    ps.bestv[blockIdx.x] = bv_s[0];
    ps.besti[blockIdx.x] = bi_s[0];
  }
}

// the pivot of column col = k + c, the row swap inside the panel, the pivot
// row. One warp (kNb = 32 threads): each lane scans every 32nd partial
// maximum, then a butterfly leaves on every lane the largest magnitude, the
// smaller row index among equal ones (the order of k_lu_panel).
template <typename V>
__global__ void k_pan_pivot(V *A, long ld, long k, int c, int nb, int *piv, int *info, PanelScratch ps) {
  __shared__ long p_s;
  const long col = k + c;
  {
    double bv = -2.0;  // below every partial maximum (those are >= -1)
    long bi = col;
    for(int b = threadIdx.x; b < ps.nblk; b += 32) {
      const double v = ps.bestv[b];
      const long i = ps.besti[b];
      if(v > bv || (v == bv && i < bi)) {
        bv = v;
        bi = i;
      }
    }
#pragma unroll
    for(int h = 16; h > 0; h >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, h);
      const long oi = __shfl_xor_sync(0xffffffffu, bi, h);
      if(ov > bv || (ov == bv && oi < bi)) {
        bv = ov;
        bi = oi;
      }
    }
    if(threadIdx.x == 0) {
      piv[col] = (int)bi;
      if(bv <= 0.0 && *info == 0)
        *info = (int)col + 1;
      p_s = bi;
    }
  }
  __syncthreads();
  const long p = p_s;
  const int t = threadIdx.x;
  V *prow = reinterpret_cast<V *>(ps.prow);
  if(t < nb) {
    V a = A[(k + t) * ld + col];
    if(p != col) {
      V q = A[(k + t) * ld + p];
      A[(k + t) * ld + col] = q;
      A[(k + t) * ld + p] = a;
      a = q;
    }
    prow[t] = a;
  }
}

// column c below the pivot scaled by 1 / pivot, the later panel columns
// updated; partial maxima of column c + 1 (when there is one)
template <typename V>
__global__ void __launch_bounds__(kPanThreads) k_pan_update(V *A, long ld, long n, long k, int c, int nb,
                                                            PanelScratch ps) {
  __shared__ V u[kNb];
  __shared__ double bv_s[kPanThreads];
  __shared__ long bi_s[kPanThreads];
  const long col = k + c;
  const V *prow = reinterpret_cast<const V *>(ps.prow);
  if(threadIdx.x < nb)
    u[threadIdx.x] = prow[threadIdx.x];
  __syncthreads();
  const bool ok = mag2(u[c]) > 0.0;
  const V inv = ok ? crecip(u[c]) : u[c];
  const bool next = c + 1 < nb;
  const long ncol = col + 1;
  double bv = -1.0;
  long bi = ncol;
  for(long i = col + 1 + blockIdx.x * (long)kPanThreads + threadIdx.x; i < n;
      i += (long)gridDim.x * kPanThreads) {
    if(ok) {
      V l = cmul(A[col * ld + i], inv);
      A[col * ld + i] = l;
      panel_row_update(A, ld, k, i, c, nb, l, u);
    }
    if(next && i >= ncol) {
      const double v = mag2(A[ncol * ld + i]);
      if(v > bv) {
        bv = v;
        bi = i;
      }
    }
  }
  if(!next)
    return;
  bv_s[threadIdx.x] = bv;
  bi_s[threadIdx.x] = bi;
  __syncthreads();
  for(int h = kPanThreads / 2; h > 0; h >>= 1) {
    if(threadIdx.x < h && (bv_s[threadIdx.x + h] > bv_s[threadIdx.x] ||
                           (bv_s[threadIdx.x + h] == bv_s[threadIdx.x] &&
                            bi_s[threadIdx.x + h] < bi_s[threadIdx.x]))) {
      bv_s[threadIdx.x] = bv_s[threadIdx.x + h];
      bi_s[threadIdx.x] = bi_s[threadIdx.x + h];
    }
    __syncthreads();
  }
  if(threadIdx.x == 0) {
    ps.bestv[blockIdx.x] = bv_s[0];
    ps.besti[blockIdx.x] = bi_s[0];
  }
}

// A tall panel in one cooperative launch (all CTAs resident), one grid-wide
// barrier per column instead of a pivot kernel and an update kernel. The row
// interchanges are kept as a small permutation table (the positions a swap
// has touched and the physical row at each) instead of being carried out at
// once: a CTA updates the physical rows of its grid-stride range that are not
// yet pivot rows, and the pivot row of column c is read from its physical
// row, which no CTA writes during that step. Every CTA reduces the per-CTA
// partial maxima itself (larger magnitude, then the smaller position, the
// order of k_lu_panel) and applies the same table updates, so no CTA waits for
// another's pivot. After the last column CTA 0 moves the touched rows of the
// panel's columns to their final positions. Each entry takes the operations
// of k_lu_panel, so the factors are the same. Barrier waits are bounded; on
// time-out the kernel raises *err and returns.
struct PanelPerm {
  long pos[2 * kNb], row[2 * kNb];
  int cnt;
};

__device__ __forceinline__ long perm_row(const PanelPerm &pm, long pos) {
  for(int e = 0; e < pm.cnt; ++e)
    if(pm.pos[e] == pos)
      return pm.row[e];
  return pos;
}
__device__ __forceinline__ long perm_pos(const PanelPerm &pm, long row) {
  for(int e = 0; e < pm.cnt; ++e)
    if(pm.row[e] == row)
      return pm.pos[e];
  return row;
}
__device__ __forceinline__ void perm_set(PanelPerm &pm, long pos, long row) {
  for(int e = 0; e < pm.cnt; ++e)
    if(pm.pos[e] == pos) {
      pm.row[e] = row;
      return;
    }
  pm.pos[pm.cnt] = pos;
  pm.row[pm.cnt] = row;
  ++pm.cnt;
}

// grid-wide barrier on a counter that only grows: this CTA's arrival (a
// release add: the CTA's earlier writes, ordered before it by the CTA
// barrier, become visible with it), then a bounded wait with acquire loads
// for `target` arrivals
__device__ __forceinline__ bool grid_barrier(unsigned *bar, unsigned target, int *err) {
  __shared__ int ok_s;
  __syncthreads();
  if(threadIdx.x == 0) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(bar), "r"(1u) : "memory");
    int ok = 0;
    for(long it = 0; it < (1L << 22); ++it) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(bar) : "memory");
      if(v >= target) {
        ok = 1;
        break;
      }
      if((it & 63) == 63 && *(volatile int *)err)
        break;  // another CTA (or an earlier launch) gave up
      __nanosleep(32);  // fewer polls of the counter's line while the arrivals land
    }
    if(!ok)
      atomicExch(err, 1);
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

template <typename V>
__global__ void __launch_bounds__(kPanThreads) k_pan_coop(V *A, long ld, long n, long k, int nb, int *piv,
                                                          int *info, PanelScratch ps, unsigned *bar,
                                                          unsigned bar_base, int *err) {
  __shared__ V u[kNb];
  __shared__ PanelPerm pm;
  __shared__ long piv_row[kNb];  // physical rows of the pivots so far
  __shared__ double wv[kPanThreads / 32];
  __shared__ long wi[kPanThreads / 32];
  __shared__ long p_s;
  __shared__ double pv_s;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const unsigned G = gridDim.x;
  if(*(volatile int *)err)  // an earlier wait timed out: the factorization is void
    return;
  if(t == 0)
    pm.cnt = 0;
  // partial maximum of |A[col, r]|^2 over the active physical rows r of this
  // CTA (positions for ties), reduced over the CTA into ps.bestv / besti
  auto partial_max = [&](long col, int npiv) {
    double bv = -1.0;
    long bp = col;
    for(long r = k + blockIdx.x * (long)kPanThreads + t; r < n; r += (long)G * kPanThreads) {
      bool retired = false;
      for(int e = 0; e < npiv; ++e)
        retired |= piv_row[e] == r;
      if(retired)
        continue;
      const double v = mag2(A[col * ld + r]);
      if(v >= bv) {
        const long pos = perm_pos(pm, r);
        if(v > bv || pos < bp) {
          bv = v;
          bp = pos;
        }
      }
    }
#pragma unroll
    for(int h = 16; h > 0; h >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, h);
      const long op = __shfl_xor_sync(0xffffffffu, bp, h);
      if(ov > bv || (ov == bv && op < bp)) {
        bv = ov;
        bp = op;
      }
    }
    if(lane == 0) {
      wv[wid] = bv;
      wi[wid] = bp;
    }
    __syncthreads();
    if(t == 0) {
      for(int w = 1; w < kPanThreads / 32; ++w)
        if(wv[w] > bv || (wv[w] == bv && wi[w] < bp)) {
          bv = wv[w];
          bp = wi[w];
        }
      ps.bestv[blockIdx.x] = bv;
      ps.besti[blockIdx.x] = bp;
    }
  };
  __syncthreads();
  partial_max(k, 0);
  unsigned target = bar_base;
  for(int c = 0; c < nb; ++c) {
    const long col = k + c;
    target += G;
    if(!grid_barrier(bar, target, err))
      return;
    // the pivot: every CTA reduces all partial maxima (in CTA order)
    {
      double bv = -2.0;
      long bp = col;
      for(unsigned b = t; b < G; b += kPanThreads) {
        const double v = ps.bestv[b];
        const long i = ps.besti[b];
        if(v > bv || (v == bv && i < bp)) {
          bv = v;
          bp = i;
        }
      }
#pragma unroll
      for(int h = 16; h > 0; h >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, h);
        const long op = __shfl_xor_sync(0xffffffffu, bp, h);
        if(ov > bv || (ov == bv && op < bp)) {
          bv = ov;
          bp = op;
        }
      }
      if(lane == 0) {
        wv[wid] = bv;
        wi[wid] = bp;
      }
      __syncthreads();
      if(t == 0) {
        for(int w = 1; w < kPanThreads / 32; ++w)
          if(wv[w] > bv || (wv[w] == bv && wi[w] < bp)) {
            bv = wv[w];
            bp = wi[w];
          }
        if(blockIdx.x == 0) {
          piv[col] = (int)bp;
          if(bv <= 0.0 && *info == 0)
            *info = (int)col + 1;
        }
        // interchange positions col and bp in the table
        const long a = perm_row(pm, col), b = perm_row(pm, bp);
        if(bp != col) {
          perm_set(pm, col, b);
          perm_set(pm, bp, a);
        }
        piv_row[c] = b;
        p_s = b;
        pv_s = bv;
      }
      __syncthreads();
    }
    const long prow = p_s;
    if(t < nb)
      u[t] = A[(k + t) * ld + prow];
    __syncthreads();
    if(pv_s > 0.0) {
      const V inv = crecip(u[c]);
      for(long r = k + blockIdx.x * (long)kPanThreads + t; r < n; r += (long)G * kPanThreads) {
        bool retired = false;
        for(int e = 0; e <= c; ++e)
          retired |= piv_row[e] == r;
        if(retired)
          continue;
        V l = cmul(A[col * ld + r], inv);
        A[col * ld + r] = l;
        panel_row_update(A, ld, k, r, c, nb, l, u);
      }
    }
    if(c + 1 < nb) {
      __syncthreads();
      partial_max(col + 1, c + 1);
    }
  }
  target += G;
  if(!grid_barrier(bar, target, err) || blockIdx.x != 0)
    return;
  // CTA 0: the touched rows of the panel's columns to their final positions
  __shared__ V tmp[2 * kNb][kNb];
  const int cnt = pm.cnt;
  for(int idx = t; idx < cnt * nb; idx += kPanThreads) {
    const int e = idx / nb, j = idx - e * nb;
    tmp[e][j] = A[(k + j) * ld + pm.row[e]];
  }
  __syncthreads();
  for(int idx = t; idx < cnt * nb; idx += kPanThreads) {
    const int e = idx / nb, j = idx - e * nb;
    A[(k + j) * ld + pm.pos[e]] = tmp[e][j];
  }
}

// The cooperative panel with each CTA's rows held in shared memory for the
// whole panel: CTA b takes the contiguous rows k + b R .. k + (b + 1) R - 1
// (R = ceil((n - k) / G)), all nb columns of them, and writes them back after
// the last column. Besides its partial maximum a CTA publishes the row that
// holds it (its current values, all nb columns) in cand[b], so that after the
// barrier every CTA takes the pivot row from the winning CTA's slot: one
// grid-wide barrier and two small reads per column, no global traffic on the
// panel itself. The entries take the operations of k_lu_panel, in the same
// order, so the factors are the same bits.
template <typename V>
__global__ void __launch_bounds__(kPanThreads) k_pan_coop_sm(V *A, long ld, long n, long k, int nb, int *piv,
                                                             int *info, PanelScratch ps, V *cand,
                                                             unsigned *bar, unsigned bar_base, int *err) {
  extern __shared__ __align__(16) unsigned char pan_sm[];
  __shared__ V u[kNb];
  // the interchanges so far: the physical row at each position of the
  // panel's diagonal range (row_at), and the rows moved below it (position,
  // row; a later entry for the same position replaces an earlier one)
  __shared__ long row_at[kNb], ext_pos[kNb], ext_row[kNb];
  __shared__ int ext_cnt;
  __shared__ double wv[kPanThreads / 32];
  __shared__ long wi[kPanThreads / 32];
  __shared__ int wl[kPanThreads / 32];
  __shared__ long wr[kPanThreads / 32];
  __shared__ int rl_s;
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const long G = gridDim.x, b = blockIdx.x;
  const long R = (n - k + G - 1) / G, r0 = k + b * R, r1 = min(n, r0 + R);
  const int nr = (int)max(0L, r1 - r0);
  V *P = reinterpret_cast<V *>(pan_sm);                                 // P[c R + rl]
  long *posl = reinterpret_cast<long *>(pan_sm + sizeof(V) * (size_t)nb * R);  // position of local row rl
  unsigned char *retired = reinterpret_cast<unsigned char *>(posl + R);         // per local row
  if(*(volatile int *)err)
    return;
  if(t < nb)
    row_at[t] = k + t;
  if(t == 0)
    ext_cnt = 0;
  for(int c = 0; c < nb; ++c)
    for(int rl = t; rl < nr; rl += kPanThreads)
      P[c * R + rl] = A[(k + c) * ld + r0 + rl];
  for(int rl = t; rl < nr; rl += kPanThreads) {
    retired[rl] = 0;
    posl[rl] = r0 + rl;
  }
  __syncthreads();
  // partial maximum of column c over the active local rows (positions for
  // ties), and the row holding it published in cand[b]
  auto partial_max = [&](int c) {
    double bv = -1.0;
    long bp = k + c;
    int bl = -1;
    for(int rl = t; rl < nr; rl += kPanThreads) {
      if(retired[rl])
        continue;
      const double v = mag2(P[c * R + rl]);
      const long pos = posl[rl];
      if(v > bv || (v == bv && pos < bp)) {
        bv = v;
        bp = pos;
        bl = rl;
      }
    }
#pragma unroll
    for(int h = 16; h > 0; h >>= 1) {
      const double ov = __shfl_xor_sync(0xffffffffu, bv, h);
      const long op = __shfl_xor_sync(0xffffffffu, bp, h);
      const int ol = __shfl_xor_sync(0xffffffffu, bl, h);
      if(ov > bv || (ov == bv && op < bp)) {
        bv = ov;
        bp = op;
        bl = ol;
      }
    }
    if(lane == 0) {
      wv[wid] = bv;
      wi[wid] = bp;
      wl[wid] = bl;
    }
    __syncthreads();
    if(t == 0) {
      for(int w = 1; w < kPanThreads / 32; ++w)
        if(wv[w] > bv || (wv[w] == bv && wi[w] < bp)) {
          bv = wv[w];
          bp = wi[w];
          bl = wl[w];
        }
      ps.bestv[b] = bv;
      ps.besti[b] = bp;
      ps.bestr[b] = bl >= 0 ? r0 + bl : -1;
      rl_s = bl;
    }
    __syncthreads();
    if(t < nb && rl_s >= 0)
      cand[b * kNb + t] = P[t * R + rl_s];
  };
  partial_max(0);
  unsigned target = bar_base;
  double pv_s_local = 0.0;  // the pivot's |value|^2 (every thread reduces it)
  for(int c = 0; c < nb; ++c) {
    const long col = k + c;
    target += (unsigned)G;
    if(!grid_barrier(bar, target, err))
      return;
    {
      // every thread reduces the per-CTA maxima (the physical row rides
      // along), so the pivot row's load starts while thread 0 updates the
      // interchange tables
      double bv = -2.0;
      long bp = col, br = -1;
      int bw = 0;
      for(long w = t; w < G; w += kPanThreads) {
        const double v = __ldcg(ps.bestv + w);
        const long i = __ldcg(ps.besti + w), r = __ldcg(ps.bestr + w);
        if(v > bv || (v == bv && i < bp)) {
          bv = v;
          bp = i;
          br = r;
          bw = (int)w;
        }
      }
#pragma unroll
      for(int h = 16; h > 0; h >>= 1) {
        const double ov = __shfl_xor_sync(0xffffffffu, bv, h);
        const long op = __shfl_xor_sync(0xffffffffu, bp, h);
        const long orw = __shfl_xor_sync(0xffffffffu, br, h);
        const int ow = __shfl_xor_sync(0xffffffffu, bw, h);
        if(ov > bv || (ov == bv && op < bp)) {
          bv = ov;
          bp = op;
          br = orw;
          bw = ow;
        }
      }
      if(lane == 0) {
        wv[wid] = bv;
        wi[wid] = bp;
        wr[wid] = br;
        wl[wid] = bw;
      }
      __syncthreads();
      bv = wv[0];
      bp = wi[0];
      br = wr[0];
      bw = wl[0];
      for(int w = 1; w < kPanThreads / 32; ++w)
        if(wv[w] > bv || (wv[w] == bv && wi[w] < bp)) {
          bv = wv[w];
          bp = wi[w];
          br = wr[w];
          bw = wl[w];
        }
      if(t < nb)
        u[t] = __ldcg(cand + (long)bw * kNb + t);
      if(t == 0) {
        if(b == 0) {
          piv[col] = (int)bp;
          if(bv <= 0.0 && *info == 0)
            *info = (int)col + 1;
        }
        // interchange positions col and bp: the pivot row br (published by
        // the winning CTA) comes to col, the row at col goes to bp
        const long pr = br, a = row_at[c];
        if(bp != col) {
          row_at[c] = pr;
          if(bp - k < nb) {
            row_at[bp - k] = a;
          } else {
            ext_pos[ext_cnt] = bp;
            ext_row[ext_cnt] = a;
            ++ext_cnt;
          }
          if(a >= r0 && a < r1)
            posl[a - r0] = bp;
        }
        if(pr >= r0 && pr < r1) {
          retired[pr - r0] = 1;
          posl[pr - r0] = col;
        }
      }
      pv_s_local = bv;
      __syncthreads();
    }
    if(pv_s_local > 0.0) {
      const V inv = crecip(u[c]);
      for(int rl = t; rl < nr; rl += kPanThreads) {
        if(retired[rl])
          continue;
        const V l = cmul(P[c * R + rl], inv);
        P[c * R + rl] = l;
        for(int j = c + 1; j < nb; ++j) {
          const V uu = u[j];
          V a = P[j * R + rl];
          a.x = sub_rn(a.x, fma(l.x, uu.x, -mul_rn(l.y, uu.y)));
          a.y = sub_rn(a.y, fma(l.x, uu.y, mul_rn(l.y, uu.x)));
          P[j * R + rl] = a;
        }
      }
    }
    __syncthreads();
    if(c + 1 < nb)
      partial_max(c + 1);
  }
  // the rows back in place, then (CTA 0, after every CTA's rows are out) the
  // touched rows of the panel's columns to their final positions
  for(int c = 0; c < nb; ++c)
    for(int rl = t; rl < nr; rl += kPanThreads)
      A[(k + c) * ld + r0 + rl] = P[c * R + rl];
  target += (unsigned)G;
  if(!grid_barrier(bar, target, err) || b != 0)
    return;
  // (position, row) pairs: the diagonal range, then the moved rows below it
  // (the last entry of each position)
  __shared__ long fpos[2 * kNb], frow[2 * kNb];
  __shared__ int fcnt;
  if(t == 0) {
    int cnt = 0;
    for(int c = 0; c < nb; ++c)
      if(row_at[c] != k + c) {
        fpos[cnt] = k + c;
        frow[cnt] = row_at[c];
        ++cnt;
      }
    for(int e = ext_cnt - 1; e >= 0; --e) {
      bool later = false;
      for(int f = e + 1; f < ext_cnt; ++f)
        later |= ext_pos[f] == ext_pos[e];
      if(!later) {
        fpos[cnt] = ext_pos[e];
        frow[cnt] = ext_row[e];
        ++cnt;
      }
    }
    fcnt = cnt;
  }
  __syncthreads();
  V *tmp = P;  // [2 kNb][kNb], the shared rows are written back
  const int cnt = fcnt;
  for(int idx = t; idx < cnt * nb; idx += kPanThreads) {
    const int e = idx / nb, j = idx - e * nb;
    tmp[e * kNb + j] = __ldcg(A + (k + j) * ld + frow[e]);
  }
  __syncthreads();
  for(int idx = t; idx < cnt * nb; idx += kPanThreads) {
    const int e = idx / nb, j = idx - e * nb;
    A[(k + j) * ld + fpos[e]] = tmp[e * kNb + j];
  }
}

// The row interchanges of rows k .. k + nb - 1 (pivots piv[k .. k + nb), in
// order) as one permutation: (position, row) pairs, the new row at each
// position they move; pos_row[0] = the count, then the pairs. One warp: the
// interchanges are applied in order (nb <= 256 steps) to a table of the rows
// at positions k .. k + nb - 1 and to a list of the rows moved below them,
// whose last entry for a position counts; the lanes search that list
// together and emit the pairs in order (the table's positions ascending, then
// the list's live entries from the last one back).
constexpr int kPermMax = 256;  // interchanges per table
__global__ void k_lu_perm_table(const int *piv, long k, int nb, long *pos_row) {
  __shared__ long row_at[kPermMax], ext_pos[kPermMax], ext_row[kPermMax];
  __shared__ unsigned char live[kPermMax];
  const int lane = threadIdx.x;
  for(int c = lane; c < nb; c += 32)
    row_at[c] = k + c;
  __syncwarp();
  int ext = 0;
  for(int c = 0; c < nb; ++c) {
    const long p = piv[k + c];
    if(p == k + c)
      continue;
    if(p - k < nb) {
      if(lane == 0) {
        const long a = row_at[c];
        row_at[c] = row_at[p - k];
        row_at[p - k] = a;
      }
    } else {
      int last = -1;  // the latest list entry for position p
      for(int e = lane; e < ext; e += 32)
        if(ext_pos[e] == p)
          last = e;
      last = __reduce_max_sync(0xffffffffu, last);
      if(lane == 0) {
        const long a = row_at[c];
        row_at[c] = last >= 0 ? ext_row[last] : p;
        ext_pos[ext] = p;
        ext_row[ext] = a;
      }
      ++ext;
    }
    __syncwarp();
  }
  // list entries that no later entry for the same position overrides
  for(int e = lane; e < ext; e += 32) {
    bool later = false;
    for(int f = e + 1; f < ext; ++f)
      later |= ext_pos[f] == ext_pos[e];
    live[e] = !later;
  }
  __syncwarp();
  long cnt = 0;
  for(int c0 = 0; c0 < nb; c0 += 32) {  // table positions, ascending
    const int c = c0 + lane;
    const bool moved = c < nb && row_at[c] != k + c;
    const unsigned m = __ballot_sync(0xffffffffu, moved);
    if(moved) {
      const long at = cnt + __popc(m & ((1u << lane) - 1u));
      pos_row[1 + 2 * at] = k + c;
      pos_row[2 + 2 * at] = row_at[c];
    }
    cnt += __popc(m);
  }
  for(int e0 = ext - 1; e0 >= 0; e0 -= 32) {  // list entries, from the last one back
    const int e = e0 - lane;
    const bool take = e >= 0 && live[e];
    const unsigned m = __ballot_sync(0xffffffffu, take);
    if(take) {
      const long at = cnt + __popc(m & ((1u << lane) - 1u));
      pos_row[1 + 2 * at] = ext_pos[e];
      pos_row[2 + 2 * at] = ext_row[e];
    }
    cnt += __popc(m);
  }
  if(lane == 0)
    pos_row[0] = cnt;
}

// The permutation of k_lu_perm_table applied to the columns jlo .. jhi - 1
// other than slo .. shi - 1: a warp per column, each lane gathering its
// pairs' rows (loads issued together; consecutive positions on consecutive
// lanes) before any store.
template <typename V>
__global__ void __launch_bounds__(256) k_lu_permute(V *A, long ld, long jlo, long jhi, long slo, long shi,
                                                    const long *pos_row) {
  const long cnt = pos_row[0];
  const long warp = (blockIdx.x * (long)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  long j = jlo + warp;
  if(j >= slo)
    j += shi - slo;  // skip the panel's own columns
  if(j >= jhi)
    return;
  V *col = A + j * ld;
  constexpr int kPer = 2 * kPermMax / 32;
  V v[kPer];
#pragma unroll
  for(int i = 0; i < kPer; ++i) {
    const long e = lane + 32L * i;
    if(e < cnt)
      v[i] = col[pos_row[2 + 2 * e]];
  }
  __syncwarp();
#pragma unroll
  for(int i = 0; i < kPer; ++i) {
    const long e = lane + 32L * i;
    if(e < cnt)
      col[pos_row[1 + 2 * e]] = v[i];
  }
}

// U12 = L11^{-1} A12 (unit lower L11: rows and columns k .. k + nb - 1) for
// the columns jlo .. jhi - 1, one thread per column; products and
// differences written with explicit fused and unfused operations, as in the
// panels.
template <typename V>
__global__ void k_lu_trsm(V *A, long ld, long jlo, long jhi, long k, int nb) {
  __shared__ V L[kNb][kNb];
  for(int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    int r = idx % nb, c = idx / nb;
    L[r][c] = A[(k + c) * ld + k + r];
  }
  __syncthreads();
  const long j = jlo + blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(j >= jhi)
    return;
  V *col = A + j * ld + k;
  if(nb == kNb) {
    // the full block: the column's 32 loads issued together, the
    // substitution in registers, then the stores
    V xr[kNb];
#pragma unroll
    for(int r = 0; r < kNb; ++r)
      xr[r] = col[r];
#pragma unroll
    for(int r = 1; r < kNb; ++r) {
      V v = xr[r];
#pragma unroll
      for(int s = 0; s < r; ++s) {
        const V p = cmul(L[r][s], xr[s]);
        v.x = sub_rn(v.x, p.x);
        v.y = sub_rn(v.y, p.y);
      }
      xr[r] = v;
    }
#pragma unroll
    for(int r = 0; r < kNb; ++r)
      col[r] = xr[r];
    return;
  }
  V x[kNb];
  for(int r = 0; r < nb; ++r) {
    V v = col[r];
    for(int s = 0; s < r; ++s) {
      const V p = cmul(L[r][s], x[s]);
      v.x = sub_rn(v.x, p.x);
      v.y = sub_rn(v.y, p.y);
    }
    x[r] = v;
    col[r] = v;
  }
}

// A22 -= L21 U12 over rows/cols >= k + nb; 32x32 output tiles, 256 threads.
template <typename V>
__global__ void __launch_bounds__(256) k_lu_gemm(V *A, long ld, long n, long k, int nb) {
  __shared__ V Ls[32][kNb + 1];
  __shared__ V Us[kNb][32 + 1];
  const long r0 = k + nb + blockIdx.x * 32L, c0 = k + nb + blockIdx.y * 32L;
  const int t = threadIdx.x;
  for(int idx = t; idx < 32 * nb; idx += 256) {
    int rr = idx % 32, cc = idx / 32;
    long r = r0 + rr;
    V z;
    z.x = z.y = 0;
    Ls[rr][cc] = r < n ? A[(k + cc) * ld + r] : z;
  }
  for(int idx = t; idx < nb * 32; idx += 256) {
    int rr = idx % nb, cc = idx / nb;
    long c = c0 + cc;
    V z;
    z.x = z.y = 0;
    Us[rr][cc] = c < n ? A[c * ld + k + rr] : z;
  }
  __syncthreads();
  const int tr = t % 32, tc = t / 32;  // 4 columns per thread: tc, tc+8, tc+16, tc+24
  const long r = r0 + tr;
  if(r >= n)
    return;
  for(int q = 0; q < 4; ++q) {
    const int cc = tc + 8 * q;
    const long c = c0 + cc;
    if(c >= n)
      continue;
    V acc;
    acc.x = acc.y = 0;
    for(int s = 0; s < nb; ++s)
      acc = cfma(Ls[tr][s], Us[s][cc], acc);
    V a = A[c * ld + r];
    a.x -= acc.x;
    a.y -= acc.y;
    A[c * ld + r] = a;
  }
}

// y = P b, P the product of the row interchanges in order, as a gather:
// perm[i] is the row of b that the interchanges bring to row i.
template <typename V> __global__ void k_lu_gather(const V *b, V *y, const int *perm, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i < n)
    y[i] = b[perm[i]];
}

// dinv[i] = 1 / U[i][i] (the backward solve's divisions, done once)
template <typename V> __global__ void k_lu_diag_inv(const V *A, long ld, long n, V *dinv) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i < n)
    dinv[i] = crecip(A[i * ld + i]);
}

// perm (device, n entries) from the pivots of lu_factor: the interchanges
// applied in order to the row indices, on the host (one download of piv and
// one upload, after the factorization).
int lu_perm(om_context *ctx, const int *piv, long n, int *perm) {
  std::vector<int> hp((size_t)n), idx((size_t)n);
  cudaMemcpyAsync(hp.data(), piv, sizeof(int) * n, cudaMemcpyDeviceToHost, ctx->stream);
  const cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess) {
    ctx->err = std::string("LU pivots: ") + cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  for(long i = 0; i < n; ++i)
    idx[i] = (int)i;
  for(long r = 0; r < n; ++r) {
    const long p = hp[r];
    if(p > r && p < n)
      std::swap(idx[r], idx[p]);
  }
  cudaMemcpyAsync(perm, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, ctx->stream);
  // idx must outlive the copy
  const cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
  if(e2 != cudaSuccess) {
    ctx->err = std::string("LU permutation: ") + cudaGetErrorString(e2);
    return OM_ERR_CUDA;
  }
  return OM_OK;
}

// One block of kNb rows of a triangular solve in a single launch: every CTA
// solves the diagonal block from src[k .. k+nb) in shared memory (warp 0, a
// lane per row: forward with the unit lower factor, or backward with the upper
// factor and the reciprocals of its diagonal, dinv, computed once per
// factorization), then updates its rows [lo, hi) of src outside the
// block; CTA 0 writes the block's solution to dst. The rows read and the rows
// written are disjoint, so the CTAs need no ordering among themselves.
template <typename V> __device__ __forceinline__ V shfl_v(V a, int src) {
  a.x = __shfl_sync(0xffffffffu, a.x, src);
  a.y = __shfl_sync(0xffffffffu, a.y, src);
  return a;
}

template <typename V>
__global__ void __launch_bounds__(256) k_tri_block(const V *A, long ld, long k, int nb, V *src, V *dst,
                                                   long lo, long hi, int upper, const V *dinv) {
  __shared__ V Ad[kNb][kNb + 1];
  __shared__ V xs[kNb];
  for(int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x) {
    const int r = idx % nb, c = idx / nb;
    Ad[r][c] = A[(k + c) * ld + k + r];
  }
  __syncthreads();
  if(threadIdx.x < 32) {
    const int lane = threadIdx.x;
    V v;
    v.x = v.y = 0;
    V dl = v;  // lane c: 1 / U[c][c] of this block (backward solve)
    if(lane < nb) {
      v = src[k + lane];
      if(upper)
        dl = dinv[k + lane];
    }
    if(!upper) {
      for(int c = 0; c < nb; ++c) {
        const V xc = shfl_v(v, c);
        if(lane > c && lane < nb)
          v = cfma(Ad[lane][c], make_neg(xc), v);
      }
    } else {
      for(int c = nb - 1; c >= 0; --c) {
        if(lane == c)
          v = cmul(v, dl);
        const V xc = shfl_v(v, c);
        if(lane < c)
          v = cfma(Ad[lane][c], make_neg(xc), v);
      }
    }
    if(lane < nb)
      xs[lane] = v;
  }
  __syncthreads();
  if(blockIdx.x == 0 && threadIdx.x < nb)
    dst[k + threadIdx.x] = xs[threadIdx.x];
  const long i = lo + blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i < hi) {
    V v = src[i];
    if(nb == kNb) {  // a full block: the row's kNb loads issued together
      V a[kNb];
#pragma unroll
      for(int c = 0; c < kNb; ++c)
        a[c] = A[(k + c) * ld + i];
#pragma unroll
      for(int c = 0; c < kNb; ++c)
        v = cfma(a[c], make_neg(xs[c]), v);
    } else {
      for(int c = 0; c < nb; ++c)
        v = cfma(A[(k + c) * ld + i], make_neg(xs[c]), v);
    }
    src[i] = v;
  }
}

// A whole triangular sweep in one launch. CTA b owns the 32-row blocks
// r = b, b + G, b + 2G, ... (G CTAs); its seven compute warps take the owned
// blocks in turn (local block q to warp q % 8) and keep their running values
// in shared memory. A warp walks the sweep's column blocks in order: once
// block j's solution is published it applies that block's columns to each of
// its rows still to be solved (the next one to be solved first), and when a
// block has received every column it needs, the warp solves its diagonal
// block and publishes the solution (the values to dst, then flags[j] = this
// sweep's epoch). An eighth warp polls the flags in sweep order and counts the
// published blocks in shared memory for the others. Every row takes the same
// operations in the same order as with k_tri_block (one launch per block),
// so the results are the same bits. The epoch (sync[0]) is read at the start
// and moved on by the last CTA to finish, so a captured sweep replays. Waits
// are bounded by a clock budget; on time-out the kernel raises *err, and a
// sweep that starts with *err raised does nothing.
constexpr int kSweepWarps = 7;
constexpr int kSweepThreads = 32 * (kSweepWarps + 1);

__device__ __forceinline__ bool clock_wait_expired(long long t0) {
  return clock64() - t0 > (1LL << 32);  // about two seconds
}

template <typename V>
__global__ void __launch_bounds__(kSweepThreads, 1) k_tri_sweep(const V *A, long ld, long n, const V *src, V *dst,
                                                             int upper, const V *dinv, unsigned *flags,
                                                             unsigned long long *msg, unsigned *sync, int *err) {
  // complex64: a solved block travels as 64 words (epoch << 32 | the bits of
  // one real or imaginary part; single-copy atomic 64-bit stores), so a
  // reader that sees the epoch in both of a lane's words has that lane's
  // value, with no flag and no fence. complex128 publishes flags[j] after a
  // fence and readers take the values from dst.
  constexpr bool kPacked = sizeof(V) == 8;
  constexpr int kRing = 64;  // steps of solved values held in shared memory (complex64)
  __shared__ V xring[kPacked ? kRing * kNb : 1];
  __shared__ volatile int prog[kSweepWarps];  // steps each compute warp has finished
  extern __shared__ __align__(16) unsigned char sweep_sm[];
  V *vals = reinterpret_cast<V *>(sweep_sm);
  __shared__ volatile int ready;    // sweep steps whose solution is published
  __shared__ volatile int abort_s;
  __shared__ unsigned epoch_s;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long nblk = (n + kNb - 1) / kNb;
  const long G = gridDim.x, b = blockIdx.x;
  const int ob = (int)((nblk - b + G - 1) / G);  // owned blocks r = b + q G, q < ob
  if(threadIdx.x == 0) {
    ready = 0;
    abort_s = *(volatile int *)err;
    epoch_s = *(volatile unsigned *)sync;
  }
  // a compute warp's progress starts at 0 when it has blocks (set before the
  // poller can start, so that it never runs the ring past a warp's steps)
  if(threadIdx.x < kSweepWarps)
    prog[threadIdx.x] = ob > (int)threadIdx.x ? 0 : 0x7fffffff;
  __syncthreads();
  const unsigned epoch = epoch_s;
  // sweep step of column block j, and the block solved at step s
  auto step_of = [&](long j) { return upper ? nblk - 1 - j : j; };
  // the diagonal block of local block q (lane: its row), loaded into a[]
  auto load_diag = [&](int q, V(&a)[kNb]) {
    const long kk = (b + q * G) * kNb;
    const int nbr = (int)min((long)kNb, n - kk);
#pragma unroll
    for(int c = 0; c < kNb; ++c)
      if(c < nbr && lane < nbr)
        a[c] = A[(kk + c) * ld + kk + lane];
  };
  auto solve_publish = [&](int q, V(&a)[kNb], bool loaded) {
    const long r = b + q * G, kk = r * kNb;
    const int nbr = (int)min((long)kNb, n - kk);
    V v = vals[q * kNb + lane];
    if(!loaded)
      load_diag(q, a);
    // (fully unrolled over kNb columns so that a[] stays in registers; the
    // columns past nbr change nothing)
    if(!upper) {
#pragma unroll
      for(int c = 0; c < kNb; ++c) {
        const V xc = shfl_v(v, c);
        if(lane > c && lane < nbr)
          v = cfma(a[c], make_neg(xc), v);
      }
    } else {
      V dl;
      dl.x = dl.y = 0;
      if(lane < nbr)
        dl = dinv[kk + lane];
#pragma unroll
      for(int c = kNb - 1; c >= 0; --c) {
        if(lane == c && c < nbr)
          v = cmul(v, dl);
        const V xc = shfl_v(v, c);
        if(lane < c && c < nbr)
          v = cfma(a[c], make_neg(xc), v);
      }
    }
    if(lane < nbr)
      dst[kk + lane] = v;
    if constexpr(kPacked) {
      const unsigned long long tag = (unsigned long long)epoch << 32;
      volatile unsigned long long *mm = msg + (r * kNb + lane) * 2;
      mm[0] = tag | __float_as_uint((float)v.x);
      mm[1] = tag | __float_as_uint((float)v.y);
    } else {
      __threadfence();
      __syncwarp();
      if(lane == 0)
        atomicExch(flags + r, epoch);
    }
  };
  if(!abort_s && warp == kSweepWarps) {
    // the poller: steps this CTA still needs (forward: the columns left of its
    // last block; backward: those right of its first block)
    const long need = upper ? nblk - 1 - b : b + (long)(ob - 1) * G;
    if constexpr(kPacked) {
      // the whole warp polls block j's 64 words, then stores the values in
      // the ring once every compute warp is done with the step kRing back
      for(long st = 0; st < need; ++st) {
        const long j = upper ? nblk - 1 - st : st;
        const long long t0 = clock64();
        bool ok = true;
        for(;;) {
          int lag = 0x7fffffff;
#pragma unroll
          for(int w = 0; w < kSweepWarps; ++w)
            lag = min(lag, prog[w]);
          if(lag > st - kRing)
            break;
          if(abort_s || clock_wait_expired(t0)) {
            ok = false;
            break;
          }
          __nanosleep(20);
        }
        unsigned long long m0 = 0, m1 = 0;
        const volatile unsigned long long *mm = msg + (j * kNb + lane) * 2;
        while(ok) {
          m0 = mm[0];
          m1 = mm[1];
          if(__all_sync(0xffffffffu, (unsigned)(m0 >> 32) == epoch && (unsigned)(m1 >> 32) == epoch))
            break;
          if(abort_s || *(volatile int *)err || clock_wait_expired(t0))
            ok = false;
          __nanosleep(16);
        }
        if(!__all_sync(0xffffffffu, ok)) {
          if(lane == 0) {
            atomicExch(err, 1);
            abort_s = 1;
          }
          break;
        }
        V x;
        x.x = __uint_as_float((unsigned)m0);
        x.y = __uint_as_float((unsigned)m1);
        xring[(st % kRing) * kNb + lane] = x;
        __syncwarp();
        __threadfence_block();
        if(lane == 0)
          ready = (int)(st + 1);
      }
    } else if(lane == 0) {
      for(long st = 0; st < need; ++st) {
        const long j = upper ? nblk - 1 - st : st;
        const long long t0 = clock64();
        bool ok = true;
        while(*(volatile unsigned *)(flags + j) != epoch) {
          if(abort_s || *(volatile int *)err || clock_wait_expired(t0)) {
            ok = false;
            break;
          }
        }
        if(!ok) {
          atomicExch(err, 1);
          abort_s = 1;
          break;
        }
        __threadfence();
        ready = (int)(st + 1);
      }
    }
  } else if(!abort_s && warp < kSweepWarps) {
    for(int q = warp; q < ob; q += kSweepWarps) {
      const long row = (b + q * G) * kNb + lane;
      V v;
      v.x = v.y = 0;
      if(row < n)
        v = src[row];
      vals[q * kNb + lane] = v;
    }
    __syncwarp();
    // this warp's blocks in the order they become ready
    const int nq = ob > warp ? (ob - warp + kSweepWarps - 1) / kSweepWarps : 0;
    auto qi = [&](int t) { return upper ? warp + (nq - 1 - t) * kSweepWarps : warp + t * kSweepWarps; };
    int first = 0;  // the warp's blocks before `first` are solved
    if(nq > 0 && step_of(b + qi(0) * G) == 0) {  // the sweep's first block
      V dg[kNb];
      solve_publish(qi(0), dg, false);
      first = 1;
    }
    for(long st = 0; first < nq; ++st) {
      const long j = upper ? nblk - 1 - st : st;
      const long k = j * kNb;
      const int nbj = (int)min((long)kNb, n - k);
      // The next block to be solved (the first unsolved one) is on the
      // critical path: its tile of column block j, and its diagonal block
      // when it is solved at this step (complex64: registers allow both), are
      // loaded before block j's solution is in.
      const int t0 = first, q0 = qi(t0);
      const long r0c = b + q0 * G, i0 = r0c * kNb + lane;
      const bool solve0 = step_of(r0c) == st + 1;
      V a0[kNb], dg[kNb];
#pragma unroll
      for(int c = 0; c < kNb; ++c) {
        a0[c].x = a0[c].y = 0;
        if(c < nbj && i0 < n)
          a0[c] = A[(k + c) * ld + i0];
      }
      constexpr bool kPreDiag = sizeof(V) == 8;
      if(kPreDiag && solve0)
        load_diag(q0, dg);
      // wait for block j's solution
      const long long w0 = clock64();
      bool ok = true;
      while(ready <= st) {
        if(abort_s || clock_wait_expired(w0)) {
          ok = false;
          break;
        }
        __nanosleep(20);
      }
      if(!__all_sync(0xffffffffu, ok)) {
        if(lane == 0) {
          atomicExch(err, 1);
          abort_s = 1;
        }
        break;
      }
      __threadfence_block();
      V xl;
      xl.x = xl.y = 0;
      if(lane < nbj) {
        if constexpr(kPacked)
          xl = xring[(st % kRing) * kNb + lane];
        else
          xl = __ldcg(dst + k + lane);
      }
      {
        V v = vals[q0 * kNb + lane];
#pragma unroll
        for(int c = 0; c < kNb; ++c) {
          const V xc = shfl_v(xl, c);
          if(c < nbj && i0 < n)
            v = cfma(a0[c], make_neg(xc), v);
        }
        vals[q0 * kNb + lane] = v;
        __syncwarp();
        if(solve0) {  // every column this block needs is in
          solve_publish(q0, dg, kPreDiag);
          ++first;
        }
      }
      // the warp's other blocks (none of them is complete at this step)
      for(int t = t0 + 1; t < nq; ++t) {
        const int q = qi(t);
        const long r = b + q * G, i = r * kNb + lane;
        // (every lane takes part in the shuffles; rows past n stay unused)
        V v = vals[q * kNb + lane];
        if(nbj == kNb) {  // two halves of 16 loads issued together
#pragma unroll
          for(int h = 0; h < kNb; h += kNb / 2) {
            V a[kNb / 2];
#pragma unroll
            for(int c = 0; c < kNb / 2; ++c) {
              a[c].x = a[c].y = 0;
              if(i < n)
                a[c] = A[(k + h + c) * ld + i];
            }
#pragma unroll
            for(int c = 0; c < kNb / 2; ++c)
              v = cfma(a[c], make_neg(shfl_v(xl, h + c)), v);
          }
        } else {
          for(int c = 0; c < nbj; ++c) {
            const V xc = shfl_v(xl, c);
            if(i < n)
              v = cfma(A[(k + c) * ld + i], make_neg(xc), v);
          }
        }
        vals[q * kNb + lane] = v;
        __syncwarp();
      }
      if(lane == 0)
        prog[warp] = first < nq ? (int)(st + 1) : 0x7fffffff;
    }
    if(lane == 0)  // (done, or given up)
      prog[warp] = 0x7fffffff;
  }
  __syncthreads();
  if(threadIdx.x == 0) {  // the last CTA out moves the epoch on
    __threadfence();
    if(atomicAdd(sync + 1, 1u) == (unsigned)G - 1) {
      sync[1] = 0;
      __threadfence();
      atomicAdd(sync, 1u);
    }
  }
}

// Complex64 LU with tensor-core updates, blocked in two levels (the order of
// LAPACK's blocked getrf): each block of kTcBlock columns is factored as a
// tall panel, in panels of kNb columns whose interchanges and updates stay
// inside the block; then the block's interchanges are applied to the columns
// outside it, its rows of U to the right are solved (L11^{-1} A12, kNb rows
// at a time), and the trailing matrix takes one rank-kTcBlock update, so that
// it is read and written once per kTcBlock columns instead of once per kNb.
// The pivots are those of the unblocked order (each panel's pivot search sees
// fully updated columns); the roundings differ.
constexpr long kTcBlock = 256;
static_assert(kTcBlock <= kPermMax, "a block's interchanges fit one permutation table");

// The interchanges of rows k .. k + nb - 1 on the columns jlo .. jhi - 1
// other than slo .. shi - 1 (inside that range): one permutation, gathered
// before it is stored, instead of nb dependent swaps per column.
template <typename V>
void lu_interchange(om_context *ctx, V *A, long n, long jlo, long jhi, long slo, long shi, long k, int nb,
                    const int *piv, long *ptab) {
  const long cols = (jhi - jlo) - (shi - slo);
  if(cols <= 0)
    return;
  k_lu_perm_table<<<1, 32, 0, ctx->stream>>>(piv, k, nb, ptab);
  k_lu_permute<V><<<blocks_for(cols, 8), 256, 0, ctx->stream>>>(A, n, jlo, jhi, slo, shi, ptab);
  ctx->last_launches += 2;
}

template <typename Panel>
void lu_blocked_tc(om_context *ctx, float2 *A, long n, int *piv, int *info, Panel &panel, void *split, long *ptab) {
  for(long K = 0; K < n; K += kTcBlock) {
    const long W = std::min<long>(kTcBlock, n - K), KE = K + W;
    for(long k = K; k < KE; k += kNb) {
      const int nb = (int)std::min<long>(kNb, KE - k);
      const long kn = k + nb;
      panel(k, nb);
      if(W > nb) {  // the block's other columns
        lu_interchange<float2>(ctx, A, n, K, KE, k, kn, k, nb, piv, ptab);
      }
      if(kn < KE) {  // the block's later columns: U rows, then all rows below
        k_lu_trsm<float2><<<blocks_for(KE - kn, 128), 128, 0, ctx->stream>>>(A, n, kn, KE, k, nb);
        ctx->last_launches++;
        launch_cgemm_sub_tc_split(ctx, A + k * n + kn, n, A + kn * n + k, n, A + kn * n + kn, n, n - kn,
                                  KE - kn, nb, split, info + 1);
      }
    }
    if(W < n) {  // the block's interchanges on the columns left and right of it
      lu_interchange<float2>(ctx, A, n, 0, n, K, KE, K, (int)W, piv, ptab);
    }
    const long rest = n - KE;
    if(rest <= 0)
      continue;
    for(long k = K; k < KE; k += kNb) {  // U12 = L11^{-1} A12
      const int nb = (int)std::min<long>(kNb, KE - k);
      const long kn = k + nb;
      k_lu_trsm<float2><<<blocks_for(rest, 128), 128, 0, ctx->stream>>>(A, n, KE, n, k, nb);
      ctx->last_launches++;
      if(kn < KE)
        launch_cgemm_sub_tc_split(ctx, A + k * n + kn, n, A + KE * n + k, n, A + KE * n + kn, n, KE - kn,
                                  rest, nb, split, info + 1);
    }
    timer_begin(ctx, ctx->ev_luu);
    launch_cgemm_sub_tc_split(ctx, A + K * n + KE, n, A + KE * n + K, n, A + KE * n + KE, n, rest, rest,
                              (int)W, split, info + 1);
    timer_end(ctx, ctx->ev_luu);
  }
}

// info[0]: first zero pivot (1-based) or 0; info[1]: set when a wait timed
// out (a tensor-core trailing update or a cooperative panel's barrier).
template <typename V>
int lu_factor(om_context *ctx, V *A, long n, int *piv, int *info) {
  cudaMemsetAsync(info, 0, 2 * sizeof(int), ctx->stream);
  Work ws;
  ws.ctx = ctx;
  PanelScratch ps{};
  const int maxblk = 4 * ctx->sm_count;
  size_t split_bytes = 0;  // the pre-split operands of the tensor-core updates (the largest)
  if constexpr(std::is_same<V, float2>::value)
    if(ctx->lu_tc)
      split_bytes = cgemm_sub_tc_split_bytes(n, n, (int)kTcBlock);
  const size_t pan_bytes =
      n >= kCoopPanel ? maxblk * (sizeof(double) + 2 * sizeof(long) + kNb * sizeof(V)) + kNb * sizeof(V) + 6 * 256
                      : 0;
  void *split = nullptr;
  unsigned *bar = nullptr, bar_base = 0;  // the cooperative panels' barrier counter
  V *cand = nullptr;                       // their per-CTA candidate pivot rows
  // CTAs of one cooperative panel launch: one per SM. The panel's rows stay
  // in shared memory when the tallest panel's share fits (coop_smem bytes).
  int coop_grid = 0;
  size_t coop_smem = 0;
  if(ctx->lu_persist != 2 && n >= kCoopPanel) {
    int per_sm = 0, coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
    // rows a CTA holds: n / G for the tallest panel, at least 64 (see below)
    const long R = std::max<long>((n + ctx->sm_count - 1) / ctx->sm_count, 64);
    const size_t sm = std::max((sizeof(V) * kNb + sizeof(long) + 1) * (size_t)R, sizeof(V) * 2 * kNb * kNb);
    if(coop && ctx->lu_persist == 1 && sm <= 220 * 1024 &&
       cudaFuncSetAttribute(k_pan_coop_sm<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm) ==
           cudaSuccess &&
       cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pan_coop_sm<V>, kPanThreads, sm) ==
           cudaSuccess &&
       per_sm >= 1) {
      coop_grid = ctx->sm_count;
      coop_smem = sm;
    } else if(coop && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_pan_coop<V>, kPanThreads, 0) ==
                          cudaSuccess) {
      coop_grid = std::min(per_sm, 1) * ctx->sm_count;
    }
    cudaGetLastError();
  }
  long *ptab = nullptr;  // the row-interchange permutation table
  {
    const size_t ptab_bytes = sizeof(long) * (1 + 4 * kPermMax);
    const int rc = alloc_work(ctx, ws, pan_bytes + split_bytes + ptab_bytes + 512);
    if(rc)
      return rc;
    size_t off = 0;
    ptab = ws.take<long>(1 + 4 * kPermMax, off);
    if(pan_bytes) {
      ps.bestv = ws.take<double>(maxblk, off);
      ps.besti = ws.take<long>(maxblk, off);
      ps.bestr = ws.take<long>(maxblk, off);
      ps.prow = ws.take<V>(kNb, off);
      bar = ws.take<unsigned>(1, off);
      cand = ws.take<V>((size_t)maxblk * kNb, off);
      cudaMemsetAsync(bar, 0, sizeof(unsigned), ctx->stream);
    }
    if(split_bytes)
      split = ws.take<unsigned char>(split_bytes, off);
  }
  timer_begin(ctx, ctx->ev_luf);
  // LU of the panel A[k:n, k:k+nb) with its row interchanges inside the panel
  auto panel = [&](long k, int nb) {
    timer_begin(ctx, ctx->ev_lup);
    const long rows = n - k;
    if((rows >= kTallPanel || (coop_smem && rows >= kCoopPanel)) && coop_grid > 0) {
      int *err = info + 1;
      cudaError_t e;
      if(coop_smem) {  // rows in shared memory, 64 rows a CTA at least
        ps.nblk = (int)std::min<long>(coop_grid, (rows + 63) / 64);
        const long R = (rows + ps.nblk - 1) / ps.nblk;
        const size_t sm = std::max((sizeof(V) * nb + sizeof(long) + 1) * (size_t)R, sizeof(V) * 2 * kNb * kNb);
        void *args[] = {&A, (void *)&n, (void *)&n, (void *)&k, (void *)&nb, &piv, &info, &ps, &cand, &bar,
                        &bar_base, &err};
        e = cudaLaunchCooperativeKernel((const void *)k_pan_coop_sm<V>, dim3(ps.nblk), dim3(kPanThreads), args,
                                        sm, ctx->stream);
      } else {
        ps.nblk = (int)std::min<long>(coop_grid, (rows + kPanThreads - 1) / kPanThreads);
        void *args[] = {&A, (void *)&n, (void *)&n, (void *)&k, (void *)&nb, &piv, &info, &ps, &bar, &bar_base,
                        &err};
        e = cudaLaunchCooperativeKernel((const void *)k_pan_coop<V>, dim3(ps.nblk), dim3(kPanThreads), args, 0,
                                        ctx->stream);
      }
      if(e == cudaSuccess) {
        bar_base += (unsigned)(nb + 1) * (unsigned)ps.nblk;
        ctx->last_launches++;
        timer_end(ctx, ctx->ev_lup);
        return;
      }
      cudaGetLastError();  // refused: the per-column kernels below
      coop_grid = 0;
    }
    if(rows >= kTallPanel) {
      ps.nblk = (int)std::min<long>(maxblk, (rows + kPanThreads - 1) / kPanThreads);
      k_pan_max<V><<<ps.nblk, kPanThreads, 0, ctx->stream>>>(A, n, n, k, ps);
      for(int c = 0; c < nb; ++c) {
        k_pan_pivot<V><<<1, kNb, 0, ctx->stream>>>(A, n, k, c, nb, piv, info, ps);
        k_pan_update<V><<<ps.nblk, kPanThreads, 0, ctx->stream>>>(A, n, n, k, c, nb, ps);
      }
      ctx->last_launches += 1 + 2 * nb;
    } else {
      k_lu_panel<V><<<1, 1024, 0, ctx->stream>>>(A, n, n, k, nb, piv, info);
      ctx->last_launches++;
    }
    timer_end(ctx, ctx->ev_lup);
  };
  if constexpr(std::is_same<V, float2>::value) {
    if(ctx->lu_tc) {
      lu_blocked_tc(ctx, A, n, piv, info, panel, split, ptab);
      timer_end(ctx, ctx->ev_luf);
      return OM_OK;
    }
  }
  for(long k = 0; k < n; k += kNb) {
    const int nb = (int)std::min<long>(kNb, n - k);
    panel(k, nb);
    lu_interchange<V>(ctx, A, n, 0, n, k, k + nb, k, nb, piv, ptab);
    const long rest = n - k - nb;
    if(rest > 0) {
      k_lu_trsm<V><<<blocks_for(rest, 128), 128, 0, ctx->stream>>>(A, n, k + nb, n, k, nb);
      dim3 g((unsigned)((rest + 31) / 32), (unsigned)((rest + 31) / 32));
      timer_begin(ctx, ctx->ev_luu);
      k_lu_gemm<V><<<g, 256, 0, ctx->stream>>>(A, n, n, k, nb);
      timer_end(ctx, ctx->ev_luu);
      ctx->last_launches += 2;
    }
  }
  timer_end(ctx, ctx->ev_luf);
  return OM_OK;
}

// b := A^{-1} b with A = P^T L U from lu_factor, perm from lu_perm and dinv
// from k_lu_diag_inv; y: n entries of scratch. 2 + 2 ceil(n / kNb) launches,
// all stream-ordered (capturable as a graph): y = P b, the forward solve from
// y into b, the backward solve from b into y, and y copied back to b.
// Workspace of the one-launch sweeps: flags (one per 32-row block, set to
// all ones) and the epoch / finished-CTA pair.
// Workspace of the one-launch sweeps: the complex64 messages (64 words of 8
// bytes per 32-row block), flags (one per block) and the epoch / finished-CTA
// pair; messages and flags start as all ones (an epoch never reached).
inline size_t sweep_ws_words(long n) {
  const size_t nblk = (size_t)((n + kNb - 1) / kNb);
  return nblk * 2 * kNb * 2 + nblk + 2;
}
inline void sweep_ws_init(om_context *ctx, unsigned *ws, long n) {
  const size_t nblk = (size_t)((n + kNb - 1) / kNb);
  cudaMemsetAsync(ws, 0xFF, (nblk * 2 * kNb * 2 + nblk) * sizeof(unsigned), ctx->stream);
  cudaMemsetAsync(ws + nblk * 2 * kNb * 2 + nblk, 0, 2 * sizeof(unsigned), ctx->stream);
}

template <typename V>
int lu_solve_vec(om_context *ctx, const V *A, long n, const int *perm, const V *dinv, V *b, V *y,
                 unsigned *sweep_ws = nullptr, int *err = nullptr) {
  k_lu_gather<V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(b, y, perm, n);
  int launches = 1;
  if(ctx->lu_persist != 2 && sweep_ws && err) {
    const long nblk = (n + kNb - 1) / kNb;
    const long G = std::min<long>(ctx->sm_count, nblk);
    const size_t smem = sizeof(V) * kNb * (size_t)((nblk + G - 1) / G);
    unsigned long long *msg = reinterpret_cast<unsigned long long *>(sweep_ws);
    unsigned *flags = sweep_ws + nblk * 2 * kNb * 2, *sync = flags + nblk;
    if(smem > 48 * 1024)
      cudaFuncSetAttribute(k_tri_sweep<V>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    k_tri_sweep<V><<<(unsigned)G, kSweepThreads, smem, ctx->stream>>>(A, n, n, y, b, 0, dinv, flags, msg, sync,
                                                                      err);
    k_tri_sweep<V><<<(unsigned)G, kSweepThreads, smem, ctx->stream>>>(A, n, n, b, y, 1, dinv, flags, msg, sync,
                                                                      err);
    k_scale_copy<V, V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(y, 1.0, b, n);
    launches += 3;
    ctx->last_launches += launches;
    return launches;
  }
  for(long k = 0; k < n; k += kNb) {
    const int nb = (int)std::min<long>(kNb, n - k);
    const long rows = n - k - nb;
    k_tri_block<V><<<(unsigned)std::max<long>(1, blocks_for(rows, 256)), 256, 0, ctx->stream>>>(
        A, n, k, nb, y, b, k + nb, n, 0, dinv);
    ++launches;
  }
  for(long k = ((n - 1) / kNb) * kNb; k >= 0; k -= kNb) {
    const int nb = (int)std::min<long>(kNb, n - k);
    k_tri_block<V><<<(unsigned)std::max<long>(1, blocks_for(k, 256)), 256, 0, ctx->stream>>>(
        A, n, k, nb, b, y, 0, k, 1, dinv);
    ++launches;
  }
  k_scale_copy<V, V><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(y, 1.0, b, n);
  ++launches;
  ctx->last_launches += launches;
  return launches;
}

}  // namespace

// `products` inner FP32 GMRES products y = S x on device buffers, the bf16
// copy made by the first one when the context's inner_half is set (the test
// entry point om_matvec_inner_c64).
int inner_products(om_context *ctx, const float2 *S, long n, const float2 *x, float2 *y, int products) {
  Work w;
  w.ctx = ctx;
  const size_t ld = (size_t)(n + 3) / 4 * 4;
  const size_t part = (size_t)mv_nsplit(ctx, n) * n;
  int rc = alloc_work(ctx, w, sizeof(float2) * part + sizeof(Bf16c) * ld * n + 1024);
  if(rc)
    return rc;
  size_t off = 0;
  float2 *pt = w.take<float2>(part, off);
  Bf16Copy hc;
  if(ctx->inner_half) {
    hc.H = w.take<Bf16c>(ld * n, off);
    hc.ld = (long)ld;
  }
  for(int p = 0; p < products; ++p)
    matvec_inner(ctx, S, n, &hc, x, pt, y);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e == cudaSuccess)
    e = cudaGetLastError();
  if(e != cudaSuccess) {
    ctx->err = std::string("inner product: ") + cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  return OM_OK;
}

// Direct solve of S X = Q for the given harmonic. The FP64 matrix is factored
// in a copy (S stays available for residuals and repeated solves).
int solve_lu_rhs(om_problem *pr, int harmonic, const double2 *b, double2 *x, om_solve_stats *st) {
  om_context *ctx = pr->ctx;
  const long n = pr->n;
  if(pr->S_prec[harmonic] != OM_C128) {
    ctx->err = "LU solve needs the complex128 matrix";
    return OM_ERR_STATE;
  }
  Work w;
  w.ctx = ctx;
  size_t bytes = sizeof(double2) * ((size_t)n * n + 2 * n) + sizeof(int) * (2 * n + 2) +
                 sizeof(unsigned) * sweep_ws_words(n) + 2048;
  int rc = alloc_work(ctx, w, bytes);
  if(rc)
    return rc;
  size_t off = 0;
  double2 *A = w.take<double2>((size_t)n * n, off);
  double2 *y = w.take<double2>(n, off);
  int *piv = w.take<int>(n, off);
  int *info = w.take<int>(2, off);
  int *perm = w.take<int>(n, off);
  double2 *dinv = w.take<double2>(n, off);
  unsigned *sweep = w.take<unsigned>(sweep_ws_words(n), off);
  sweep_ws_init(ctx, sweep, n);
  cudaMemcpyAsync(A, pr->d_S[harmonic], sizeof(double2) * (size_t)n * n, cudaMemcpyDeviceToDevice,
                  ctx->stream);
  rc = lu_factor<double2>(ctx, A, n, piv, info);
  if(!rc)
    rc = lu_perm(ctx, piv, n, perm);
  if(rc)
    return rc;
  k_lu_diag_inv<double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(A, n, n, dinv);
  ctx->last_launches++;
  cudaMemcpyAsync(x, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->stream);
  timer_begin(ctx, ctx->ev_lus);
  lu_solve_vec<double2>(ctx, A, n, perm, dinv, x, y, sweep, info + 1);
  timer_end(ctx, ctx->ev_lus);
  int hinfo[2] = {0, 0};
  cudaMemcpyAsync(hinfo, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if(hinfo[1]) {
    ctx->err = "LU kernel wait timed out (panel barrier or triangular sweep)";
    return OM_ERR_CUDA;
  }
  if(hinfo[0]) {
    ctx->err = "singular matrix: zero pivot at column " + std::to_string(hinfo[0]);
    return OM_ERR_SINGULAR;
  }
  if(st) {
    st->iterations = 0;
    st->inner_iterations = 0;
    st->rel_residual = 0.0;
  }
  return OM_OK;
}

int solve_gmres_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                    double2 *x, om_solve_stats *st) {
  om_context *ctx = pr->ctx;
  int it = 0;
  double rr = 0;
  int rc;
  if(pr->S_prec[harmonic] == OM_C128) {
    rc = gmres64<double2>(ctx, (const double2 *)pr->d_S[harmonic], pr->n, b, x, o->tol,
                          o->max_iter, o->restarts, nullptr, &it, &rr);
  } else if(pr->S_prec[harmonic] == OM_ACA) {  // Gmres_Zcomp role
    const AcaOp op = aca_op(pr, harmonic);
    rc = gmres64<AcaOp>(ctx, &op, pr->n, b, x, o->tol, o->max_iter, o->restarts, nullptr, &it, &rr);
  } else  // FP64 GMRES on the complex64 system
    rc = gmres64<float2>(ctx, (const float2 *)pr->d_S32[harmonic], pr->n, b, x, o->tol,
                         o->max_iter, o->restarts, nullptr, &it, &rr);
  if(st) {
    st->iterations = it;
    st->inner_iterations = 0;
    st->rel_residual = rr;
  }
  if(rc == OM_ERR_NOT_CONVERGED)
    ctx->err = "GMRES did not reach the requested tolerance";
  return rc;
}

// Precision form: FP64 outer FGMRES whose residuals use the complex64 matrix
// in FP64 arithmetic, with a fixed-length FP32 GMRES on the same matrix as the
// flexible preconditioner.
int solve_fgmres_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                     double2 *x, om_solve_stats *st) {
  om_context *ctx = pr->ctx;
  const float2 *S32 = (const float2 *)pr->d_S32[harmonic];
  InnerGmres32 inner(ctx, S32, pr->n, std::max(1, o->inner_iter), o->inner_tol);
  int rc = inner.init();
  if(rc)
    return rc;
  int it = 0;
  double rr = 0;
  const int outer_m = std::max(1, std::min(o->max_iter, 32));
  rc = gmres64<float2>(ctx, S32, pr->n, b, x, o->tol, outer_m, o->restarts, &inner, &it, &rr);
  if(st) {
    st->iterations = it;
    st->inner_iterations = inner.total;
    st->rel_residual = rr;
  }
  if(rc == OM_ERR_NOT_CONVERGED)
    ctx->err = "FGMRES did not reach the requested tolerance";
  return rc;
}

// FP32 LU of the complex64 matrix used as the preconditioner of FP64 outer
// FGMRES (GMRES-based iterative refinement, Carson & Higham 2018): the
// mixed-precision LU refinement role.
struct LuPrecond32 : PrecondFn {
  om_context *ctx;
  long n;
  Work w;
  float2 *A = nullptr, *v32 = nullptr, *y32 = nullptr, *dinv = nullptr;
  int *piv = nullptr, *info = nullptr, *perm = nullptr;
  unsigned *sweep = nullptr;  // flags and epoch of the one-launch triangular sweeps
  int applied = 0;
  // the triangular solves on v32, captured once as a graph and replayed
  cudaGraphExec_t solve_graph = nullptr;
  int solve_launches = 0;
  LuPrecond32(om_context *c, long n_) : ctx(c), n(n_) { w.ctx = c; }
  ~LuPrecond32() {
    if(solve_graph)
      cudaGraphExecDestroy(solve_graph);
  }
  int init(const float2 *S32) {
    size_t bytes = sizeof(float2) * ((size_t)n * n + 3 * n) + sizeof(int) * (2 * n + 2) +
                   sizeof(unsigned) * sweep_ws_words(n) + 2048;
    int rc = alloc_work(ctx, w, bytes);
    if(rc)
      return rc;
    size_t off = 0;
    A = w.take<float2>((size_t)n * n, off);
    v32 = w.take<float2>(n, off);
    y32 = w.take<float2>(n, off);
    piv = w.take<int>(n, off);
    info = w.take<int>(2, off);
    perm = w.take<int>(n, off);
    dinv = w.take<float2>(n, off);
    sweep = w.take<unsigned>(sweep_ws_words(n), off);
    sweep_ws_init(ctx, sweep, n);
    cudaMemcpyAsync(A, S32, sizeof(float2) * (size_t)n * n, cudaMemcpyDeviceToDevice, ctx->stream);
    rc = lu_factor<float2>(ctx, A, n, piv, info);
    if(rc)
      return rc;
    int hinfo[2] = {0, 0};
    cudaMemcpyAsync(hinfo, info, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if(hinfo[1]) {
      ctx->err = "LU kernel wait timed out (tensor-core trailing update or panel barrier)";
      return OM_ERR_CUDA;
    }
    if(hinfo[0]) {
      ctx->err = "singular complex64 matrix: zero pivot at column " + std::to_string(hinfo[0]);
      return OM_ERR_SINGULAR;
    }
    rc = lu_perm(ctx, piv, n, perm);
    if(rc)
      return rc;
    k_lu_diag_inv<float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(A, n, n, dinv);
    ctx->last_launches++;
    // capture the solve sequence (its pointers are fixed); plain launches if
    // capture is refused
    cudaGraph_t g = nullptr;
    if(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
      const int before = ctx->last_launches;
      solve_launches = lu_solve_vec<float2>(ctx, A, n, perm, dinv, v32, y32, sweep, info + 1);
      ctx->last_launches = before;
      if(cudaStreamEndCapture(ctx->stream, &g) != cudaSuccess ||
         cudaGraphInstantiate(&solve_graph, g, 0) != cudaSuccess)
        solve_graph = nullptr;
      if(g)
        cudaGraphDestroy(g);
    }
    cudaGetLastError();
    return OM_OK;
  }
  void apply(const double2 *v, double2 *z) override {
    k_scale_copy<double2, float2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(v, 1.0, v32, n);
    timer_begin(ctx, ctx->ev_lus);
    if(solve_graph) {
      cudaGraphLaunch(solve_graph, ctx->stream);
      ctx->last_launches += solve_launches;
    } else {
      lu_solve_vec<float2>(ctx, A, n, perm, dinv, v32, y32, sweep, info + 1);
    }
    timer_end(ctx, ctx->ev_lus);
    k_scale_copy<float2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(v32, 1.0, z, n);
    ctx->last_launches += 2;
    ++applied;
  }
};

// GMRES-based iterative refinement (Carson & Higham 2018), the
// mixed-precision LU refinement role: FP64 residuals r = b - S x of the
// complex64 system (compensated products), each correction from GMRES on the
// left-preconditioned system M^{-1} S d = M^{-1} r with M the FP32 LU. GMRES
// on M^{-1} S (close to the identity) controls the correction's error, not
// only its residual; right preconditioning with an inexact LU can leave
// solution components along near-null directions of S that a small residual
// does not reveal.
struct LuLeftOp {
  const float2 *S;
  LuPrecond32 *lu;
  double2 *t;  // n scratch
};

__global__ void k_sub_vec(const double2 *b, const double2 *t, double2 *y, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i < n)
    y[i] = make_double2(b[i].x - t[i].x, b[i].y - t[i].y);
}
__global__ void k_add_vec(const double2 *d, double2 *x, long n) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i < n)
    x[i] = make_double2(x[i].x + d[i].x, x[i].y + d[i].y);
}

// y = M^{-1} S x, or y = b - M^{-1} S x when b is given
inline void op_apply(om_context *ctx, const LuLeftOp *op, long n, const double2 *x, double2 *part,
                     double2 *y, const double2 *b) {
  double2 *t = b ? op->t : y;
  matvec<float2, double2>(ctx, op->S, n, x, part, t, nullptr);
  op->lu->apply(t, t);
  if(b) {
    k_sub_vec<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(b, t, y, n);
    ctx->last_launches++;
  }
}

int solve_lu_mixed_rhs(om_problem *pr, int harmonic, const om_solve_options *o, const double2 *b,
                       double2 *x, om_solve_stats *st) {
  om_context *ctx = pr->ctx;
  const long n = pr->n;
  const float2 *S32 = (const float2 *)pr->d_S32[harmonic];
  LuPrecond32 lu(ctx, n);
  int rc = lu.init(S32);
  if(rc)
    return rc;
  Work w;
  w.ctx = ctx;
  const int nsplit = mv_nsplit(ctx, n);
  const int nblk = (int)((n + kDotRows - 1) / kDotRows);
  rc = alloc_work(ctx, w, sizeof(double2) * (4 * (size_t)n + (size_t)std::max<long>((long)nsplit * n, 2L * nblk) + 8) +
                              16 * 256);
  if(rc)
    return rc;
  size_t off = 0;
  double2 *r = w.take<double2>(n, off), *c = w.take<double2>(n, off), *d = w.take<double2>(n, off);
  double2 *t = w.take<double2>(n, off);
  double2 *part = w.take<double2>((size_t)std::max<long>((long)nsplit * n, 2L * nblk), off);
  double2 *hd = w.take<double2>(8, off);
  LuLeftOp op{S32, &lu, t};
  cudaMemsetAsync(x, 0, sizeof(double2) * n, ctx->stream);
  const double bnorm = vec_norm(ctx, b, n, part, hd);
  // at most 8 refinement steps per restart allowed by the options; each
  // correction: GMRES(m) on M^{-1} S to 1e-4, two cycles at most
  const int max_ref = 8 * std::max(1, o->restarts);
  const int m = std::max(1, std::min(o->max_iter, 32));
  int ref = 0, inner = 0;
  double rr = bnorm > 0.0 ? 1.0 : 0.0;
  for(; bnorm > 0.0; ++ref) {
    if(ref == 0)
      cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->stream);
    else
      matvec<float2, double2>(ctx, S32, n, x, part, r, b);
    rr = vec_norm(ctx, r, n, part, hd) / bnorm;
    if(rr <= o->tol || ref == max_ref)
      break;
    lu.apply(r, c);
    int it = 0;
    double irr = 0.0;
    const int e = gmres64<LuLeftOp>(ctx, &op, n, c, d, 1e-4, m, 2, nullptr, &it, &irr);
    if(e && e != OM_ERR_NOT_CONVERGED)
      return e;
    inner += it;
    k_add_vec<<<blocks_for(n, 256), 256, 0, ctx->stream>>>(d, x, n);
    ctx->last_launches++;
  }
  if(st) {
    st->iterations = ref;
    st->inner_iterations = inner;
    st->rel_residual = rr;
  }
  int sweep_err = 0;  // a triangular sweep's wait timed out
  cudaMemcpyAsync(&sweep_err, lu.info + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  cudaStreamSynchronize(ctx->stream);
  if(sweep_err) {
    ctx->err = "LU triangular sweep wait timed out";
    return OM_ERR_CUDA;
  }
  if(rr > o->tol) {
    ctx->err = "LU-preconditioned refinement did not reach the requested tolerance";
    return OM_ERR_NOT_CONVERGED;
  }
  return OM_OK;
}


// ---------------------------------------------------------------------------
// Solve without device allocation.
//
// Some callers cannot allocate device memory while they solve: a serving loop
// that has handed all of HBM to resident matrices and an arena of its own, or
// host code that must not call cudaMalloc/cudaFree because those calls can
// synchronise the whole device in the middle of latency-critical work. For
// them om_solve_rhs_noalloc runs the same restarted GMRES as om_solve_rhs but
// keeps every device buffer it needs (right-hand side, solution, Krylov basis,
// split-K partial sums) in the fixed array below, which every GPU that loads
// this library holds until the process exits.
// ---------------------------------------------------------------------------
constexpr size_t kNoAllocBytes = size_t(64) << 20;  // 64 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

namespace {

// Device address of g_noalloc_scratch, looked up once per device (with that
// device current) on the first no-alloc call made on it.
void *noalloc_scratch(om_context *ctx) {
  static std::mutex mu;
  static void *addr[256] = {};
  std::lock_guard<std::mutex> lock(mu);
  if(ctx->device < 0 || ctx->device >= 256)
    return nullptr;
  if(!addr[ctx->device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if(e != cudaSuccess) {
      ctx->err = std::string("cudaGetSymbolAddress(no-alloc scratch): ") + cudaGetErrorString(e);
      return nullptr;
    }
    addr[ctx->device] = p;
  }
  return addr[ctx->device];
}

// Restarted GMRES (no preconditioner) on a caller-provided workspace: the
// algorithm of gmres64 with its buffers carved from `ws` instead of allocated.
template <typename M>
int gmres_on_workspace(om_context *ctx, const M *S, long n, const double2 *b, double2 *x,
                       double tol, int m, int restarts, char *ws, int *iters, double *relres) {
  const int nsplit = mv_nsplit(ctx, n);
  const int nblk = (int)((n + kDotRows - 1) / kDotRows);
  Work w;  // view only: buf is not owned
  w.ctx = ctx;
  size_t off = 0;
  w.buf = ws;
  double2 *Vb = w.take<double2>((size_t)(m + 1) * n, off);
  double2 *r = w.take<double2>(n, off);
  double2 *part = w.take<double2>((size_t)std::max<long>((long)nsplit * n, (long)nblk * (m + 2)), off);
  double2 *hd = w.take<double2>(2 * (m + 2), off);
  double2 *yd = w.take<double2>(m + 2, off);
  w.buf = nullptr;  // keep ~Work from freeing the static array

  cudaMemsetAsync(x, 0, sizeof(double2) * n, ctx->stream);  // the array keeps old contents
  const double bnorm = vec_norm(ctx, b, n, part, hd);
  *iters = 0;
  if(bnorm == 0.0) {
    *relres = 0.0;
    return OM_OK;
  }
  double err = 1.0;
  int total = 0;
  for(int rest = 0; rest < restarts && err > tol; ++rest) {
    double beta;
    if(rest == 0) {
      cudaMemcpyAsync(r, b, sizeof(double2) * n, cudaMemcpyDeviceToDevice, ctx->stream);
      beta = bnorm;
    } else {
      matvec<M, double2>(ctx, S, n, x, part, r, b);
      beta = vec_norm(ctx, r, n, part, hd);
      err = beta / bnorm;
      if(err <= tol)
        break;
    }
    if(beta == 0.0) {
      err = 0.0;
      break;
    }
    k_scale_copy<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(r, 1.0 / beta, Vb, n);
    ctx->last_launches++;
    std::vector<std::vector<std::complex<double>>> H;
    std::vector<std::complex<double>> cs, sn, g(1, beta);
    int k = 0;
    double cur = beta / bnorm;
    while(k < m && cur > tol) {
      double2 *wv = Vb + (size_t)(k + 1) * n;
      matvec<M, double2>(ctx, S, n, Vb + (size_t)k * n, part, wv, nullptr);
      std::vector<std::complex<double>> h;
      arnoldi_orth<double2>(ctx, Vb, n, k + 1, wv, part, hd, h);
      const double hn = h[k + 1].real();
      if(hn > 0.0) {
        k_scale_copy<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(wv, 1.0 / hn, wv, n);
        ctx->last_launches++;
      }
      for(int i = 0; i < k; ++i) {
        std::complex<double> a = h[i], bb = h[i + 1];
        h[i] = std::conj(cs[i]) * a + std::conj(-sn[i]) * bb;
        h[i + 1] = sn[i] * a + cs[i] * bb;
      }
      std::complex<double> c, s;
      givens(h[k], h[k + 1], c, s);
      cs.push_back(c);
      sn.push_back(s);
      std::complex<double> hk = h[k], hk1 = h[k + 1];
      h[k] = std::conj(c) * hk + std::conj(-s) * hk1;
      h[k + 1] = s * hk + c * hk1;
      g.push_back(0.0);
      std::complex<double> g0 = g[k], g1 = g[k + 1];
      g[k] = std::conj(c) * g0 + std::conj(-s) * g1;
      g[k + 1] = s * g0 + c * g1;
      H.push_back(h);
      cur = std::abs(g[k + 1]) / bnorm;
      ++k;
      ++total;
      if(hn == 0.0)
        break;
    }
    std::vector<std::complex<double>> y(k);
    for(int j = k - 1; j >= 0; --j) {
      std::complex<double> v = g[j];
      for(int q = j + 1; q < k; ++q)
        v -= H[q][j] * y[q];
      y[j] = v / H[j][j];
    }
    std::vector<double2> yh(k);
    for(int j = 0; j < k; ++j)
      yh[j] = make_double2(y[j].real(), y[j].imag());
    cudaMemcpyAsync(yd, yh.data(), sizeof(double2) * k, cudaMemcpyHostToDevice, ctx->stream);
    k_add_combo<double2, double2><<<blocks_for(n, 256), 256, 0, ctx->stream>>>(Vb, n, k, yd, x, n);
    ctx->last_launches++;
    err = cur;  // the estimate, as gmres64
  }
  *iters = total;
  *relres = err;
  return err <= tol ? OM_OK : OM_ERR_NOT_CONVERGED;
}

}  // namespace

}  // namespace om

extern "C" int om_solve_rhs_noalloc(om_problem *pr, int harmonic, const om_solve_options *opts,
                                    const double *b, double *x, om_solve_stats *stats) {
  using namespace om;
  if(!pr || !opts || !b || !x || (harmonic != OM_FF && harmonic != OM_SH))
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  if(opts->method != OM_SOLVE_GMRES) {
    ctx->err = "om_solve_rhs_noalloc supports OM_SOLVE_GMRES only";
    return OM_ERR_INVALID;
  }
  if(pr->S_prec[harmonic] < 0 || pr->S_prec[harmonic] == OM_ACA) {
    ctx->err = pr->S_prec[harmonic] < 0 ? "matrix not assembled"
                                        : "om_solve_rhs_noalloc needs a dense matrix";
    return OM_ERR_STATE;
  }
  const long n = pr->n;
  const int m = opts->max_iter;
  if(m < 1 || opts->restarts < 1) {
    ctx->err = "max_iter and restarts must be positive";
    return OM_ERR_INVALID;
  }
  // bytes the solve needs: b and x, then the workspace of gmres_on_workspace
  auto round = [](size_t v) { return ((v + 255) / 256) * 256; };
  const size_t nsplit = (size_t)mv_nsplit(ctx, n);
  const size_t nblk = (size_t)((n + kDotRows - 1) / kDotRows);
  const size_t z = sizeof(double2);
  const size_t need = 2 * round(z * n) + round(z * (size_t)(m + 1) * n) + round(z * n) +
                      round(z * std::max(nsplit * n, nblk * (size_t)(m + 2))) +
                      round(z * 2 * (size_t)(m + 2)) + round(z * (size_t)(m + 2));
  if(need > kNoAllocBytes) {
    ctx->err = "problem too large for the no-alloc scratch: needs " + std::to_string(need) +
               " bytes, the fixed array holds " + std::to_string(kNoAllocBytes) +
               " (reduce max_iter or use om_solve_rhs)";
    return OM_ERR_INVALID;
  }
  char *ws = static_cast<char *>(noalloc_scratch(ctx));
  if(!ws)
    return OM_ERR_CUDA;
  const auto t0 = std::chrono::steady_clock::now();
  double2 *db = reinterpret_cast<double2 *>(ws);
  double2 *dx = reinterpret_cast<double2 *>(ws + round(z * n));
  char *rest = ws + 2 * round(z * n);
  cudaMemcpyAsync(db, b, z * n, cudaMemcpyHostToDevice, ctx->stream);
  int it = 0;
  double rr = 0;
  int rc;
  if(pr->S_prec[harmonic] == OM_C128)
    rc = gmres_on_workspace<double2>(ctx, (const double2 *)pr->d_S[harmonic], n, db, dx, opts->tol,
                                     m, opts->restarts, rest, &it, &rr);
  else
    rc = gmres_on_workspace<float2>(ctx, (const float2 *)pr->d_S32[harmonic], n, db, dx, opts->tol,
                                    m, opts->restarts, rest, &it, &rr);
  cudaMemcpyAsync(x, dx, z * n, cudaMemcpyDeviceToHost, ctx->stream);
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e == cudaSuccess)
    e = cudaGetLastError();  // launch-configuration errors, which the synchronisation does not return
  if(e != cudaSuccess) {
    ctx->err = std::string("om_solve_rhs_noalloc: ") + cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  if(stats) {
    stats->iterations = it;
    stats->inner_iterations = 0;
    stats->rel_residual = rr;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  if(rc == OM_ERR_NOT_CONVERGED)
    ctx->err = "GMRES did not reach the requested tolerance";
  return rc;
}

namespace om {
}  // namespace om
