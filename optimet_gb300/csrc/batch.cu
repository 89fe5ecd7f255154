// Batched wavelength solves: the batching form (om_batch_solve).
//
// Many requests (clusters and wavelengths of uneven N and nMax, fundamental
// with optional second harmonic) are grouped into size classes: the same
// precision form, nMax and solve options, and N padded up to a class size
// (1, 2, 3, 4, 6, 8, 12, ... : steps of at most 1.5x). A class runs its
// requests in batches of up to B slots, where B follows from the device memory
// a slot needs. Per batch:
//
//  * the per-sphere state of every request (T-matrix factors, incident
//    coefficients, source vector) is set up with the kernels of the
//    single-request path;
//  * ONE launch of the translation/assembly kernel builds the FF and the SH
//    matrices of all requests of the batch (one CTA per sphere pair per
//    matrix, `k_assemble` in batch mode);
//  * the FF systems, then the SH systems, are solved together by restarted
//    GMRES in lockstep: every slot runs the same Arnoldi step at the same
//    time, a slot that has converged is masked (its kernels return at once),
//    one matvec launch serves all slots (split-K tiles of every slot's
//    matrix taken from one counter), and the Hessenberg/Givens updates run on
//    the device, so that the whole iteration reads its step index and its
//    flags from device memory;
//  * those iterations are captured once per size class as three CUDA graphs
//    (start of a cycle: residual, its norm, convergence test; a segment of
//    kSegSteps Arnoldi steps; end of a cycle: back substitution and update)
//    and replayed; the host reads two counters after each segment.
//
// Forms: the plain form (OM_C128 with OM_SOLVE_GMRES) is restarted GMRES on
// the complex128 matrices; the precision form (OM_C64 with
// OM_SOLVE_FGMRES_MIXED) is GMRES-based iterative refinement (Carson & Higham
// 2018): each cycle takes the residual of the complex64 system in FP64-accurate
// arithmetic (compensated products), runs FP32 Arnoldi on the complex64 matrix
// until the residual estimate falls by inner_tol, and adds the FP64 correction.
//
// A slot's arithmetic does not depend on the other slots, on its position or
// on the class it runs in (fixed split-K chunks and dot-product blocks, fixed
// reduction orders), so a request's results are bitwise the same alone and in
// any batch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "om_internal.h"
#include "om_krylov.cuh"

namespace om {

namespace {

constexpr int kBT = 256;         // threads of the vector kernels; rows per matvec tile
constexpr int kBCols = 1024;     // columns per split-K chunk
constexpr int kBDotRows = 2048;  // rows per block of the residual norm
constexpr int kFRows = 512;      // rows per block of the Arnoldi vector kernels
constexpr int kSegSteps = 8;     // Arnoldi steps per captured segment
constexpr int kMaxSlots = 256;   // slots per batch (one thread per slot in the control kernels)

// Per-slot solver state (device).
struct Slot {
  long n;          // unknowns; 0 = empty slot
  const void *S;   // matrix, column-major, ld = n
  const F16c *H;   // precision form: the Arnoldi products' fp16 copy (ld = n), or null
  const float *D;  // its scales: D[b n + j] for rows [256 b, 256 b + 256) of column j
  double bnorm;    // ||b||; negative until the first cycle
  double rho;      // ||b - S x|| at the start of the latest cycle
  double thr;      // this cycle's stop threshold on |g_{j+1}|
  int outer;       // still needs cycles
  int inner;       // Arnoldi of this cycle running
  int k;           // Arnoldi steps of this cycle
  int xzero;       // x = 0 (the residual is b)
  int steps;       // Arnoldi steps, all cycles
  int cycles;      // cycles run
  int status;      // OM_OK or OM_ERR_NOT_CONVERGED once outer = 0
  int pad;
};

// Batch control (device).
struct Ctl {
  int j;        // Arnoldi step of the slots (the new basis vector is column j + 1)
  int n_inner;  // slots whose Arnoldi runs
  int n_outer;  // slots that still need cycles
  int ntiles;   // matvec tiles of the current system
};

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 cconj(double2 a) { return make_double2(a.x, -a.y); }
__device__ __forceinline__ double2 cneg(double2 a) { return make_double2(-a.x, -a.y); }
__device__ __forceinline__ double2 cdiv(double2 a, double2 b) {
  // Smith's algorithm
  if(fabs(b.x) >= fabs(b.y)) {
    const double r = b.y / b.x, d = b.x + b.y * r;
    return make_double2((a.x + a.y * r) / d, (a.y - a.x * r) / d);
  }
  const double r = b.x / b.y, d = b.x * r + b.y;
  return make_double2((a.x * r + a.y) / d, (a.y * r - a.x) / d);
}
__device__ __forceinline__ double cabs2(double2 a) { return hypot(a.x, a.y); }

// Givens rotation of det_approx (PreconditionedMatrix.cpp:1102-1118), as the
// host solver uses it
__device__ void givens_dev(double2 h1, double2 h2, double2 &c, double2 &s) {
  const double a1 = cabs2(h1), a2 = cabs2(h2);
  if(a1 == 0.0 && a2 == 0.0) {
    c = make_double2(1.0, 0.0);
    s = make_double2(0.0, 0.0);
    return;
  }
  if(a2 > a1) {
    const double2 t = cdiv(h1, h2);
    const double at = cabs2(t);
    s = make_double2(1.0 / sqrt(1.0 + at * at), 0.0);
    c = cneg(cmul(t, s));
  } else {
    const double2 t = cdiv(h2, h1);
    const double at = cabs2(t);
    c = make_double2(1.0 / sqrt(1.0 + at * at), 0.0);
    s = cneg(cmul(t, c));
  }
}

template <typename V> __device__ __forceinline__ double2 to_d2(V v) { return make_double2(v.x, v.y); }

// ---------------------------------------------------------------------------
// Matrix-vector products over all slots. A tile is (slot, 256 rows, 1024
// columns); the capped grid takes tiles from a counter (zeroed before the
// launch). part[(s nsm + chunk) np + i] holds a chunk's partial sum.
// ---------------------------------------------------------------------------

// Arnoldi product: S_s times basis column j of slot s (slots with inner set).
// R rows per tile (one thread each): the row sums do not depend on R.
template <typename M, typename V, int R>
__global__ void __launch_bounds__(R) k_b_mv(const Slot *st, const int4 *tiles, const Ctl *ctl,
                                           const V *Vb, long vslot, long np, int nsm, V *part,
                                           unsigned long long *next) {
  __shared__ V xs[kBCols];
  __shared__ int tile;
  const int ntiles = ctl->ntiles;
  const int jcol = ctl->j;
  for(;;) {
    __syncthreads();
    if(threadIdx.x == 0)
      tile = (int)atomicAdd(next, 1ull);
    __syncthreads();
    const int t = tile;
    if(t >= ntiles)
      break;
    const int4 d = tiles[t];
    if(!st[d.x].inner)
      continue;
    const long n = st[d.x].n;
    const M *S = (const M *)(std::is_same<M, F16c>::value ? (const void *)st[d.x].H : st[d.x].S);
    const V *x = Vb + d.x * vslot + (long)jcol * np;
    const long i = (long)d.y * R + threadIdx.x;
    const long j0 = (long)d.z * kBCols, j1 = min(n, j0 + kBCols);
    if constexpr(std::is_same<M, F16c>::value) {
      // x times the scales of the tile's 256-row block
      const float *Dc = st[d.x].D + ((long)d.y * R / 256) * n;
      for(long j = j0 + threadIdx.x; j < j1; j += R) {
        V v = x[j];
        const float f = Dc[j];
        v.x = v.x * f;
        v.y = v.y * f;
        xs[j - j0] = v;
      }
    } else {
      for(long j = j0 + threadIdx.x; j < j1; j += R)
        xs[j - j0] = x[j];
    }
    __syncthreads();
    if(i < n)
      part[((long)d.x * nsm + d.z) * np + i] = mv_row<M, V>(S + j0 * n + i, n, xs, 0L, j1 - j0);
  }
}

// Residual product: S_s x_s with x in FP64 (slots with outer set and x != 0);
// a complex64 matrix takes the compensated FP64-accurate sums
template <typename M, int R>
__global__ void __launch_bounds__(R) k_b_resid(const Slot *st, const int4 *tiles, const Ctl *ctl,
                                              const double2 *x, long np, int nsm, double2 *part,
                                              unsigned long long *next) {
  constexpr bool kDF = std::is_same<M, float2>::value;
  typedef typename std::conditional<kDF, DFX, double2>::type XS;
  __shared__ XS xs[kBCols];
  __shared__ int tile;
  const int ntiles = ctl->ntiles;
  for(;;) {
    __syncthreads();
    if(threadIdx.x == 0)
      tile = (int)atomicAdd(next, 1ull);
    __syncthreads();
    const int t = tile;
    if(t >= ntiles)
      break;
    const int4 d = tiles[t];
    if(!st[d.x].outer || st[d.x].xzero)
      continue;
    const long n = st[d.x].n;
    const M *S = (const M *)st[d.x].S;
    const double2 *xv = x + d.x * np;
    const long i = (long)d.y * R + threadIdx.x;
    const long j0 = (long)d.z * kBCols, j1 = min(n, j0 + kBCols);
    for(long j = j0 + threadIdx.x; j < j1; j += R) {
      if constexpr(kDF)
        xs[j - j0] = df_split(xv[j]);
      else
        xs[j - j0] = xv[j];
    }
    __syncthreads();
    if(i >= n)
      continue;
    double2 v;
    if constexpr(kDF)
      v = mv_row_df(S + j0 * n + i, n, xs, 0L, j1 - j0);
    else
      v = mv_row<double2, double2>(S + j0 * n + i, n, xs, 0L, j1 - j0);
    part[((long)d.x * nsm + d.z) * np + i] = v;
  }
}

// r = b - S x (r = b while x = 0)
__global__ void k_b_reduce_r(const Slot *st, const double2 *part, long np, int nsm, const double2 *b,
                             double2 *r) {
  const int s = blockIdx.y;
  if(!st[s].outer)
    return;
  const long n = st[s].n, i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  const double2 bv = b[s * np + i];
  if(st[s].xzero) {
    r[s * np + i] = bv;
    return;
  }
  const int ns = (int)((n + kBCols - 1) / kBCols);
  const double2 *p = part + (long)s * nsm * np + i;
  double2 acc = p[0];
  for(int c = 1; c < ns; ++c) {
    const double2 v = p[(long)c * np];
    acc.x += v.x;
    acc.y += v.y;
  }
  r[s * np + i] = make_double2(bv.x - acc.x, bv.y - acc.y);
}

// ||r||^2 block partials of the residual: rows [blockIdx.x kBDotRows, ...)
// of slot blockIdx.y (slots with outer set), into dpart[(s nblk + block) m2]
__global__ void __launch_bounds__(kBT) k_b_rnorm(const Slot *st, const double2 *r, long np, int nblk,
                                                int m2, double2 *dpart) {
  __shared__ double red[kBT];
  const int s = blockIdx.y;
  if(!st[s].outer)
    return;
  const long n = st[s].n;
  const long r0 = (long)blockIdx.x * kBDotRows;
  if(r0 >= n)
    return;
  const long r1 = min(n, r0 + kBDotRows);
  double acc = 0.0;
  for(long i = r0 + threadIdx.x; i < r1; i += kBT) {
    const double2 a = r[s * np + i];
    acc = fma(a.x, a.x, acc);
    acc = fma(a.y, a.y, acc);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for(int h = kBT / 2; h > 0; h >>= 1) {
    if(threadIdx.x < h)
      red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if(threadIdx.x == 0)
    dpart[((long)s * nblk + blockIdx.x) * m2] = make_double2(red[0], 0.0);
}

// The Arnoldi vector kernels work on row blocks of kFRows rows of one slot
// (grid: row blocks x slots); a block's partial sums go to
// dp[(s nbf + block) m2 + t] and the next kernel adds them in block order.
template <typename V> __device__ __forceinline__ V warp_sum(V a) {
  for(int o = 16; o > 0; o >>= 1) {
    a.x += __shfl_xor_sync(0xffffffffu, a.x, o);
    a.y += __shfl_xor_sync(0xffffffffu, a.y, o);
  }
  return a;
}

// out[t] = sum over rows [r0, r1) of conj(v_t) w, t < k: one warp per t
template <typename V>
__device__ __forceinline__ void block_proj(const V *vs, const V *w, long np, long r0, long r1, int k,
                                           V *out) {
  const int lane = threadIdx.x & 31;
  for(int t = threadIdx.x >> 5; t < k; t += kBT / 32) {
    const V *v = vs + (long)t * np;
    V acc;
    acc.x = acc.y = 0;
    for(long i = r0 + lane; i < r1; i += 32)
      acc = cfma_conj(v[i], w[i], acc);
    acc = warp_sum(acc);
    if(lane == 0)
      out[t] = acc;
  }
}

// h[t] = sum over the slot's nb blocks of dp (block order), t < k, in shared memory
template <typename V>
__device__ __forceinline__ void gather_h(const V *dp, int nb, int m2, int k, V *h) {
  for(int t = threadIdx.x; t < k; t += kBT) {
    V acc = dp[t];
    for(int b = 1; b < nb; ++b) {
      acc.x += dp[(long)b * m2 + t].x;
      acc.y += dp[(long)b * m2 + t].y;
    }
    h[t] = acc;
  }
  __syncthreads();
}

// w (basis column j + 1) = the split-K partials summed in chunk order; then
// the first projection pass V[:, 0..j]^H w
template <typename V>
__global__ void __launch_bounds__(kBT) k_b_red_proj(const Slot *st, const Ctl *ctl, const V *part, long np,
                                                   int nsm, V *Vb, long vslot, int nbf, int m2, V *dpA) {
  const int s = blockIdx.y;
  if(!st[s].inner)
    return;
  const long n = st[s].n, r0 = (long)blockIdx.x * kFRows;
  if(r0 >= n)
    return;
  const long r1 = min(n, r0 + kFRows);
  const int k = ctl->j + 1;
  V *vs = Vb + s * vslot, *w = vs + (long)k * np;
  const int ns = (int)((n + kBCols - 1) / kBCols);
  for(long i = r0 + threadIdx.x; i < r1; i += kBT) {
    const V *p = part + (long)s * nsm * np + i;
    V acc = p[0];
    for(int c = 1; c < ns; ++c) {
      const V v = p[(long)c * np];
      acc.x += v.x;
      acc.y += v.y;
    }
    w[i] = acc;
  }
  __syncthreads();
  block_proj(vs, w, np, r0, r1, k, dpA + ((long)s * nbf + blockIdx.x) * m2);
}

// w -= V h with h the previous pass's projections (hacc = h on pass 0, += h
// on pass 1, written by block 0); then the second projection pass (pass 0)
// or |w|^2 into entry m2 - 1 of the block's partials (pass 1)
template <typename V>
__global__ void __launch_bounds__(kBT) k_b_sub_proj(const Slot *st, const Ctl *ctl, V *Vb, long vslot,
                                                   long np, int nbf, int m2, const V *dp_in, V *dp_out,
                                                   double2 *hacc, int pass) {
  extern __shared__ unsigned char h_raw[];
  V *h = reinterpret_cast<V *>(h_raw);
  __shared__ double red[kBT / 32];
  const int s = blockIdx.y;
  if(!st[s].inner)
    return;
  const long n = st[s].n, r0 = (long)blockIdx.x * kFRows;
  if(r0 >= n)
    return;
  const long r1 = min(n, r0 + kFRows);
  const int k = ctl->j + 1;
  const int nb = (int)((n + kFRows - 1) / kFRows);
  gather_h(dp_in + (long)s * nbf * m2, nb, m2, k, h);
  if(blockIdx.x == 0)
    for(int t = threadIdx.x; t < k; t += kBT)
      hacc[s * m2 + t] = pass ? cadd(hacc[s * m2 + t], to_d2(h[t])) : to_d2(h[t]);
  V *vs = Vb + s * vslot, *w = vs + (long)k * np;
  double nrm = 0.0;
  for(long i = r0 + threadIdx.x; i < r1; i += kBT) {
    V acc = w[i];
    for(int t = 0; t < k; ++t) {
      V c = h[t];
      c.x = -c.x;
      c.y = -c.y;
      acc = cfma(vs[(long)t * np + i], c, acc);
    }
    w[i] = acc;
    nrm = fma((double)acc.x, (double)acc.x, nrm);
    nrm = fma((double)acc.y, (double)acc.y, nrm);
  }
  V *out = dp_out + ((long)s * nbf + blockIdx.x) * m2;
  if(!pass) {
    __syncthreads();
    block_proj(vs, w, np, r0, r1, k, out);
    return;
  }
  for(int o = 16; o > 0; o >>= 1)
    nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
  if((threadIdx.x & 31) == 0)
    red[threadIdx.x >> 5] = nrm;
  __syncthreads();
  if(threadIdx.x == 0) {
    double a = 0.0;
    for(int q = 0; q < kBT / 32; ++q)
      a += red[q];
    out[m2 - 1].x = a;
    out[m2 - 1].y = 0;
  }
}

// Hessenberg column j of every Arnoldi slot: previous rotations, the new
// rotation, the residual estimate |g_{j+1}| and the stop test; one thread
// per slot. Then the step index advances (if any slot ran).
template <typename V>
__global__ void k_b_givens(Slot *st, Ctl *ctl, const V *dp, int nbf, int m2, const double2 *hacc,
                           double2 *Hm, double2 *cs, double2 *sn, double2 *g, double *inv, int m,
                           int B) {
  const int s = threadIdx.x;
  const int j = ctl->j;
  const int act = s < B ? st[s].inner : 0;
  const int any = __syncthreads_count(act);
  int still = 0;
  if(act) {
    Slot &sl = st[s];
    const int nb = (int)((sl.n + kFRows - 1) / kFRows);
    const V *p = dp + (long)s * nbf * m2 + (m2 - 1);
    double acc = p[0].x;
    for(int b = 1; b < nb; ++b)
      acc += p[(long)b * m2].x;
    const double hn = sqrt(acc);
    double2 *col = Hm + ((long)s * m + j) * (m + 1);
    for(int t = 0; t <= j; ++t)
      col[t] = hacc[s * m2 + t];
    double2 *c_s = cs + (long)s * m, *s_s = sn + (long)s * m;
    for(int i = 0; i < j; ++i) {
      const double2 a = col[i], bb = col[i + 1];
      col[i] = cadd(cmul(cconj(c_s[i]), a), cmul(cconj(cneg(s_s[i])), bb));
      col[i + 1] = cadd(cmul(s_s[i], a), cmul(c_s[i], bb));
    }
    double2 c, sr;
    const double2 hk1 = make_double2(hn, 0.0);
    givens_dev(col[j], hk1, c, sr);
    c_s[j] = c;
    s_s[j] = sr;
    const double2 hk = col[j];
    col[j] = cadd(cmul(cconj(c), hk), cmul(cconj(cneg(sr)), hk1));
    double2 *gs = g + (long)s * (m + 1);
    const double2 g0 = gs[j];
    gs[j] = cmul(cconj(c), g0);
    gs[j + 1] = cmul(sr, g0);
    inv[s] = hn > 0.0 ? 1.0 / hn : 0.0;
    sl.k = j + 1;
    sl.steps++;
    still = !(cabs2(gs[j + 1]) <= sl.thr || hn == 0.0 || j + 1 >= m);
    sl.inner = still;
  }
  const int n_in = __syncthreads_count(still);
  if(threadIdx.x == 0 && any) {
    ctl->j = j + 1;
    ctl->n_inner = n_in;
  }
}

// v_{j+1} = w / h_{j+1,j} (the step index has advanced: w = column j)
template <typename V>
__global__ void k_b_scale(const Slot *st, const Ctl *ctl, const double *inv, V *Vb, long vslot, long np) {
  const int s = blockIdx.y;
  if(!st[s].inner)
    return;
  const long n = st[s].n, i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  V *w = Vb + s * vslot + (long)ctl->j * np;
  const double f = inv[s];
  w[i].x = w[i].x * f;
  w[i].y = w[i].y * f;
}

// Start of a cycle: rho = ||r||, the convergence test, g_0 = rho.
__global__ void k_b_start(Slot *st, Ctl *ctl, const double2 *dpart, int nblk, int m2, double2 *g,
                          int m, int B, double tol, double inner_rel, int max_cycles) {
  const int s = threadIdx.x;
  int out = 0, in = 0;
  if(s < B) {
    Slot &sl = st[s];
    sl.k = 0;
    sl.inner = 0;
    if(sl.outer) {
      const int nb = (int)((sl.n + kBDotRows - 1) / kBDotRows);
      const double2 *p = dpart + (long)s * nblk * m2;
      double acc = p[0].x;
      for(int b = 1; b < nb; ++b)
        acc += p[(long)b * m2].x;
      const double rho = sqrt(acc);
      if(sl.bnorm < 0.0)
        sl.bnorm = rho;
      sl.rho = rho;
      if(sl.bnorm == 0.0 || rho <= tol * sl.bnorm) {
        sl.outer = 0;
        sl.status = OM_OK;
      } else if(sl.cycles >= max_cycles) {
        sl.outer = 0;
        sl.status = OM_ERR_NOT_CONVERGED;
      } else {
        sl.inner = 1;
        sl.thr = fmax(inner_rel * rho, tol * sl.bnorm);
        g[(long)s * (m + 1)] = make_double2(rho, 0.0);
      }
      out = sl.outer;
      in = sl.inner;
    }
  }
  const int n_out = __syncthreads_count(out);
  const int n_in = __syncthreads_count(in);
  if(threadIdx.x == 0) {
    ctl->j = 0;
    ctl->n_outer = n_out;
    ctl->n_inner = n_in;
  }
}

// v_0 = r / rho
template <typename V>
__global__ void k_b_v0(const Slot *st, const double2 *r, long np, V *Vb, long vslot) {
  const int s = blockIdx.y;
  if(!st[s].inner)
    return;
  const long n = st[s].n, i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  const double f = 1.0 / st[s].rho;
  const double2 v = r[s * np + i];
  V o;
  o.x = v.x * f;
  o.y = v.y * f;
  Vb[s * vslot + i] = o;
}

// End of a cycle: y = R^{-1} g over the slot's k steps (one thread per slot).
__global__ void k_b_end(Slot *st, const double2 *Hm, const double2 *g, double2 *y, int m, int B) {
  const int s = threadIdx.x;
  if(s >= B)
    return;
  Slot &sl = st[s];
  const int k = sl.k;
  if(k == 0)
    return;
  const double2 *H = Hm + (long)s * m * (m + 1);
  const double2 *gs = g + (long)s * (m + 1);
  double2 *ys = y + (long)s * m;
  for(int j = k - 1; j >= 0; --j) {
    double2 v = gs[j];
    for(int q = j + 1; q < k; ++q)
      v = cadd(v, cneg(cmul(H[(long)q * (m + 1) + j], ys[q])));
    ys[j] = cdiv(v, H[(long)j * (m + 1) + j]);
  }
  sl.cycles++;
  sl.xzero = 0;
}

// x += sum_t y_t v_t (FP64)
template <typename V>
__global__ void k_b_update(const Slot *st, const V *Vb, long vslot, long np, const double2 *y, int m,
                           double2 *x) {
  const int s = blockIdx.y;
  const int k = st[s].k;
  if(k == 0)
    return;
  const long n = st[s].n, i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= n)
    return;
  const V *vs = Vb + s * vslot;
  double2 acc = x[s * np + i];
  for(int t = 0; t < k; ++t)
    acc = cfma(to_d2(vs[(long)t * np + i]), y[(long)s * m + t], acc);
  x[s * np + i] = acc;
}

// The fp16 copies of a batch's complex64 matrices (precision form): per
// matrix, column j and 256-row block b, the scale d = 2^(e - 15) with e the
// exponent of the block column's largest part (frexp, at least -100), D[b n + j] = d and
// H = fp16(S / d), round to nearest even. One warp per (matrix, column,
// block) item; items numbered matrix by matrix (first[m] = the matrix's
// first item).
struct CvMat {
  const float2 *S;
  F16c *H;
  float *D;
  long n, first;
};
__global__ void __launch_bounds__(256) k_b_tof16(const CvMat *mats, int nmats, long items) {
  const int lane = threadIdx.x & 31;
  const long warps = (long)gridDim.x * (blockDim.x / 32);
  for(long q = (long)blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); q < items; q += warps) {
    int lo = 0, hi = nmats - 1;  // the matrix whose items hold q
    while(lo < hi) {
      const int mid = (lo + hi + 1) / 2;
      if(mats[mid].first <= q)
        lo = mid;
      else
        hi = mid - 1;
    }
    const CvMat mt = mats[lo];
    const long nb = (mt.n + 255) / 256, r = q - mt.first, j = r / nb, b = r - j * nb;
    float2 v[8];
    float mx = 0.f;
#pragma unroll
    for(int u = 0; u < 8; ++u) {
      const long i = b * 256 + lane + 32 * u;
      v[u] = i < mt.n ? mt.S[j * mt.n + i] : make_float2(0.f, 0.f);
      mx = fmaxf(mx, fmaxf(fabsf(v[u].x), fabsf(v[u].y)));
    }
    for(int o = 16; o > 0; o >>= 1)
      mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    int e = 0;
    if(mx > 0.f)
      frexpf(mx, &e);
    // block columns of tiny entries (high orders of small spheres reach 1e-35
    // and below) keep finite, normal scales: e >= -100 bounds 2^(15 - e) by
    // 2^115 and d by 2^-115 (their entries then stay below 2^15 as well)
    e = max(e, -100);
    const float up = ldexpf(1.f, 15 - e);
#pragma unroll
    for(int u = 0; u < 8; ++u) {
      const long i = b * 256 + lane + 32 * u;
      if(i < mt.n)
        mt.H[j * mt.n + i] = F16c{__floats2half2_rn(v[u].x * up, v[u].y * up)};
    }
    if(lane == 0)
      mt.D[b * mt.n + j] = ldexpf(1.f, e - 15);
  }
}

// ---------------------------------------------------------------------------
// Fused solves of the small size classes (at most kFusedRows padded
// unknowns): one cooperative launch runs every slot's restarted GMRES /
// GMRES-IR to the end. A group of C = ceil(np / kFRows) CTAs serves one slot
// at a time (group g of G takes slots g, g + G, ...); CTA c of the group owns
// rows [c kFRows, (c + 1) kFRows) of the slot's vectors, so its matvec rows,
// its Arnoldi vector work and its block partial sums are the row block the
// lockstep kernels give CTA c. The CTAs of a group meet at a bounded barrier
// in global memory three times per Arnoldi step (after the first
// projections, after the second, after |w|^2) and twice per cycle. Every CTA
// forms the residual norm, the projections, the Hessenberg column, the
// rotation and the stop test itself from the same partial sums, so the CTAs
// take the same branches without further exchange; CTA 0 keeps the
// Hessenberg columns for the back substitution. Each value is formed by the
// same inline functions, over the same rows and in the same order as in the
// lockstep kernels above, so a slot's bits do not depend on the form that
// solved it.
// ---------------------------------------------------------------------------
constexpr int kFusedBlocks = 8;                    // CTAs per slot at most
constexpr int kFusedRows = kFusedBlocks * kFRows;  // 4,096 padded unknowns
// By default the fused form takes the classes of at most kFusedAuto padded
// unknowns (groups of one or two CTAs, one column chunk). Per size class of
// the c3 sweep it measured 8-20 % faster there than the lockstep graphs, and
// up to two times slower from about 1,300 unknowns on: the CTAs of a group then
// run matvec rows of several chunks each one after the other, where the
// lockstep matvec spreads a slot's tiles over the whole GPU.
constexpr int kFusedAuto = 2 * kFRows;
constexpr long kFusedSpin = 1L << 24;              // polls before a group barrier gives up
constexpr int kFusedSmemMax = 200 * 1024;          // dynamic shared memory of k_b_fused at most
static_assert(kFRows == 2 * kBT, "a fused CTA's thread takes two rows of its block");

template <typename V> struct FusedArgs {
  Slot *st;
  int B;
  const double2 *b;
  double2 *x, *r;
  V *Vb;
  long vslot, np;
  V *wbuf;        // 2 np per slot: w after its second pass, read by the next step's product
  V *dpA, *dpB;   // [slot][nbf][m2] block partials (entry m2 - 1 of dpA: the block's |w|^2)
  double2 *Hm;    // [slot][m][m + 1] (CTA 0 of the group)
  int m, m2, nbf, C;
  double tol, inner_rel;
  int max_cycles;
  unsigned *bar;  // one arrival counter per group, 32 words apart
  int *err;       // set when a barrier gave up
};

// Dynamic shared memory of k_b_fused: the staged column chunk (the residual's
// split x or the basis column), the CTA's w rows, the projections and the
// Hessenberg / rotation state.
template <typename V> struct FusedSmem {
  int m2, m;
  size_t xs, w, h, hacc, col, cs, sn, g, y, bytes;
  __host__ __device__ FusedSmem(int m_, int m2_) : m2(m2_), m(m_) {
    auto up = [](size_t v) { return (v + 15) / 16 * 16; };
    size_t o = 0;
    xs = o;
    o += up(kBCols * (sizeof(DFX) > sizeof(double2) ? sizeof(DFX) : sizeof(double2)));
    w = o;
    o += up(kFRows * sizeof(V));
    h = o;
    o += up(m2 * sizeof(V));
    hacc = o;
    o += up(m2 * sizeof(double2));
    col = o;
    o += up((m + 1) * sizeof(double2));
    cs = o;
    o += up(m * sizeof(double2));
    sn = o;
    o += up(m * sizeof(double2));
    g = o;
    o += up((m + 1) * sizeof(double2));
    y = o;
    o += up(m * sizeof(double2));
    bytes = o;
  }
};

// The group's barrier: every CTA adds one arrival with release semantics
// (its threads' writes, ordered before thread 0 by the CTA barrier, become
// visible with it) and waits, with acquire loads and a bounded number of
// polls, until the counter reaches `target`.
__device__ __forceinline__ bool group_barrier(unsigned *ctr, unsigned target, int C, int *err) {
  __shared__ int ok_s;
  __syncthreads();
  if(C == 1)
    return true;
  if(threadIdx.x == 0) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(ctr), "r"(1u) : "memory");
    int ok = 0;
    for(long it = 0; it < kFusedSpin; ++it) {
      unsigned v;
      asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ctr) : "memory");
      if((int)(v - target) >= 0) {
        ok = 1;
        break;
      }
      if((it & 63) == 63 && *(volatile int *)err)
        break;  // another group's CTA gave up
      __nanosleep(32);
    }
    if(!ok)
      atomicExch(err, 1);
    ok_s = ok;
  }
  __syncthreads();
  return ok_s != 0;
}

// block_proj with the block's w rows in shared memory (ws[i - r0])
template <typename V>
__device__ __forceinline__ void block_proj_sm(const V *vs, const V *ws, long np, long r0, long r1, int k,
                                              V *out) {
  const int lane = threadIdx.x & 31;
  for(int t = threadIdx.x >> 5; t < k; t += kBT / 32) {
    const V *v = vs + (long)t * np;
    V acc;
    acc.x = acc.y = 0;
    for(long i = r0 + lane; i < r1; i += 32)
      acc = cfma_conj(v[i], ws[i - r0], acc);
    acc = warp_sum(acc);
    if(lane == 0)
      out[t] = acc;
  }
}

template <typename M, typename V>
__global__ void __launch_bounds__(kBT) k_b_fused(FusedArgs<V> a) {
  constexpr bool kDF = std::is_same<M, float2>::value;
  typedef typename std::conditional<kDF, DFX, double2>::type XS;
  extern __shared__ __align__(16) unsigned char fsm[];
  const FusedSmem<V> L(a.m, a.m2);
  XS *xr = reinterpret_cast<XS *>(fsm + L.xs);
  V *xs = reinterpret_cast<V *>(fsm + L.xs);
  V *w = reinterpret_cast<V *>(fsm + L.w);
  V *h = reinterpret_cast<V *>(fsm + L.h);
  double2 *hacc = reinterpret_cast<double2 *>(fsm + L.hacc);
  double2 *col = reinterpret_cast<double2 *>(fsm + L.col);
  double2 *c_s = reinterpret_cast<double2 *>(fsm + L.cs);
  double2 *s_s = reinterpret_cast<double2 *>(fsm + L.sn);
  double2 *gs = reinterpret_cast<double2 *>(fsm + L.g);
  double2 *ys = reinterpret_cast<double2 *>(fsm + L.y);
  __shared__ Slot sl;
  __shared__ double red[kBT];
  __shared__ double inv_s;
  const int tid = threadIdx.x;
  const int C = a.C, c = blockIdx.x % C, grp = blockIdx.x / C, G = gridDim.x / C;
  const int m = a.m, m2 = a.m2;
  const long np = a.np;
  unsigned *ctr = a.bar + 32 * grp;
  unsigned target = 0;
  for(int s = grp; s < a.B; s += G) {
    __syncthreads();
    if(tid == 0)
      sl = a.st[s];
    __syncthreads();
    if(sl.n == 0 || !sl.outer)
      continue;
    const long n = sl.n;
    const M *S = (const M *)sl.S;
    const F16c *Hf = sl.H;  // precision form: the Arnoldi products read the fp16 copy when set
    const long r0 = (long)c * kFRows, r1 = min(n, r0 + kFRows);  // r1 <= r0: no rows of this slot
    const int nb = (int)((n + kFRows - 1) / kFRows);
    const int ns = (int)((n + kBCols - 1) / kBCols);
    V *vs = a.Vb + s * a.vslot;
    const double2 *bs = a.b + s * np;
    double2 *xv = a.x + s * np, *rv = a.r + s * np;
    V *dA = a.dpA + (long)s * a.nbf * m2, *dB = a.dpB + (long)s * a.nbf * m2;
    V *wb = a.wbuf + (long)s * 2 * np;
    double2 *H = a.Hm + (long)s * m * (m + 1);
    for(;;) {
      // r = b - S x over the CTA's rows (k_b_resid, k_b_reduce_r)
      if(sl.xzero) {
        for(long i = r0 + tid; i < r1; i += kBT)
          rv[i] = bs[i];
      } else {
        double2 acc[2];
        for(int cc = 0; cc < ns; ++cc) {
          const long j0 = (long)cc * kBCols, j1 = min(n, j0 + kBCols);
          __syncthreads();
          for(long j = j0 + tid; j < j1; j += kBT) {
            if constexpr(kDF)
              xr[j - j0] = df_split(xv[j]);
            else
              xr[j - j0] = xv[j];
          }
          __syncthreads();
#pragma unroll
          for(int q = 0; q < 2; ++q) {
            const long i = r0 + q * kBT + tid;
            if(i >= r1)
              continue;
            double2 v;
            if constexpr(kDF)
              v = mv_row_df(S + j0 * n + i, n, xr, 0L, j1 - j0);
            else
              v = mv_row<double2, double2>(S + j0 * n + i, n, xr, 0L, j1 - j0);
            if(cc == 0) {
              acc[q] = v;
            } else {
              acc[q].x += v.x;
              acc[q].y += v.y;
            }
          }
        }
#pragma unroll
        for(int q = 0; q < 2; ++q) {
          const long i = r0 + q * kBT + tid;
          if(i < r1)
            rv[i] = make_double2(bs[i].x - acc[q].x, bs[i].y - acc[q].y);
        }
      }
      if(!group_barrier(ctr, target += C, C, a.err))
        return;
      // ||r|| over kBDotRows-row blocks in block order (k_b_rnorm, k_b_start)
      double tot = 0.0;
      for(long q0 = 0; q0 < n; q0 += kBDotRows) {
        const long q1 = min(n, q0 + kBDotRows);
        double acc = 0.0;
        for(long i = q0 + tid; i < q1; i += kBT) {
          const double2 v = rv[i];
          acc = fma(v.x, v.x, acc);
          acc = fma(v.y, v.y, acc);
        }
        red[tid] = acc;
        __syncthreads();
        for(int hh = kBT / 2; hh > 0; hh >>= 1) {
          if(tid < hh)
            red[tid] += red[tid + hh];
          __syncthreads();
        }
        tot = q0 == 0 ? red[0] : tot + red[0];
        __syncthreads();
      }
      if(tid == 0) {
        sl.k = 0;
        sl.inner = 0;
        const double rho = sqrt(tot);
        if(sl.bnorm < 0.0)
          sl.bnorm = rho;
        sl.rho = rho;
        if(sl.bnorm == 0.0 || rho <= a.tol * sl.bnorm) {
          sl.outer = 0;
          sl.status = OM_OK;
        } else if(sl.cycles >= a.max_cycles) {
          sl.outer = 0;
          sl.status = OM_ERR_NOT_CONVERGED;
        } else {
          sl.inner = 1;
          sl.thr = fmax(a.inner_rel * rho, a.tol * sl.bnorm);
          gs[0] = make_double2(rho, 0.0);
        }
      }
      __syncthreads();
      if(!sl.outer)
        break;
      // v_0 = r / rho (k_b_v0); the first product stages it from r
      const double f0 = 1.0 / sl.rho;
      for(long i = r0 + tid; i < r1; i += kBT) {
        const double2 v = rv[i];
        V o;
        o.x = v.x * f0;
        o.y = v.y * f0;
        vs[i] = o;
      }
      for(int j = 0;; ++j) {
        const int k = j + 1;
        // w = S v_j over the CTA's rows, chunk sums in chunk order (k_b_mv,
        // k_b_red_proj); v_j is staged from r / rho or from the previous
        // step's w times 1 / h_{j,j-1}, the values k_b_v0 / k_b_scale store
        const V *wp = wb + (long)((j + 1) & 1) * np;
        V acc[2];
        for(int cc = 0; cc < ns; ++cc) {
          const long j0 = (long)cc * kBCols, j1 = min(n, j0 + kBCols);
          __syncthreads();
          for(long jj = j0 + tid; jj < j1; jj += kBT) {
            V o;
            if(j == 0) {
              const double2 v = rv[jj];
              o.x = v.x * f0;
              o.y = v.y * f0;
            } else {
              const V v = wp[jj];
              o.x = v.x * inv_s;
              o.y = v.y * inv_s;
            }
            if constexpr(kDF) {
              if(Hf) {  // the values k_b_mv stages: v_j times each 256-row block's scales
#pragma unroll
                for(int q = 0; q < 2; ++q) {
                  if((2L * c + q) * 256 >= n)
                    break;  // no rows of the slot in this block (nor a scale column)
                  const float f = sl.D[(2L * c + q) * n + jj];
                  V t;
                  t.x = o.x * f;
                  t.y = o.y * f;
                  xs[q * kBCols + jj - j0] = t;
                }
                continue;
              }
            }
            xs[jj - j0] = o;
          }
          __syncthreads();
#pragma unroll
          for(int q = 0; q < 2; ++q) {
            const long i = r0 + q * kBT + tid;
            if(i >= r1)
              continue;
            V v;
            if constexpr(kDF) {
              if(Hf)
                v = mv_row<F16c, V>(Hf + j0 * n + i, n, xs + q * kBCols, 0L, j1 - j0);
              else
                v = mv_row<M, V>(S + j0 * n + i, n, xs, 0L, j1 - j0);
            } else {
              v = mv_row<M, V>(S + j0 * n + i, n, xs, 0L, j1 - j0);
            }
            if(cc == 0) {
              acc[q] = v;
            } else {
              acc[q].x += v.x;
              acc[q].y += v.y;
            }
          }
        }
#pragma unroll
        for(int q = 0; q < 2; ++q)
          if(r0 + q * kBT + tid < r1)
            w[q * kBT + tid] = acc[q];
        __syncthreads();
        if(r0 < r1)
          block_proj_sm(vs, w, np, r0, r1, k, dA + (long)c * m2);
        if(!group_barrier(ctr, target += C, C, a.err))
          return;
        // w -= V h, then the second projections (k_b_sub_proj, pass 0)
        gather_h(dA, nb, m2, k, h);
        for(int t = tid; t < k; t += kBT)
          hacc[t] = to_d2(h[t]);
        for(long i = r0 + tid; i < r1; i += kBT) {
          V v = w[i - r0];
          for(int t = 0; t < k; ++t) {
            V cf = h[t];
            cf.x = -cf.x;
            cf.y = -cf.y;
            v = cfma(vs[(long)t * np + i], cf, v);
          }
          w[i - r0] = v;
        }
        __syncthreads();
        if(r0 < r1)
          block_proj_sm(vs, w, np, r0, r1, k, dB + (long)c * m2);
        if(!group_barrier(ctr, target += C, C, a.err))
          return;
        // w -= V h and |w|^2 (k_b_sub_proj, pass 1); w kept for the next product
        gather_h(dB, nb, m2, k, h);
        for(int t = tid; t < k; t += kBT)
          hacc[t] = cadd(hacc[t], to_d2(h[t]));
        double nrm = 0.0;
        V *wn = wb + (long)(j & 1) * np;
        for(long i = r0 + tid; i < r1; i += kBT) {
          V v = w[i - r0];
          for(int t = 0; t < k; ++t) {
            V cf = h[t];
            cf.x = -cf.x;
            cf.y = -cf.y;
            v = cfma(vs[(long)t * np + i], cf, v);
          }
          w[i - r0] = v;
          wn[i] = v;
          nrm = fma((double)v.x, (double)v.x, nrm);
          nrm = fma((double)v.y, (double)v.y, nrm);
        }
        for(int o = 16; o > 0; o >>= 1)
          nrm += __shfl_xor_sync(0xffffffffu, nrm, o);
        if((tid & 31) == 0)
          red[tid >> 5] = nrm;
        __syncthreads();
        if(tid == 0 && r0 < r1) {
          double sum = 0.0;
          for(int q = 0; q < kBT / 32; ++q)
            sum += red[q];
          V *out = dA + (long)c * m2;
          out[m2 - 1].x = sum;
          out[m2 - 1].y = 0;
        }
        if(!group_barrier(ctr, target += C, C, a.err))
          return;
        // Hessenberg column j, rotations, |g_{j+1}| and the stop test (k_b_givens)
        if(tid == 0) {
          double accn = dA[m2 - 1].x;
          for(int q = 1; q < nb; ++q)
            accn += dA[(long)q * m2 + m2 - 1].x;
          const double hn = sqrt(accn);
          for(int t = 0; t <= j; ++t)
            col[t] = hacc[t];
          for(int i = 0; i < j; ++i) {
            const double2 p = col[i], q = col[i + 1];
            col[i] = cadd(cmul(cconj(c_s[i]), p), cmul(cconj(cneg(s_s[i])), q));
            col[i + 1] = cadd(cmul(s_s[i], p), cmul(c_s[i], q));
          }
          double2 cr, sr;
          const double2 hk1 = make_double2(hn, 0.0);
          givens_dev(col[j], hk1, cr, sr);
          c_s[j] = cr;
          s_s[j] = sr;
          const double2 hk = col[j];
          col[j] = cadd(cmul(cconj(cr), hk), cmul(cconj(cneg(sr)), hk1));
          const double2 g0 = gs[j];
          gs[j] = cmul(cconj(cr), g0);
          gs[j + 1] = cmul(sr, g0);
          inv_s = hn > 0.0 ? 1.0 / hn : 0.0;
          sl.k = j + 1;
          sl.steps++;
          sl.inner = !(cabs2(gs[j + 1]) <= sl.thr || hn == 0.0 || j + 1 >= m);
          if(c == 0)
            for(int t = 0; t <= j; ++t)
              H[(long)j * (m + 1) + t] = col[t];
        }
        __syncthreads();
        if(!sl.inner)
          break;
        // v_{j+1} = w / h_{j+1,j} (k_b_scale)
        for(long i = r0 + tid; i < r1; i += kBT) {
          const V v = w[i - r0];
          V o;
          o.x = v.x * inv_s;
          o.y = v.y * inv_s;
          vs[(long)(j + 1) * np + i] = o;
        }
      }
      // end of the cycle: y = R^{-1} g from CTA 0's columns (k_b_end), x += V y
      if(!group_barrier(ctr, target += C, C, a.err))
        return;
      if(tid == 0) {
        const int k = sl.k;
        for(int j = k - 1; j >= 0; --j) {
          double2 v = gs[j];
          for(int q = j + 1; q < k; ++q)
            v = cadd(v, cneg(cmul(H[(long)q * (m + 1) + j], ys[q])));
          ys[j] = cdiv(v, H[(long)j * (m + 1) + j]);
        }
        sl.cycles++;
        sl.xzero = 0;
      }
      __syncthreads();
      for(long i = r0 + tid; i < r1; i += kBT) {
        double2 v = xv[i];
        for(int t = 0; t < sl.k; ++t)
          v = cfma(to_d2(vs[(long)t * np + i]), ys[t], v);
        xv[i] = v;
      }
      if(!group_barrier(ctr, target += C, C, a.err))
        return;
    }
    if(tid == 0 && c == 0)
      a.st[s] = sl;
  }
}

// ---------------------------------------------------------------------------
// Size classes
// ---------------------------------------------------------------------------

// N padded to the class size: 1, 2, 3, 4, 6, 8, 12, 16, 24, ... (x1.5 / x1.33 steps)
int pad_spheres(int N) {
  int a = 1;
  while(a < N) {
    const int b = a < 2 ? 2 : (a & (a - 1)) == 0 ? a + a / 2 : a / 3 * 4;
    a = b;
  }
  return a;
}

struct ClassKey {
  int precision, nmax, Npad, m, max_cycles;
  double tol, inner_rel;
  int f16;  // precision form: the Arnoldi products read scaled fp16 copies of the matrices
  bool operator<(const ClassKey &o) const {
    return std::tie(precision, nmax, Npad, m, max_cycles, tol, inner_rel, f16) <
           std::tie(o.precision, o.nmax, o.Npad, o.m, o.max_cycles, o.tol, o.inner_rel, o.f16);
  }
};

inline size_t rup(size_t v) { return ((v + 255) / 256) * 256; }

// Tile shapes and schedules of the batched matvecs (k_b_mv, k_b_resid) that
// the autotuner chooses among, per size class: rows per tile (threads per
// CTA), the tile order (slot by slot, or interleaved across slots so that the
// counter spreads every slot over the SMs) and the grid (CTAs per SM; halved
// when the next batch's assembly runs beside the solves). None of them
// changes a row's sum (the 1,024-column chunks and their order are fixed), so
// a request's bits do not depend on the choice.
struct MvCfg {
  int rows, order, cap;
};
constexpr MvCfg kMvCands[] = {{256, 0, 8},  {256, 1, 8},  {128, 0, 8}, {128, 1, 8},
                              {256, 0, 16}, {128, 1, 16}, {256, 1, 4}, {128, 0, 4}};
constexpr int kNumMvCands = (int)(sizeof(kMvCands) / sizeof(kMvCands[0]));

// the autotuner's choices, per context and size class, kept beyond the
// class's buffers (which the cache may evict)
struct TunedEntry {
  om_context *ctx;
  int precision, nmax, Npad, m;
  int cand;
  double us;
};
std::mutex g_tuned_mu;
std::vector<TunedEntry> g_tuned;

// Device and pinned host buffers of one size class, and its graphs.
template <typename M, typename V> struct Class {
  om_context *ctx = nullptr;
  ClassKey key{};
  int B = 0, m = 0, m2 = 0, nsm = 0, nblk = 0, nbf = 0, max_tiles = 0;
  long np = 0, vslot = 0;
  unsigned mv_grid = 1;
  void *buf = nullptr;
  size_t bytes = 0;
  Slot *st = nullptr;
  Ctl *ctl = nullptr;
  int4 *tiles = nullptr;
  int nbuf = 1;                       // batches in flight: 2 when they overlap
  BatchMat *mats = nullptr;           // nbuf x 2B entries
  double2 *b = nullptr, *x = nullptr, *r = nullptr, *part = nullptr;
  V *Vb = nullptr;
  double2 *dpA = nullptr, *dpB = nullptr;  // block partial sums (two passes; entries of V or double2)
  double2 *hacc = nullptr, *Hm = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr;
  double *inv = nullptr;
  unsigned long long *counter = nullptr;
  // the fused solve (np <= kFusedRows): w of the last two steps per slot, the
  // groups' barrier counters and the give-up flag
  bool fused_ok = false;
  V *wbuf = nullptr;
  unsigned *fbar = nullptr;
  int *ferr = nullptr;
  int *h_ferr = nullptr;
  size_t fsmem = 0;
  int fcap = 0;  // CTAs of k_b_fused resident on the device
  // pinned host mirrors
  Slot *h_st = nullptr;
  Ctl *h_ctl = nullptr;
  int4 *h_tiles = nullptr;
  BatchMat *h_mats = nullptr;
  CvMat *h_cv = nullptr;  // nbuf x 2B: the fp16 conversion's matrix table
  CvMat *cv = nullptr;
  double *h_xsec = nullptr;  // 8 per slot: the FF and SH cross sections
  cudaEvent_t ev_main = nullptr;        // main stream -> auxiliary streams
  std::vector<cudaEvent_t> ev_aux;      // auxiliary streams -> main / assembly stream
  cudaEvent_t ev_asm[2] = {nullptr, nullptr};    // assembly of batch buffer i done
  cudaEvent_t ev_alloc[2] = {nullptr, nullptr};  // matrix storage of batch buffer i allocated
  cudaGraphExec_t g_start = nullptr, g_seg = nullptr, g_end = nullptr;
  int k_start = 0, k_seg = 0, k_end = 0;  // kernels per replay
  MvCfg mv = kMvCands[0];  // the matvec tiles and schedule (autotuned at the first solve)
  bool tuned = false;

  // device bytes of one slot's vectors and tables (the matrices are
  // allocated per batch at the requests' own sizes)
  static size_t slot_bytes(long np, int m, int nbuf) {
    const int m2 = m + 2;
    const long nsm = (np + kBCols - 1) / kBCols, nbf = (np + kFRows - 1) / kFRows;
    return 3 * sizeof(double2) * np +
           sizeof(V) * (size_t)(m + 1) * np + sizeof(double2) * (size_t)nsm * np +
           2 * sizeof(double2) * (size_t)nbf * m2 +
           sizeof(double2) * ((size_t)m2 + (size_t)m * (m + 1) + 2 * (size_t)m + (m + 1) + m) +
           sizeof(int4) * (size_t)((np + 127) / 128) * nsm + sizeof(Slot) +
           2 * nbuf * sizeof(BatchMat) + 64 + (np <= kFusedRows ? 2 * sizeof(V) * np + 128 : 0);
  }

  int init(om_context *c, const ClassKey &k, int slots, int buffers) {
    ctx = c;
    key = k;
    B = slots;
    nbuf = buffers;
    m = k.m;
    m2 = m + 2;
    np = (long)rup((size_t)2 * pmax(k.nmax) * k.Npad);
    vslot = (long)(m + 1) * np;
    nsm = (int)((np + kBCols - 1) / kBCols);
    nblk = (int)((np + kBDotRows - 1) / kBDotRows);
    nbf = (int)((np + kFRows - 1) / kFRows);
    max_tiles = B * (int)((np + 127) / 128) * nsm;  // (the smallest tiles)
    // the matrices are allocated per batch, at the requests' own sizes
    const size_t Bz = (size_t)B;
    size_t sz[] = {Bz * sizeof(Slot), sizeof(Ctl), sizeof(int4) * (size_t)max_tiles,
                   2 * Bz * nbuf * sizeof(BatchMat),
                   Bz * sizeof(double2) * np, Bz * sizeof(double2) * np, Bz * sizeof(double2) * np,
                   Bz * sizeof(double2) * nsm * np, Bz * sizeof(V) * vslot,
                   Bz * sizeof(double2) * nbf * m2, Bz * sizeof(double2) * nbf * m2,
                   Bz * sizeof(double2) * m2,
                   Bz * sizeof(double2) * m * (m + 1), Bz * sizeof(double2) * m,
                   Bz * sizeof(double2) * m, Bz * sizeof(double2) * (m + 1), Bz * sizeof(double2) * m,
                   Bz * sizeof(double), sizeof(unsigned long long),
                   np <= kFusedRows ? Bz * 2 * sizeof(V) * np : 0, Bz * 32 * sizeof(unsigned) + 16,
                   2 * Bz * nbuf * sizeof(CvMat)};
    bytes = 0;
    for(size_t v : sz)
      bytes += rup(v);
    int rc = dev_malloc(ctx, &buf, bytes);
    if(rc)
      return rc;
    char *p = (char *)buf;
    auto take = [&](size_t v) {
      void *q = p;
      p += rup(v);
      return q;
    };
    int i = 0;
    st = (Slot *)take(sz[i++]);
    ctl = (Ctl *)take(sz[i++]);
    tiles = (int4 *)take(sz[i++]);
    mats = (BatchMat *)take(sz[i++]);
    b = (double2 *)take(sz[i++]);
    x = (double2 *)take(sz[i++]);
    r = (double2 *)take(sz[i++]);
    part = (double2 *)take(sz[i++]);
    Vb = (V *)take(sz[i++]);
    dpA = (double2 *)take(sz[i++]);
    dpB = (double2 *)take(sz[i++]);
    hacc = (double2 *)take(sz[i++]);
    Hm = (double2 *)take(sz[i++]);
    cs = (double2 *)take(sz[i++]);
    sn = (double2 *)take(sz[i++]);
    g = (double2 *)take(sz[i++]);
    y = (double2 *)take(sz[i++]);
    inv = (double *)take(sz[i++]);
    counter = (unsigned long long *)take(sz[i++]);
    wbuf = (V *)take(sz[i++]);
    fbar = (unsigned *)take(sz[i++]);
    ferr = (int *)(fbar + 32 * Bz);
    cv = (CvMat *)take(sz[i++]);
    if(cudaMallocHost(&h_st, Bz * sizeof(Slot)) != cudaSuccess ||
       cudaMallocHost(&h_ferr, sizeof(int)) != cudaSuccess ||
       cudaMallocHost(&h_ctl, sizeof(Ctl)) != cudaSuccess ||
       cudaMallocHost(&h_tiles, sizeof(int4) * (size_t)max_tiles) != cudaSuccess ||
       cudaMallocHost(&h_mats, 2 * Bz * nbuf * sizeof(BatchMat)) != cudaSuccess ||
       cudaMallocHost(&h_cv, 2 * Bz * nbuf * sizeof(CvMat)) != cudaSuccess ||
       cudaMallocHost(&h_xsec, 8 * Bz * sizeof(double)) != cudaSuccess) {
      cudaGetLastError();
      ctx->err = "pinned host staging for the batch";
      return OM_ERR_CUDA;
    }
    cudaEventCreateWithFlags(&ev_main, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_asm[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_asm[1], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_alloc[0], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&ev_alloc[1], cudaEventDisableTiming);
    ev_aux.resize(ctx->aux.size());
    for(auto &e : ev_aux)
      cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    if(np <= kFusedRows) {
      // the fused solve: its shared memory and how many of its CTAs fit
      fsmem = FusedSmem<V>(m, m2).bytes;
      int coop = 0, per_sm = 0;
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
      // (the attribute is the largest any class asks for, so that classes on
      // other host threads never launch below a smaller setting)
      if(coop && fsmem <= kFusedSmemMax &&
         cudaFuncSetAttribute(k_b_fused<M, V>, cudaFuncAttributeMaxDynamicSharedMemorySize, kFusedSmemMax) ==
             cudaSuccess &&
         cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_b_fused<M, V>, kBT, fsmem) == cudaSuccess &&
         per_sm >= 1) {
        fcap = per_sm * ctx->sm_count;
        fused_ok = fcap >= nbf;
      }
      cudaGetLastError();
    }
    // a choice made for this class before (the graphs are captured once the
    // matvec configuration is known: here, or after the autotuning)
    {
      std::lock_guard<std::mutex> lk(g_tuned_mu);
      for(const TunedEntry &e : g_tuned)
        if(e.ctx == ctx && e.precision == key.precision && e.nmax == key.nmax && e.Npad == key.Npad &&
           e.m == key.m) {
          set_mv(e.cand);
          tuned = true;
        }
    }
    if(!tuned && ctx->batch_tiles > 0) {  // a configuration fixed by om_context_tune
      set_mv(std::min(ctx->batch_tiles, kNumMvCands) - 1);
      tuned = true;
    }
    return tuned ? capture() : OM_OK;
  }

  void set_mv(int cand) {
    mv = kMvCands[cand];
    // overlapping batches: half the SM's CTA slots, so that two CTAs of the
    // next batch's assembly (FP64-bound) fit beside the matvec (HBM-bound)
    const int cap = nbuf > 1 ? std::max(2, mv.cap / 2) : mv.cap;
    mv_grid = (unsigned)std::max(1L, std::min((long)max_tiles, (long)ctx->sm_count * cap));
  }

  // the tiles of the slots whose h_st entries have outer set, in the order of
  // configuration c; returns their count
  int build_tiles(const MvCfg &c) {
    int nt = 0;
    if(c.order == 0) {
      for(int s = 0; s < B; ++s) {
        const long n = h_st[s].outer ? h_st[s].n : 0;
        const int rt = (int)((n + c.rows - 1) / c.rows), ct = (int)((n + kBCols - 1) / kBCols);
        for(int cc = 0; cc < ct; ++cc)
          for(int q = 0; q < rt; ++q)
            h_tiles[nt++] = make_int4(s, q, cc, 0);
      }
    } else {
      int most = 0;
      for(int s = 0; s < B; ++s) {
        const long n = h_st[s].outer ? h_st[s].n : 0;
        most = std::max(most, (int)(((n + c.rows - 1) / c.rows) * ((n + kBCols - 1) / kBCols)));
      }
      for(int p = 0; p < most; ++p)
        for(int s = 0; s < B; ++s) {
          const long n = h_st[s].outer ? h_st[s].n : 0;
          const int rt = (int)((n + c.rows - 1) / c.rows), ct = (int)((n + kBCols - 1) / kBCols);
          if(p < rt * ct)
            h_tiles[nt++] = make_int4(s, p % rt, p / rt, 0);
        }
    }
    return nt;
  }

  void launch_mv(cudaStream_t s) {
    if constexpr(std::is_same<M, float2>::value) {
      if(key.f16) {
        if(mv.rows == 128)
          k_b_mv<F16c, V, 128><<<mv_grid, 128, 0, s>>>(st, tiles, ctl, Vb, vslot, np, nsm, (V *)part, counter);
        else
          k_b_mv<F16c, V, 256><<<mv_grid, 256, 0, s>>>(st, tiles, ctl, Vb, vslot, np, nsm, (V *)part, counter);
        return;
      }
    }
    if(mv.rows == 128)
      k_b_mv<M, V, 128><<<mv_grid, 128, 0, s>>>(st, tiles, ctl, Vb, vslot, np, nsm, (V *)part, counter);
    else
      k_b_mv<M, V, 256><<<mv_grid, 256, 0, s>>>(st, tiles, ctl, Vb, vslot, np, nsm, (V *)part, counter);
  }
  void launch_resid(cudaStream_t s) {
    if(mv.rows == 128)
      k_b_resid<M, 128><<<mv_grid, 128, 0, s>>>(st, tiles, ctl, x, np, nsm, part, counter);
    else
      k_b_resid<M, 256><<<mv_grid, 256, 0, s>>>(st, tiles, ctl, x, np, nsm, part, counter);
  }

  // The autotuner: times the Arnoldi matvec of this batch's matrices (every
  // slot with a system) under each candidate configuration (best of three
  // launches; the product lands in scratch), keeps the fastest for the class,
  // and captures the graphs with it.
  int autotune() {
    std::vector<Slot> probe(h_st, h_st + B);
    for(Slot &sl : probe)
      sl.inner = sl.outer && sl.n > 0;
    cudaMemcpyAsync(st, probe.data(), sizeof(Slot) * B, cudaMemcpyHostToDevice, ctx->stream);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best = 0;
    float best_ms = 1e30f;
    for(int c = 0; c < kNumMvCands; ++c) {
      set_mv(c);
      h_ctl->j = 0;
      h_ctl->n_inner = h_ctl->n_outer = 0;
      h_ctl->ntiles = build_tiles(mv);
      cudaMemcpyAsync(ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, ctx->stream);
      if(h_ctl->ntiles)
        cudaMemcpyAsync(tiles, h_tiles, sizeof(int4) * h_ctl->ntiles, cudaMemcpyHostToDevice, ctx->stream);
      float ms_min = 1e30f;
      for(int rep = 0; rep < 3; ++rep) {
        cudaMemsetAsync(counter, 0, sizeof(unsigned long long), ctx->stream);
        cudaEventRecord(e0, ctx->stream);
        launch_mv(ctx->stream);
        cudaEventRecord(e1, ctx->stream);
        if(cudaEventSynchronize(e1) != cudaSuccess)
          break;
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms_min = std::min(ms_min, ms);
      }
      if(ms_min < best_ms) {
        best_ms = ms_min;
        best = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const cudaError_t e = cudaGetLastError();
    if(e != cudaSuccess) {
      ctx->err = std::string("batch autotuning: ") + cudaGetErrorString(e);
      return OM_ERR_CUDA;
    }
    set_mv(best);
    tuned = true;
    {
      std::lock_guard<std::mutex> lk(g_tuned_mu);
      g_tuned.push_back(TunedEntry{ctx, key.precision, key.nmax, key.Npad, key.m, best, 1e3 * best_ms});
    }
    return capture();
  }

  ~Class() {
    if(g_start) cudaGraphExecDestroy(g_start);
    if(g_seg) cudaGraphExecDestroy(g_seg);
    if(g_end) cudaGraphExecDestroy(g_end);
    if(buf) {
      cudaStreamSynchronize(ctx->stream);
      dev_release(ctx, buf, bytes);
    }
    if(h_st) cudaFreeHost(h_st);
    if(h_ctl) cudaFreeHost(h_ctl);
    if(h_tiles) cudaFreeHost(h_tiles);
    if(h_mats) cudaFreeHost(h_mats);
    if(h_cv) cudaFreeHost(h_cv);
    if(h_xsec) cudaFreeHost(h_xsec);
    if(h_ferr) cudaFreeHost(h_ferr);
    if(ev_main) cudaEventDestroy(ev_main);
    for(auto &e : ev_asm)
      if(e) cudaEventDestroy(e);
    for(auto &e : ev_alloc)
      if(e) cudaEventDestroy(e);
    for(auto &e : ev_aux)
      if(e) cudaEventDestroy(e);
  }

  dim3 vgrid() const { return dim3((unsigned)((np + kBT - 1) / kBT), (unsigned)B); }
  int ctl_threads() const { return ((B + 31) / 32) * 32; }

  // cycle start: r = b - S x, ||r||, the test, v_0
  int enqueue_start(cudaStream_t s) {
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    launch_resid(s);
    k_b_reduce_r<<<vgrid(), kBT, 0, s>>>(st, part, np, nsm, b, r);
    k_b_rnorm<<<dim3(nblk, B), kBT, 0, s>>>(st, r, np, nblk, m2, dpA);
    k_b_start<<<1, ctl_threads(), 0, s>>>(st, ctl, dpA, nblk, m2, g, m, B, key.tol, key.inner_rel,
                                          key.max_cycles);
    k_b_v0<V><<<vgrid(), kBT, 0, s>>>(st, r, np, Vb, vslot);
    return 5;
  }
  // one Arnoldi step with CGS2: the matvec; w and the first projections;
  // subtraction and the second projections; subtraction and |w|^2; the
  // rotation; the scaling
  int enqueue_step(cudaStream_t s) {
    V *pA = (V *)dpA, *pB = (V *)dpB;
    const dim3 fg((unsigned)nbf, (unsigned)B);
    const size_t hsm = sizeof(V) * m2;
    cudaMemsetAsync(counter, 0, sizeof(unsigned long long), s);
    launch_mv(s);
    k_b_red_proj<V><<<fg, kBT, 0, s>>>(st, ctl, (const V *)part, np, nsm, Vb, vslot, nbf, m2, pA);
    k_b_sub_proj<V><<<fg, kBT, hsm, s>>>(st, ctl, Vb, vslot, np, nbf, m2, pA, pB, hacc, 0);
    k_b_sub_proj<V><<<fg, kBT, hsm, s>>>(st, ctl, Vb, vslot, np, nbf, m2, pB, pA, hacc, 1);
    k_b_givens<V><<<1, ctl_threads(), 0, s>>>(st, ctl, pA, nbf, m2, hacc, Hm, cs, sn, g, inv, m, B);
    k_b_scale<V><<<vgrid(), kBT, 0, s>>>(st, ctl, inv, Vb, vslot, np);
    return 6;
  }
  int enqueue_end(cudaStream_t s) {
    k_b_end<<<1, ctl_threads(), 0, s>>>(st, Hm, g, y, m, B);
    k_b_update<V><<<vgrid(), kBT, 0, s>>>(st, Vb, vslot, np, y, m, x);
    return 2;
  }

  int capture_one(cudaGraphExec_t *out, int which, int *kernels) {
    cudaStream_t s = ctx->stream;
    cudaGraph_t gr = nullptr;
    if(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return OM_ERR_CUDA;
    int k = 0;
    if(which == 0)
      k = enqueue_start(s);
    else if(which == 1)
      for(int t = 0; t < kSegSteps; ++t)
        k += enqueue_step(s);
    else
      k = enqueue_end(s);
    cudaError_t e = cudaStreamEndCapture(s, &gr);
    if(e == cudaSuccess)
      e = cudaGraphInstantiate(out, gr, 0);
    if(gr)
      cudaGraphDestroy(gr);
    if(e != cudaSuccess) {
      cudaGetLastError();
      ctx->err = std::string("batch graph capture: ") + cudaGetErrorString(e);
      return OM_ERR_CUDA;
    }
    *kernels = k;
    return OM_OK;
  }
  int capture() {
    int rc = capture_one(&g_start, 0, &k_start);
    if(!rc) rc = capture_one(&g_seg, 1, &k_seg);
    if(!rc) rc = capture_one(&g_end, 2, &k_end);
    return rc;
  }

  int read_ctl() {
    cudaMemcpyAsync(h_ctl, ctl, sizeof(Ctl), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(e != cudaSuccess) {
      ctx->err = std::string("batched solve: ") + cudaGetErrorString(e);
      return OM_ERR_CUDA;
    }
    return OM_OK;
  }

  // The fused form of solve(): one cooperative launch of k_b_fused, a group of
  // nbf CTAs per slot, as many groups as fit (at most one per slot with a
  // system).
  int solve_fused(long *launches) {
    int active = 0;
    for(int s = 0; s < B; ++s)
      active += h_st[s].n > 0 && h_st[s].outer;
    cudaMemcpyAsync(st, h_st, sizeof(Slot) * B, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(x, 0, sizeof(double2) * B * np, ctx->stream);
    cudaMemsetAsync(fbar, 0, sizeof(unsigned) * 32 * B + 16, ctx->stream);
    if(active) {
      const int groups = std::max(1, std::min(active, fcap / nbf));
      FusedArgs<V> fa{st, B, b, x, r, Vb, vslot, np, wbuf, (V *)dpA, (V *)dpB, Hm, m, m2, nbf, nbf,
                      key.tol, key.inner_rel, key.max_cycles, fbar, ferr};
      void *args[] = {&fa};
      cudaError_t e = cudaLaunchCooperativeKernel((const void *)k_b_fused<M, V>, dim3((unsigned)(groups * nbf)),
                                                  dim3(kBT), args, fsmem, ctx->stream);
      if(e != cudaSuccess) {
        ctx->err = std::string("fused batched solve: ") + cudaGetErrorString(e);
        return OM_ERR_CUDA;
      }
      ++*launches;
    }
    cudaMemcpyAsync(h_st, st, sizeof(Slot) * B, cudaMemcpyDeviceToHost, ctx->stream);
    cudaMemcpyAsync(h_ferr, ferr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(e != cudaSuccess) {
      ctx->err = std::string("fused batched solve: ") + cudaGetErrorString(e);
      return OM_ERR_CUDA;
    }
    if(*h_ferr) {
      ctx->err = "fused batched solve: a group barrier wait timed out";
      return OM_ERR_CUDA;
    }
    return OM_OK;
  }

  // Solve the systems of the slots whose h_st entries are set (uploaded here):
  // replays the graphs until no slot needs another cycle.
  int solve(long *launches) {
    if(fused_ok && (ctx->batch_fused == 2 || (ctx->batch_fused == 1 && np <= kFusedAuto)))
      return solve_fused(launches);
    if(!tuned) {
      const int rc = autotune();
      if(rc)
        return rc;
    }
    const int nt = build_tiles(mv);
    h_ctl->j = 0;
    h_ctl->n_inner = 0;
    h_ctl->n_outer = 0;
    h_ctl->ntiles = nt;
    cudaMemcpyAsync(st, h_st, sizeof(Slot) * B, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(ctl, h_ctl, sizeof(Ctl), cudaMemcpyHostToDevice, ctx->stream);
    if(nt)
      cudaMemcpyAsync(tiles, h_tiles, sizeof(int4) * nt, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(x, 0, sizeof(double2) * B * np, ctx->stream);
    // each cycle ends within m steps, and a slot runs at most max_cycles cycles
    const long guard = (long)(key.max_cycles + 2) * (m / kSegSteps + 2) + 8;
    long rounds = 0;
    for(;;) {
      cudaGraphLaunch(g_start, ctx->stream);
      cudaGraphLaunch(g_seg, ctx->stream);
      *launches += k_start + k_seg;
      int rc = read_ctl();
      if(rc)
        return rc;
      if(h_ctl->n_outer == 0)
        break;
      while(h_ctl->n_inner > 0) {
        if(++rounds > guard) {
          ctx->err = "batched solve: iteration guard reached";
          return OM_ERR_CUDA;
        }
        cudaGraphLaunch(g_seg, ctx->stream);
        *launches += k_seg;
        rc = read_ctl();
        if(rc)
          return rc;
      }
      cudaGraphLaunch(g_end, ctx->stream);
      *launches += k_end;
      if(++rounds > guard) {
        ctx->err = "batched solve: iteration guard reached";
        return OM_ERR_CUDA;
      }
    }
    cudaMemcpyAsync(h_st, st, sizeof(Slot) * B, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(e != cudaSuccess) {
      ctx->err = std::string("batched solve: ") + cudaGetErrorString(e);
      return OM_ERR_CUDA;
    }
    return OM_OK;
  }
};

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

void fill_stats(const Slot &sl, bool mixed, double seconds, om_solve_stats *o) {
  o->iterations = mixed ? sl.cycles : sl.steps;
  o->inner_iterations = mixed ? sl.steps : 0;
  o->rel_residual = sl.bnorm > 0 ? sl.rho / sl.bnorm : 0.0;
  o->seconds = seconds;
}

// Auxiliary contexts of `ctx` (created on first use, kept with it): the
// per-request set-up and post-processing kernels are small (one CTA per
// sphere), so the requests of a batch spread them over kAux streams.
constexpr int kAux = 8;
int aux_contexts(om_context *ctx) {
  while((int)ctx->aux.size() < kAux) {
    om_context *a = nullptr;
    int rc = om_context_create(ctx->device, 0, &a);
    if(rc) {
      ctx->err = "cannot create an auxiliary context for the batch";
      return rc;
    }
    a->parent = ctx;
    ctx->aux.push_back(a);
  }
  return OM_OK;
}

// Stream-order the auxiliary streams after the main stream (to_aux) or the
// main stream after the auxiliary ones.
void join(om_context *ctx, cudaEvent_t ev_main, const std::vector<cudaEvent_t> &ev_aux, bool to_aux) {
  if(to_aux) {
    cudaEventRecord(ev_main, ctx->stream);
    for(om_context *a : ctx->aux)
      cudaStreamWaitEvent(a->stream, ev_main, 0);
  } else {
    for(size_t q = 0; q < ctx->aux.size(); ++q) {
      cudaEventRecord(ev_aux[q], ctx->aux[q]->stream);
      cudaStreamWaitEvent(ctx->stream, ev_aux[q], 0);
    }
  }
}

// A batch between its set-up and its results.
struct Pending {
  std::vector<om_problem *> pr;  // per slot; null where set-up failed
  size_t b0 = 0;                 // first request (index into the class's list)
  int nb = 0;                    // requests
  int buf = 0;                   // mats table / event set
  double t0 = 0;                 // host time when its set-up started
  void *mbuf = nullptr;          // the batch's FF and SH matrices
  size_t mbytes = 0;
  std::vector<size_t> off_ff, off_sh;  // per slot: element offsets into mbuf
  // precision form with fp16 copies: mbuf = [complex64 matrices][their fp16
  // copies at the same offsets][scales]; scale offsets per slot
  size_t elems = 0, scales = 0;
  std::vector<size_t> soff_ff, soff_sh;
  F16c *copies() const { return reinterpret_cast<F16c *>(static_cast<float2 *>(mbuf) + elems); }
  float *scale_base() const { return reinterpret_cast<float *>(copies() + elems); }
};

// Set-up of a batch and its assembly: request s lives on auxiliary context
// s % kAux (per-sphere terms, incident coefficients, source vector); then one
// launch on the low-priority stream assembles the FF and SH matrices of every
// request into matrix buffer `buf`, so that it can overlap the solves of the
// previous batch on the main stream.
template <typename M, typename V>
void prepare_batch(om_context *ctx, const ClassKey &key, Class<M, V> &cl, const std::vector<int> &idx,
                   const om_request *reqs, om_result *out, double t_call, Pending &P, long *launches) {
  const long np = cl.np;
  P.t0 = now_ms();
  P.pr.assign(P.nb, nullptr);
  for(int s = 0; s < P.nb; ++s) {
    const om_request &rq = reqs[idx[P.b0 + s]];
    om_result &res = out[idx[P.b0 + s]];
    res.slot = s;
    res.queue_ms = P.t0 - t_call;
    om_context *a = ctx->aux[s % kAux];
    int r = om_problem_create(a, rq.spheres, rq.n_spheres, &rq.background, &rq.wave, &P.pr[s]);
    *launches += a->last_launches;
    if(r) {
      res.status = r;
      ctx->err = a->err;
      P.pr[s] = nullptr;
      continue;
    }
    const int L0 = a->last_launches;
    launch_source(P.pr[s]);
    *launches += a->last_launches - L0;
    P.pr[s]->have_source = true;
  }
  // matrix storage at the requests' own sizes (column-major, ld = n)
  P.off_ff.assign(P.nb, 0);
  P.off_sh.assign(P.nb, 0);
  size_t elems = 0;
  for(int s = 0; s < P.nb; ++s) {
    if(!P.pr[s])
      continue;
    const size_t nn = (size_t)P.pr[s]->n * P.pr[s]->n;
    P.off_ff[s] = elems;
    elems += nn;
    if(reqs[idx[P.b0 + s]].wave.sh) {
      P.off_sh[s] = elems;
      elems += nn;
    }
  }
  // the fp16 copies and their scales (ceil(n / 256) x n per matrix)
  P.elems = elems;
  P.scales = 0;
  P.soff_ff.assign(P.nb, 0);
  P.soff_sh.assign(P.nb, 0);
  if(key.f16)
    for(int s = 0; s < P.nb; ++s) {
      if(!P.pr[s])
        continue;
      const size_t n = (size_t)P.pr[s]->n, ns = (n + 255) / 256 * n;
      P.soff_ff[s] = P.scales;
      P.scales += ns;
      if(reqs[idx[P.b0 + s]].wave.sh) {
        P.soff_sh[s] = P.scales;
        P.scales += ns;
      }
    }
  P.mbytes = std::max<size_t>(elems, 1) * sizeof(M) +
             (key.f16 ? elems * sizeof(F16c) + P.scales * sizeof(float) : 0);
  if(dev_malloc(ctx, &P.mbuf, P.mbytes)) {
    P.mbuf = nullptr;
    for(int s = 0; s < P.nb; ++s)
      if(P.pr[s]) {
        out[idx[P.b0 + s]].status = OM_ERR_BUDGET;
        om_problem_destroy(P.pr[s]);
        P.pr[s] = nullptr;
      }
  }
  cudaEventRecord(cl.ev_alloc[P.buf], ctx->stream);
  cudaStreamWaitEvent(ctx->stream_lo, cl.ev_alloc[P.buf], 0);
  for(size_t q = 0; q < ctx->aux.size(); ++q) {
    cudaEventRecord(cl.ev_aux[q], ctx->aux[q]->stream);
    cudaStreamWaitEvent(ctx->stream_lo, cl.ev_aux[q], 0);
  }
  M *S = (M *)P.mbuf;
  // FF matrices in entries 0 .. B-1, SH in B .. 2B-1 of this buffer's table
  BatchMat *hm = cl.h_mats + (size_t)2 * cl.B * P.buf;
  for(int e = 0; e < 2 * cl.B; ++e)
    hm[e] = BatchMat{nullptr, nullptr, nullptr, 0, mk(0.0, 0.0), 0};
  bool any_sh = false;
  for(int s = 0; s < P.nb; ++s) {
    om_problem *p = P.pr[s];
    if(!p)
      continue;
    const cplx k = p->waveK;
    hm[s] = BatchMat{p->d_cart, p->d_T, S + P.off_ff[s], p->n, mk(k.real(), k.imag()), p->N};
    if(reqs[idx[P.b0 + s]].wave.sh) {
      any_sh = true;
      const cplx k2 = 2.0 * k;
      hm[cl.B + s] = BatchMat{p->d_cart, p->d_Tsh, S + P.off_sh[s], p->n, mk(k2.real(), k2.imag()),
                              p->N};
    }
  }
  const int nmats = any_sh ? 2 * cl.B : cl.B;
  BatchMat *dm = cl.mats + (size_t)2 * cl.B * P.buf;
  cudaMemcpyAsync(dm, hm, sizeof(BatchMat) * nmats, cudaMemcpyHostToDevice, ctx->stream_lo);
  const int L0 = ctx->last_launches;
  launch_assemble_batch(ctx, key.nmax, key.precision, dm, nmats, (int)((long)key.Npad * (key.Npad + 1) / 2),
                        ctx->stream_lo);
  *launches += ctx->last_launches - L0;
  if constexpr(std::is_same<M, float2>::value) {
    if(key.f16 && P.mbuf) {  // the fp16 copies, on the same stream after the assembly
      CvMat *hc = cl.h_cv + (size_t)2 * cl.B * P.buf;
      int nc = 0;
      long items = 0;
      for(int s = 0; s < P.nb; ++s) {
        if(!P.pr[s])
          continue;
        const long n = P.pr[s]->n, per = (n + 255) / 256 * n;
        hc[nc++] = CvMat{S + P.off_ff[s], P.copies() + P.off_ff[s], P.scale_base() + P.soff_ff[s], n, items};
        items += per;
        if(reqs[idx[P.b0 + s]].wave.sh) {
          hc[nc++] = CvMat{S + P.off_sh[s], P.copies() + P.off_sh[s], P.scale_base() + P.soff_sh[s], n, items};
          items += per;
        }
      }
      if(nc) {
        CvMat *dc = cl.cv + (size_t)2 * cl.B * P.buf;
        cudaMemcpyAsync(dc, hc, sizeof(CvMat) * nc, cudaMemcpyHostToDevice, ctx->stream_lo);
        const long blocks = std::min<long>((items + 7) / 8, 8L * ctx->sm_count);
        k_b_tof16<<<(unsigned)blocks, 256, 0, ctx->stream_lo>>>(dc, nc, items);
        ++*launches;
      }
    }
  }
  cudaEventRecord(cl.ev_asm[P.buf], ctx->stream_lo);
}

// The FF solves, the SH sources, the SH solves and the cross sections of a
// prepared batch.
template <typename M, typename V>
int finish_batch(om_context *ctx, const ClassKey &key, Class<M, V> &cl, const std::vector<int> &idx,
                 const om_request *reqs, om_result *out, double t_call, Pending &P, long *launches) {
  const bool mixed = key.precision == OM_C64;
  const long np = cl.np;
  const size_t per = Class<M, V>::slot_bytes(np, key.m, cl.nbuf);
  std::vector<om_problem *> &pr = P.pr;
  const int nb = P.nb;
  auto actx = [&](int s) { return ctx->aux[s % kAux]; };
  auto tracked = [&](om_context *c, auto &&fn) {
    const int L0 = c->last_launches;
    fn();
    *launches += c->last_launches - L0;
  };
  cudaStreamWaitEvent(ctx->stream, cl.ev_asm[P.buf], 0);
  // FF systems
  for(int s = 0; s < cl.B; ++s) {
    Slot z{};
    z.bnorm = -1.0;
    z.xzero = 1;
    if(s < nb && pr[s]) {
      z.n = pr[s]->n;
      z.S = (const M *)P.mbuf + P.off_ff[s];
      if(key.f16) {
        z.H = P.copies() + P.off_ff[s];
        z.D = P.scale_base() + P.soff_ff[s];
      }
      z.outer = 1;
      cudaMemcpyAsync(cl.b + (size_t)s * np, pr[s]->d_Q, sizeof(double2) * z.n,
                      cudaMemcpyDeviceToDevice, ctx->stream);
    }
    cl.h_st[s] = z;
  }
  const double ts = now_ms();
  int rc = cl.solve(launches);
  const double t_ff = (now_ms() - ts) * 1e-3;
  if(rc)
    return rc;
  // FF results and the SH sources, on the auxiliary streams
  join(ctx, cl.ev_main, cl.ev_aux, true);
  std::vector<Slot> ff(cl.h_st, cl.h_st + cl.B);
  for(int s = 0; s < nb; ++s) {
    if(!pr[s])
      continue;
    om_result &res = out[idx[P.b0 + s]];
    fill_stats(ff[s], mixed, t_ff, &res.ff);
    res.status = ff[s].status;
    om_context *a = actx(s);
    cudaMemcpyAsync(pr[s]->d_X, cl.x + (size_t)s * np, sizeof(double2) * pr[s]->n,
                    cudaMemcpyDeviceToDevice, a->stream);
    tracked(a, [&] {
      launch_internal(pr[s]);
      launch_cross_sections(pr[s]);
    });
    pr[s]->have_solution = true;
    if(reqs[idx[P.b0 + s]].wave.sh) {
      int r = sh_alloc(pr[s]);
      if(r) {
        res.status = r;
        ctx->err = a->err;
        continue;
      }
      tracked(a, [&] { launch_sh_source(pr[s]); });
    }
  }
  join(ctx, cl.ev_main, cl.ev_aux, false);
  // SH systems
  bool run = false;
  for(int s = 0; s < cl.B; ++s) {
    Slot z{};
    z.bnorm = -1.0;
    z.xzero = 1;
    if(s < nb && pr[s] && reqs[idx[P.b0 + s]].wave.sh && pr[s]->d_K && pr[s]->d_acs) {
      z.n = pr[s]->n;
      z.S = (const M *)P.mbuf + P.off_sh[s];
      if(key.f16) {
        z.H = P.copies() + P.off_sh[s];
        z.D = P.scale_base() + P.soff_sh[s];
      }
      z.outer = 1;
      run = true;
      cudaMemcpyAsync(cl.b + (size_t)s * np, pr[s]->d_K, sizeof(double2) * z.n,
                      cudaMemcpyDeviceToDevice, ctx->stream);
    }
    cl.h_st[s] = z;
  }
  double t_sh = 0.0;
  if(run) {
    const double t1 = now_ms();
    rc = cl.solve(launches);
    t_sh = (now_ms() - t1) * 1e-3;
    if(rc)
      return rc;
  }
  // SH results; every request's cross sections into pinned memory
  join(ctx, cl.ev_main, cl.ev_aux, true);
  double *hx = cl.h_xsec;
  for(int s = 0; s < nb; ++s) {
    if(!pr[s])
      continue;
    om_context *a = actx(s);
    if(run && cl.h_st[s].n) {
      om_result &res = out[idx[P.b0 + s]];
      fill_stats(cl.h_st[s], mixed, t_sh, &res.sh);
      if(res.status == OM_OK)
        res.status = cl.h_st[s].status;
      cudaMemcpyAsync(pr[s]->d_Xsh, cl.x + (size_t)s * np, sizeof(double2) * pr[s]->n,
                      cudaMemcpyDeviceToDevice, a->stream);
      tracked(a, [&] {
        launch_sh_internal(pr[s]);
        launch_sh_cross_sections(pr[s], pr[s]->d_xsec + 4);
      });
      pr[s]->have_sh = true;
    }
    cudaMemcpyAsync(hx + 8 * s, pr[s]->d_xsec, sizeof(double) * 6, cudaMemcpyDeviceToHost, a->stream);
  }
  cudaError_t e = cudaSuccess;
  for(om_context *a : ctx->aux) {
    cudaError_t ea = cudaStreamSynchronize(a->stream);
    if(e == cudaSuccess)
      e = ea;
  }
  if(e == cudaSuccess)
    e = cudaGetLastError();
  const double t_end = now_ms();
  for(int s = 0; s < nb; ++s) {
    om_result &res = out[idx[P.b0 + s]];
    if(pr[s]) {
      for(int q = 0; q < 4; ++q)
        res.xsec[q] = hx[8 * s + q];
      if(reqs[idx[P.b0 + s]].wave.sh)
        for(int q = 0; q < 2; ++q)
          res.xsec_sh[q] = hx[8 * s + 4 + q];
    }
    res.service_ms = t_end - P.t0;
    res.latency_ms = t_end - t_call;
    res.device_bytes = per;
  }
  if(e != cudaSuccess) {
    ctx->err = std::string("batch: ") + cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  return OM_OK;
}

// Class workspaces are kept between calls, per context, so that a serving
// loop that calls om_batch_solve for small runs does not rebuild the arena,
// the pinned staging and the graphs of a size class each time. Entries not
// in use are evicted least recently used beyond kCacheBytes per context.
struct CacheEntry {
  om_context *ctx;
  ClassKey key;
  int B, nbuf;
  void *cls;
  void (*del)(void *);
  size_t bytes;
  unsigned long long last;
};
std::mutex g_cache_mu;
std::vector<CacheEntry> g_cache;
unsigned long long g_cache_clock = 0;
constexpr size_t kCacheBytes = size_t(4) << 30;

bool same_key(const ClassKey &a, const ClassKey &b) { return !(a < b) && !(b < a); }

template <typename M, typename V> Class<M, V> *cache_take(om_context *ctx, const ClassKey &key, int B, int nbuf) {
  std::lock_guard<std::mutex> lk(g_cache_mu);
  for(size_t i = 0; i < g_cache.size(); ++i) {
    CacheEntry &e = g_cache[i];
    if(e.ctx == ctx && same_key(e.key, key) && e.B >= B && e.nbuf >= nbuf) {
      Class<M, V> *cl = static_cast<Class<M, V> *>(e.cls);
      g_cache.erase(g_cache.begin() + i);
      return cl;
    }
  }
  return nullptr;
}

template <typename M, typename V> void cache_put(om_context *ctx, Class<M, V> *cl) {
  std::vector<CacheEntry> victims;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    g_cache.push_back(CacheEntry{ctx, cl->key, cl->B, cl->nbuf, cl,
                                 [](void *p) { delete static_cast<Class<M, V> *>(p); }, cl->bytes,
                                 ++g_cache_clock});
    for(;;) {
      size_t total = 0;
      long oldest = -1;
      for(size_t i = 0; i < g_cache.size(); ++i)
        if(g_cache[i].ctx == ctx) {
          total += g_cache[i].bytes;
          if(oldest < 0 || g_cache[i].last < g_cache[oldest].last)
            oldest = (long)i;
        }
      if(total <= kCacheBytes || oldest < 0)
        break;
      victims.push_back(g_cache[oldest]);
      g_cache.erase(g_cache.begin() + oldest);
    }
  }
  for(auto &v : victims)
    v.del(v.cls);
}

// The requests idx of one size class, in batches of B slots; with more than
// one batch, the next batch's set-up and assembly are issued before the
// current batch's solves (two matrix buffers).
template <typename M, typename V>
int run_class(om_context *ctx, const ClassKey &key, const std::vector<int> &idx, const om_request *reqs,
              om_result *out, size_t arena, double t_call, long *launches) {
  const long np = (long)rup((size_t)2 * pmax(key.nmax) * key.Npad);
  // tables the auxiliary contexts share, ready before their streams use them
  int rc = aux_contexts(ctx);
  if(rc)
    return rc;
  coef_tables(ctx, key.nmax);
  clg_tables_dev(ctx, key.nmax);
  cudaStreamSynchronize(ctx->stream);
  const size_t count = idx.size();
  // a slot holds its vectors and, per batch in flight, the largest request's
  // matrices
  size_t maxmat = 0;
  for(int i : idx) {
    const size_t n = 2 * (size_t)pmax(key.nmax) * reqs[i].n_spheres;
    maxmat = std::max(maxmat, (sizeof(M) * n * n + (key.f16 ? sizeof(F16c) * n * n + 4 * n * ((n + 255) / 256) : 0)) *
                                  (reqs[i].wave.sh ? 2 : 1));
  }
  auto slots_for = [&](int nbuf) {
    const size_t per = Class<M, V>::slot_bytes(np, key.m, nbuf) + nbuf * maxmat;
    return (int)std::min<size_t>({count, (size_t)kMaxSlots, std::max<size_t>(1, arena / per)});
  };
  int nbuf = (size_t)slots_for(1) < count ? 2 : 1;
  int B = slots_for(nbuf);
  // a cached workspace with at least B slots serves (batches stay at B)
  Class<M, V> *cl = cache_take<M, V>(ctx, key, B, nbuf);
  while(!cl) {
    cl = new Class<M, V>();
    rc = cl->init(ctx, key, B, nbuf);
    if(!rc)
      break;
    delete cl;
    cl = nullptr;
    if(rc != OM_ERR_BUDGET || (B == 1 && nbuf == 1))
      break;
    if(B == 1)
      nbuf = 1;
    else
      B = (B + 1) / 2;
  }
  if(!cl) {
    for(int i : idx)
      out[i].status = rc;
    return OM_OK;
  }
  std::vector<Pending> pend;
  for(size_t b0 = 0; b0 < count; b0 += B) {
    Pending P;
    P.b0 = b0;
    P.nb = (int)std::min<size_t>(B, count - b0);
    P.buf = (int)(pend.size() % cl->nbuf);
    pend.push_back(P);
  }
  auto destroy = [ctx](Pending &P) {
    for(om_problem *p : P.pr)
      if(p)
        om_problem_destroy(p);
    P.pr.clear();
    if(P.mbuf)
      dev_release(ctx, P.mbuf, P.mbytes);
    P.mbuf = nullptr;
  };
  if(!pend.empty())
    prepare_batch(ctx, key, *cl, idx, reqs, out, t_call, pend[0], launches);
  for(size_t k = 0; k < pend.size(); ++k) {
    if(!rc && k + 1 < pend.size() && cl->nbuf > 1)
      prepare_batch(ctx, key, *cl, idx, reqs, out, t_call, pend[k + 1], launches);
    if(!rc)
      rc = finish_batch(ctx, key, *cl, idx, reqs, out, t_call, pend[k], launches);
    if(rc) {  // device error: wait for what is in flight before freeing
      cudaStreamSynchronize(ctx->stream_lo);
      cudaStreamSynchronize(ctx->stream);
    }
    destroy(pend[k]);
    if(!rc && k + 1 < pend.size() && cl->nbuf == 1)
      prepare_batch(ctx, key, *cl, idx, reqs, out, t_call, pend[k + 1], launches);
  }
  for(auto &P : pend)
    destroy(P);
  cudaStreamSynchronize(ctx->stream_lo);
  if(rc)
    delete cl;
  else
    cache_put(ctx, cl);
  return rc;
}

}  // namespace

// Drops the class workspaces cached for ctx (called by om_context_destroy).
void batch_release(om_context *ctx) {
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    g_tuned.erase(std::remove_if(g_tuned.begin(), g_tuned.end(),
                                 [ctx](const TunedEntry &e) { return e.ctx == ctx; }),
                  g_tuned.end());
  }
  std::vector<CacheEntry> mine;
  {
    std::lock_guard<std::mutex> lk(g_cache_mu);
    for(size_t i = 0; i < g_cache.size();) {
      if(g_cache[i].ctx == ctx) {
        mine.push_back(g_cache[i]);
        g_cache.erase(g_cache.begin() + i);
      } else {
        ++i;
      }
    }
  }
  for(auto &e : mine)
    e.del(e.cls);
}

// Device bytes one request takes in a batch: its FF (and SH) matrices at its
// own size, and its slot's vectors (padded to the class size); 0 for requests
// the batching form does not run.
size_t batch_request_bytes(const om_request &rq) {
  const om_solve_options &o = rq.opts;
  const bool plain = rq.precision == OM_C128 && o.method == OM_SOLVE_GMRES;
  const bool mixed = rq.precision == OM_C64 && o.method == OM_SOLVE_FGMRES_MIXED;
  if((!plain && !mixed) || !rq.spheres || rq.n_spheres < 1 || rq.spheres[0].nmax < 1 ||
     rq.spheres[0].nmax > kMaxNmax)
    return 0;
  const size_t P = pmax(rq.spheres[0].nmax);
  const size_t n = 2 * P * rq.n_spheres, np = rup(2 * P * pad_spheres(rq.n_spheres));
  const size_t elem = mixed ? sizeof(float2) : sizeof(double2);
  const size_t m = (size_t)std::max(1, mixed ? o.inner_iter : o.max_iter);
  const size_t nsm = (np + kBCols - 1) / kBCols;
  // (the precision form's matrices with their fp16 copies and scales)
  const size_t mat = elem * n * n + (mixed ? sizeof(F16c) * n * n + 4 * n * ((n + 255) / 256) : 0);
  return mat * (rq.wave.sh ? 2 : 1) + elem * (m + 1) * np + sizeof(double2) * (3 + nsm) * np +
         sizeof(double2) * (m + 2) * (m + 2) * 2 + (size_t(64) << 20);
}

}  // namespace om

extern "C" int om_batch_tiles(om_context *ctx, int *out, int max_entries) {
  using namespace om;
  if(!ctx || max_entries < 0 || (max_entries > 0 && !out))
    return OM_ERR_INVALID;
  std::lock_guard<std::mutex> lk(g_tuned_mu);
  int k = 0;
  for(const TunedEntry &e : g_tuned) {
    if(e.ctx != ctx)
      continue;
    if(k < max_entries) {
      const MvCfg &c = kMvCands[e.cand];
      int *o = out + 7 * k;
      o[0] = e.precision;
      o[1] = e.nmax;
      o[2] = e.Npad;
      o[3] = c.rows;
      o[4] = c.order;
      o[5] = c.cap;
      o[6] = (int)e.us;
    }
    ++k;
  }
  return k;
}

extern "C" int om_batch_solve(om_context *ctx, const om_request *reqs, int count, size_t arena_bytes,
                              om_result *results) {
  using namespace om;
  if(!ctx || (count > 0 && (!reqs || !results)) || count < 0)
    return OM_ERR_INVALID;
  cudaSetDevice(ctx->device);
  const double t_call = now_ms();
  long launches = 0;
  std::map<ClassKey, std::vector<int>> classes;
  for(int i = 0; i < count; ++i) {
    const om_request &rq = reqs[i];
    om_result &res = results[i];
    res = om_result{};
    res.status = OM_OK;
    const om_solve_options &o = rq.opts;
    const bool plain = rq.precision == OM_C128 && o.method == OM_SOLVE_GMRES;
    const bool mixed = rq.precision == OM_C64 && o.method == OM_SOLVE_FGMRES_MIXED;
    if(!plain && !mixed) {
      res.status = OM_ERR_INVALID;
      continue;
    }
    if(!rq.spheres || rq.n_spheres < 1 || rq.spheres[0].nmax < 1 || rq.spheres[0].nmax > kMaxNmax ||
       o.max_iter < 1 || o.restarts < 1 || (mixed && o.inner_iter < 1)) {
      res.status = OM_ERR_INVALID;
      continue;
    }
    ClassKey k{};
    k.precision = rq.precision;
    k.nmax = rq.spheres[0].nmax;
    k.Npad = pad_spheres(rq.n_spheres);
    k.m = mixed ? o.inner_iter : o.max_iter;
    k.max_cycles = mixed ? std::min(o.max_iter, 32) * o.restarts : o.restarts;
    k.tol = o.tol;
    k.inner_rel = mixed ? o.inner_tol : 0.0;
    k.f16 = mixed && ctx->inner_half ? 1 : 0;
    classes[k].push_back(i);
  }
  bool bad = false;
  for(int i = 0; i < count; ++i)
    bad |= results[i].status == OM_ERR_INVALID;
  if(bad)
    ctx->err = "om_batch_solve runs OM_SOLVE_GMRES on OM_C128 and OM_SOLVE_FGMRES_MIXED on OM_C64 "
               "requests with positive iteration counts and 1 <= nMax <= 15";
  size_t arena = arena_bytes;
  if(!arena) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    arena = std::min<size_t>(fr / 5 * 2, size_t(64) << 30);
    if(ctx->budget)
      arena = std::min(arena, (ctx->budget - std::min(ctx->budget, ctx->used)) / 2);
  }
  int rc = OM_OK;
  for(auto &kv : classes) {
    try {
      if(kv.first.precision == OM_C64)
        rc = run_class<float2, float2>(ctx, kv.first, kv.second, reqs, results, arena, t_call, &launches);
      else
        rc = run_class<double2, double2>(ctx, kv.first, kv.second, reqs, results, arena, t_call,
                                         &launches);
    } catch(std::exception &e) {
      ctx->err = e.what();
      rc = OM_ERR_CUDA;
    }
    if(rc)
      break;
  }
  ctx->last_launches = (int)std::min<long>(launches, 0x7fffffff);
  return rc;
}
