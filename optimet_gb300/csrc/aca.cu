// ACA-compressed scattering matrix (the reference's ACA_compression role,
// PreconditionedMatrix.cpp:402-551 and 760-890) and its matrix-vector product
// (matvec, PreconditionedMatrix.cpp:1056-1085).
//
// Off-diagonal blocks S_ij with |r_i - r_j| >= 2 (a_i + a_j) are replaced by
// a partially pivoted adaptive cross approximation U V (eps 1e-3, first row 0,
// the reference's pivot rules and running norm estimate); the others stay
// dense; diagonal blocks are the identity. The blocks are assembled in batches
// of sphere pairs into scratch (the assembly kernel's pair mode), compressed
// by one CTA per block, and packed into one store through an atomic bump
// offset; per ordered block (i, j) the store offset and the rank (-1 dense,
// -2 identity) are recorded. The matvec walks each block row in a fixed order,
// so results do not depend on where the blocks landed in the store.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "om_internal.h"

namespace om {

namespace {

constexpr int kAcaThreads = 256;

__device__ __forceinline__ zd ld2(const double2 *p, size_t i) {
  const double2 v = p[i];
  return mk(v.x, v.y);
}
__device__ __forceinline__ void st2(double2 *p, size_t i, zd v) { p[i] = make_double2(v.re, v.im); }

// getMaxInd: first index of the strict maximum of |v| among the candidates
// (flag 0); the first candidate when all are 0. Block-wide, result in *out.
__device__ void block_argmax(const zd *v, const unsigned char *taken, int kmax, double *rv, int *ri,
                             int *out) {
  double best = -1.0;
  int bi = 0x7fffffff;
  for(int c = threadIdx.x; c < kmax; c += blockDim.x) {
    if(taken[c])
      continue;
    const double a = hypot(v[c].re, v[c].im);
    if(a > best) {  // increasing c per thread: keeps the first maximum
      best = a;
      bi = c;
    }
  }
  rv[threadIdx.x] = best;
  ri[threadIdx.x] = bi;
  __syncthreads();
  for(int s = blockDim.x / 2; s > 0; s >>= 1) {
    if(threadIdx.x < s) {
      const double a = rv[threadIdx.x + s];
      const int ia = ri[threadIdx.x + s];
      if(a > rv[threadIdx.x] || (a == rv[threadIdx.x] && ia < ri[threadIdx.x])) {
        rv[threadIdx.x] = a;
        ri[threadIdx.x] = ia;
      }
    }
    __syncthreads();
  }
  if(threadIdx.x == 0)
    *out = ri[0];
  __syncthreads();
}

__device__ double block_sum(double v, double *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for(int s = blockDim.x / 2; s > 0; s >>= 1) {
    if(threadIdx.x < s)
      red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  const double r = red[0];
  __syncthreads();
  return r;
}

struct AcaBuildArgs {
  const double2 *blocks;  // 2 count blocks of kmax x kmax (pair mode of the assembly)
  long pair0;
  int count, N, kmax;
  const double *cart, *radius;
  double2 *Uws, *Vws;     // per block kmax x kmax workspace
  double2 *store;
  unsigned long long cap;
  unsigned long long *bump;
  long long *off;
  int *rank;
  int *overflow;
};

// One CTA per block of the batch: ACA_compression (PreconditionedMatrix.cpp:760-867)
// for admissible blocks, a dense copy for the others.
__global__ void __launch_bounds__(kAcaThreads) k_aca_blocks(AcaBuildArgs a) {
  extern __shared__ double asm_[];
  const int kmax = a.kmax;
  zd *row = reinterpret_cast<zd *>(asm_);
  zd *col = row + kmax;
  double *rv = reinterpret_cast<double *>(col + kmax);
  int *ri = reinterpret_cast<int *>(rv + kAcaThreads);
  unsigned char *Iset = reinterpret_cast<unsigned char *>(ri + kAcaThreads);
  unsigned char *Jset = Iset + kmax;
  __shared__ int s_ik, s_jk, s_stop, s_rank, s_adm;
  __shared__ unsigned long long s_off;

  const int b = blockIdx.x;
  const long pair = a.pair0 + b / 2;
  int j = (int)((1.0 + sqrt(1.0 + 8.0 * (double)pair)) * 0.5);
  while((long)j * (j - 1) / 2 > pair)
    --j;
  while((long)(j + 1) * j / 2 <= pair)
    ++j;
  int i = (int)(pair - (long)j * (j - 1) / 2);
  if(b & 1) {  // the second block of the pair is S_ji
    const int t = i;
    i = j;
    j = t;
  }
  const size_t kk = (size_t)kmax * kmax;
  const double2 *M = a.blocks + (size_t)b * kk;
  double2 *U = a.Uws + (size_t)b * kk, *V = a.Vws + (size_t)b * kk;
  if(threadIdx.x == 0) {
    // Tools::findDistance on the Cartesian centres
    const double dx = a.cart[3 * j] - a.cart[3 * i], dy = a.cart[3 * j + 1] - a.cart[3 * i + 1],
                 dz = a.cart[3 * j + 2] - a.cart[3 * i + 2];
    const double d = sqrt(dx * dx + dy * dy + dz * dz);
    s_adm = d >= 2.0 * (a.radius[i] + a.radius[j]);
  }
  for(int c = threadIdx.x; c < kmax; c += blockDim.x)
    Iset[c] = Jset[c] = 0;
  __syncthreads();
  const size_t slot = (size_t)i * a.N + j;
  if(!s_adm) {
    if(threadIdx.x == 0) {
      s_off = atomicAdd(a.bump, (unsigned long long)kk);
      if(s_off + kk > a.cap) {
        atomicExch(a.overflow, 1);
        a.rank[slot] = -3;
      } else {
        a.rank[slot] = -1;
        a.off[slot] = (long long)s_off;
      }
    }
    __syncthreads();
    if(s_off + kk <= a.cap)
      for(size_t e = threadIdx.x; e < kk; e += blockDim.x)
        a.store[s_off + e] = M[e];
    return;
  }
  const double eps = 1e-3;
  double norma = 0.0;
  if(threadIdx.x == 0) {
    s_ik = 0;
    s_stop = 0;
    s_rank = kmax;
    Iset[0] = 1;
  }
  __syncthreads();
  for(int k = 0; k < kmax; ++k) {
    const int ik = s_ik;
    for(int c = threadIdx.x; c < kmax; c += blockDim.x) {
      zd v = ld2(M, (size_t)c * kmax + ik);
      if(k > 0) {
        zd sum = mk(0.0, 0.0);
        for(int p = 0; p <= k - 1; ++p)
          sum = sum + ld2(U, (size_t)p * kmax + ik) * ld2(V, (size_t)p * kmax + c);
        v = v - sum;
      }
      row[c] = v;
    }
    __syncthreads();
    block_argmax(row, Jset, kmax, rv, ri, &s_jk);
    const int jk = s_jk;
    const zd piv = row[jk];
    for(int c = threadIdx.x; c < kmax; c += blockDim.x)
      st2(V, (size_t)k * kmax + c, row[c] / piv);
    if(threadIdx.x == 0)
      Jset[jk] = 1;
    __syncthreads();
    for(int r = threadIdx.x; r < kmax; r += blockDim.x) {
      zd v = ld2(M, (size_t)jk * kmax + r);
      if(k > 0) {
        zd sum = mk(0.0, 0.0);
        for(int p = 0; p <= k - 1; ++p)
          sum = sum + ld2(V, (size_t)p * kmax + jk) * ld2(U, (size_t)p * kmax + r);
        v = v - sum;
      }
      col[r] = v;
      st2(U, (size_t)k * kmax + r, v);
    }
    __syncthreads();
    double cp = 0.0, rp = 0.0;
    for(int r = threadIdx.x; r < kmax; r += blockDim.x) {
      cp += norm2(col[r]);
      rp += norm2(ld2(V, (size_t)k * kmax + r));
    }
    const double cn = sqrt(block_sum(cp, rv)), rn = sqrt(block_sum(rp, rv));
    if(k == 0) {
      norma = (cn * cn) * (rn * rn);
    } else {
      // the reference's cross terms: p = 0 .. k - 2, dot products over the
      // first k entries, no conjugation
      double cross = 0.0;
      for(int p = threadIdx.x; p < k - 1; p += blockDim.x) {
        zd pom1 = mk(0.0, 0.0), pom2 = mk(0.0, 0.0);
        for(int tt = 0; tt < k; ++tt) {
          pom1 = pom1 + ld2(U, (size_t)p * kmax + tt) * ld2(U, (size_t)k * kmax + tt);
          pom2 = pom2 + ld2(V, (size_t)p * kmax + tt) * ld2(V, (size_t)k * kmax + tt);
        }
        cross += cabs(pom1) * cabs(pom2);
      }
      cross = block_sum(cross, rv);
      norma = norma + (cn * cn) * (rn * rn) + 2.0 * cross;
      if(eps * sqrt(norma) >= cn * rn) {
        if(threadIdx.x == 0) {
          s_rank = k + 1;
          s_stop = 1;
        }
      }
    }
    __syncthreads();
    if(s_stop)
      break;
    block_argmax(col, Iset, kmax, rv, ri, &s_ik);
    if(threadIdx.x == 0)
      Iset[s_ik] = 1;
    __syncthreads();
  }
  const int r = s_rank;
  const size_t sz = 2 * (size_t)kmax * r;
  if(threadIdx.x == 0) {
    s_off = atomicAdd(a.bump, (unsigned long long)sz);
    if(s_off + sz > a.cap) {
      atomicExch(a.overflow, 1);
      a.rank[slot] = -3;
    } else {
      a.rank[slot] = r;
      a.off[slot] = (long long)s_off;
    }
  }
  __syncthreads();
  if(s_off + sz > a.cap)
    return;
  // U (kmax x r, column-major) then V (r rows of kmax)
  for(size_t e = threadIdx.x; e < 2 * (size_t)kmax * r; e += blockDim.x)
    a.store[s_off + e] = e < (size_t)kmax * r ? U[e] : V[e - (size_t)kmax * r];
}

// y_i = sum_j S_ij x_j (or b_i - that sum), one CTA per block row, blocks in
// column order: identity, dense 2P x 2P, or U (V x_j) with V x_j formed by
// one warp per row of V.
__global__ void __launch_bounds__(kAcaThreads) k_aca_matvec(AcaOp op, const double2 *x,
                                                           const double2 *b, double2 *y) {
  extern __shared__ double msm[];
  const int kmax = op.kmax, i = blockIdx.x;
  zd *xs = reinterpret_cast<zd *>(msm);
  zd *ts = xs + kmax;
  zd acc[2] = {mk(0.0, 0.0), mk(0.0, 0.0)};  // rows threadIdx.x, threadIdx.x + 256
  for(int j = 0; j < op.N; ++j) {
    for(int c = threadIdx.x; c < kmax; c += blockDim.x)
      xs[c] = ld2(x, (size_t)j * kmax + c);
    const size_t slot = (size_t)i * op.N + j;
    const int r = op.rank[slot];
    __syncthreads();
    if(r == -2) {
      for(int u = 0; u < 2; ++u) {
        const int row = threadIdx.x + u * blockDim.x;
        if(row < kmax)
          acc[u] = acc[u] + xs[row];
      }
    } else if(r == -1) {
      const double2 *S = op.store + op.off[slot];
      for(int u = 0; u < 2; ++u) {
        const int row = threadIdx.x + u * blockDim.x;
        if(row >= kmax)
          continue;
        zd s = mk(0.0, 0.0);
        for(int c = 0; c < kmax; ++c)
          s = s + ld2(S, (size_t)c * kmax + row) * xs[c];
        acc[u] = acc[u] + s;
      }
    } else if(r > 0) {
      const double2 *U = op.store + op.off[slot];
      const double2 *V = U + (size_t)kmax * r;  // r rows of kmax
      // t = V x_j: one warp per row of V, lanes along the row, fixed-order
      // shuffle reduction
      const int nw = blockDim.x >> 5, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
      for(int q = w; q < r; q += nw) {
        zd s = mk(0.0, 0.0);
        for(int c = lane; c < kmax; c += 32)
          s = s + ld2(V, (size_t)q * kmax + c) * xs[c];
        for(int o = 16; o > 0; o >>= 1) {
          s.re += __shfl_down_sync(0xffffffffu, s.re, o);
          s.im += __shfl_down_sync(0xffffffffu, s.im, o);
        }
        if(lane == 0)
          ts[q] = s;
      }
      __syncthreads();
      for(int u = 0; u < 2; ++u) {
        const int row = threadIdx.x + u * blockDim.x;
        if(row >= kmax)
          continue;
        zd s = mk(0.0, 0.0);
        for(int q = 0; q < r; ++q)
          s = s + ld2(U, (size_t)q * kmax + row) * ts[q];
        acc[u] = acc[u] + s;
      }
    }
    __syncthreads();
  }
  for(int u = 0; u < 2; ++u) {
    const int row = threadIdx.x + u * blockDim.x;
    if(row >= kmax)
      continue;
    const size_t e = (size_t)i * kmax + row;
    zd v = acc[u];
    if(b)
      v = ld2(b, e) - v;
    st2(y, e, v);
  }
}

__global__ void k_aca_init(int *rank, int N) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(t < (long)N * N)
    rank[t] = (t / N == t % N) ? -2 : -3;
}

}  // namespace

void aca_matvec(om_context *ctx, const AcaOp &op, const double2 *x, double2 *y, const double2 *b) {
  const size_t smem = 2 * (size_t)op.kmax * sizeof(zd);
  k_aca_matvec<<<op.N, kAcaThreads, smem, ctx->stream>>>(op, x, b, y);
  ctx->last_launches++;
}

// Builds the compressed operator of one harmonic; grows the store and starts
// again when the packed blocks do not fit.
int aca_build(om_problem *pr, int harmonic) {
  om_context *ctx = pr->ctx;
  AcaData &A = pr->aca[harmonic];
  const int N = pr->N, kmax = 2 * pr->P;
  const long npairs = (long)N * (N - 1) / 2;
  const size_t kk = (size_t)kmax * kmax;
  if(!A.rank) {
    int rc = dev_malloc(ctx, (void **)&A.rank, sizeof(int) * (size_t)N * N);
    if(!rc) rc = dev_malloc(ctx, (void **)&A.off, sizeof(long long) * (size_t)N * N);
    if(!rc) rc = dev_malloc(ctx, (void **)&A.ctl, 256);
    if(rc)
      return rc;
  }
  // batch of pairs: two dense blocks + U and V workspace per block
  const size_t per_pair = 2 * 3 * kk * sizeof(double2);
  const long batch = std::max(1L, std::min(npairs, (long)std::max<size_t>(1, ((size_t)1 << 31) / per_pair)));
  void *ws = nullptr;
  int rc = npairs ? dev_malloc(ctx, &ws, per_pair * batch) : OM_OK;
  if(rc)
    return rc;
  double2 *blocks = (double2 *)ws, *Uws = blocks + 2 * kk * batch, *Vws = Uws + 2 * kk * batch;
  if(!A.cap)
    A.cap = std::max<size_t>(kk, (size_t)N * N * 2 * kmax * 24);
  const size_t smem = 2 * (size_t)kmax * sizeof(zd) + kAcaThreads * (sizeof(double) + sizeof(int)) +
                      2 * (size_t)kmax + 16;
  for(int attempt = 0; attempt < 8; ++attempt) {
    if(!A.store) {
      rc = dev_malloc(ctx, (void **)&A.store, A.cap * sizeof(double2));
      if(rc)
        break;
    }
    cudaMemsetAsync(A.ctl, 0, 256, ctx->stream);
    k_aca_init<<<blocks_for((long)N * N, 256), 256, 0, ctx->stream>>>(A.rank, N);
    ctx->last_launches++;
    for(long p0 = 0; p0 < npairs; p0 += batch) {
      const int cnt = (int)std::min(batch, npairs - p0);
      launch_assemble_pairs(pr, harmonic, p0, cnt, blocks);
      AcaBuildArgs a;
      a.blocks = blocks;
      a.pair0 = p0;
      a.count = cnt;
      a.N = N;
      a.kmax = kmax;
      a.cart = pr->d_cart;
      a.radius = pr->d_radius;
      a.Uws = Uws;
      a.Vws = Vws;
      a.store = A.store;
      a.cap = A.cap;
      a.bump = (unsigned long long *)A.ctl;
      a.off = A.off;
      a.rank = A.rank;
      a.overflow = (int *)(A.ctl + 8);
      cudaFuncSetAttribute(k_aca_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      k_aca_blocks<<<2 * cnt, kAcaThreads, smem, ctx->stream>>>(a);
      ctx->last_launches++;
    }
    unsigned long long ctl[2] = {0, 0};
    cudaMemcpyAsync(ctl, A.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if(e != cudaSuccess) {
      ctx->err = std::string("ACA build: ") + cudaGetErrorString(e);
      rc = OM_ERR_CUDA;
      break;
    }
    if(!(int)ctl[1]) {
      A.used = ctl[0];
      break;
    }
    dev_release(ctx, A.store, A.cap * sizeof(double2));
    A.store = nullptr;
    A.cap = std::max<size_t>(2 * A.cap, ctl[0]);
  }
  if(ws)
    dev_release(ctx, ws, per_pair * batch);
  if(!rc && !A.used && npairs) {
    ctx->err = "ACA store could not be sized";
    rc = OM_ERR_BUDGET;
  }
  return rc;
}

void aca_free(om_problem *pr) {
  for(auto &A : pr->aca) {
    const size_t NN = (size_t)pr->N * pr->N;
    dev_release(pr->ctx, A.rank, sizeof(int) * NN);
    dev_release(pr->ctx, A.off, sizeof(long long) * NN);
    dev_release(pr->ctx, A.ctl, 256);
    dev_release(pr->ctx, A.store, A.cap * sizeof(double2));
    A = AcaData();
  }
}

AcaOp aca_op(const om_problem *pr, int harmonic) {
  AcaOp op;
  op.N = pr->N;
  op.kmax = 2 * pr->P;
  op.off = pr->aca[harmonic].off;
  op.rank = pr->aca[harmonic].rank;
  op.store = pr->aca[harmonic].store;
  return op;
}

}  // namespace om
