// Block rows of the scattering matrix for a solve sharded over several GPUs.
//
// The reference distributes the matrix by spheres (matvec_parallel,
// PreconditionedMatrix.cpp:989-1054): rank r owns the block rows of spheres
// gran1 .. gran2 - 1, multiplies them with the full vector, and the pieces are
// gathered in rank order and broadcast (MPI_Gatherv + MPI_Bcast, :1044-1051);
// the Krylov recurrence then runs on the full vector on every rank. Here a
// GPU holds the complex128 rows of its spheres (k_assemble in row-block mode)
// and multiplies them with split-K tiles (256 rows x up to 1,024 columns,
// column chunks fixed by the column index alone, so a row's sum does not
// depend on how the rows are split between GPUs) summed in a fixed order.
#include <algorithm>

#include "om_internal.h"
#include "om_krylov.cuh"

namespace om {

namespace {

constexpr int kRowThreads = 256;
constexpr int kRowCols = 1024;

__global__ void __launch_bounds__(kRowThreads) k_matvec_rows(const double2 *S, long m, long n, const double2 *x,
                                                              double2 *part) {
  __shared__ double2 xs[kRowCols];
  const long row_tiles = (m + kRowThreads - 1) / kRowThreads;
  const long ct = blockIdx.x / row_tiles, rt = blockIdx.x - ct * row_tiles;
  const long i = rt * kRowThreads + threadIdx.x;
  const long j0 = ct * kRowCols, j1 = min(n, j0 + kRowCols);
  for(long j = j0 + threadIdx.x; j < j1; j += kRowThreads)
    xs[j - j0] = x[j];
  __syncthreads();
  if(i < m)
    part[ct * m + i] = mv_row<double2, double2>(S + j0 * m + i, m, xs, j0, j1);
}

__global__ void k_rows_reduce(const double2 *part, int nsplit, long m, double2 *y) {
  const long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if(i >= m)
    return;
  double2 acc = part[i];
  for(int s = 1; s < nsplit; ++s) {
    const double2 v = part[(long)s * m + i];
    acc.x += v.x;
    acc.y += v.y;
  }
  y[i] = acc;
}

}  // namespace

}  // namespace om

using namespace om;

extern "C" {

int om_assemble_rows(om_problem *pr, int harmonic, int sphere0, int sphere1) {
  if(!pr || (harmonic != OM_FF && harmonic != OM_SH) || sphere0 < 0 || sphere1 <= sphere0 || sphere1 > pr->N)
    return OM_ERR_INVALID;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  const size_t bytes = sizeof(double2) * (size_t)(2L * pr->P * (sphere1 - sphere0)) * (size_t)pr->n;
  if(pr->d_Srows && pr->rows_bytes != bytes) {
    dev_release(ctx, pr->d_Srows, pr->rows_bytes);
    pr->d_Srows = nullptr;
    pr->rows_bytes = 0;
  }
  if(!pr->d_Srows) {
    const int rc = dev_malloc(ctx, &pr->d_Srows, bytes);
    if(rc)
      return rc;
    pr->rows_bytes = bytes;
  }
  try {
    launch_assemble_rows(pr, harmonic, sphere0, sphere1, (double2 *)pr->d_Srows);
  } catch(std::exception &e) {
    ctx->err = e.what();
    return OM_ERR_CUDA;
  }
  const cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess) {
    ctx->err = cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  pr->rows0 = sphere0;
  pr->rows1 = sphere1;
  pr->rows_harmonic = harmonic;
  return OM_OK;
}

int om_matvec_rows(om_problem *pr, int harmonic, const double *x, double *y) {
  if(!pr || !x || !y)
    return OM_ERR_INVALID;
  if(!pr->d_Srows || pr->rows_harmonic != harmonic)
    return OM_ERR_STATE;
  om_context *ctx = pr->ctx;
  cudaSetDevice(ctx->device);
  ctx->last_launches = 0;
  const long m = 2L * pr->P * (pr->rows1 - pr->rows0), n = pr->n;
  const int nsplit = (int)((n + kRowCols - 1) / kRowCols);
  void *part = nullptr;
  int rc = dev_malloc(ctx, &part, sizeof(double2) * (size_t)m * nsplit);
  if(rc)
    return rc;
  const long row_tiles = (m + kRowThreads - 1) / kRowThreads;
  k_matvec_rows<<<(unsigned)(row_tiles * nsplit), kRowThreads, 0, ctx->stream>>>(
      (const double2 *)pr->d_Srows, m, n, (const double2 *)x, (double2 *)part);
  k_rows_reduce<<<blocks_for(m, 256), 256, 0, ctx->stream>>>((const double2 *)part, nsplit, m, (double2 *)y);
  ctx->last_launches += 2;
  dev_release(ctx, part, sizeof(double2) * (size_t)m * nsplit);
  const cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if(e != cudaSuccess) {
    ctx->err = cudaGetErrorString(e);
    return OM_ERR_CUDA;
  }
  return OM_OK;
}

}  // extern "C"
