/*
 * liboptimet_gpu: GB300 (sm_103a) implementation of OPTIMET-3D's multiple-
 * scattering T-matrix hot path for clusters of spheres, behind a C ABI.
 *
 * Plain pointers and sizes only. Complex numbers are interleaved (re, im)
 * doubles; vectors follow OPTIMET's layout: per sphere a TE block of P
 * harmonics then a TM block, P = nMax (nMax + 2), harmonic p = n(n+1) - m - 1;
 * matrices are column-major. Lengths are metres, angles radians.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the OPTIMET-3D source tree).
 */
#ifndef OPTIMET_GPU_H
#define OPTIMET_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference throws std::runtime_error in these cases. */
#define OM_OK 0
#define OM_ERR_INVALID 1          /* bad argument (null, size, mixed nMax: PreconditionedMatrix.cpp:1161-1165) */
#define OM_ERR_OVERLAP 2          /* overlapping spheres (Geometry.cpp:39-51) */
#define OM_ERR_CUDA 3             /* CUDA runtime failure */
#define OM_ERR_BUDGET 4           /* device-memory budget of the context exceeded */
#define OM_ERR_NOT_CONVERGED 5    /* iterative solve stopped above tolerance */
#define OM_ERR_SINGULAR 6         /* zero pivot in the LU factorisation (ScalapackSolver.cpp:76-77) */
#define OM_ERR_STATE 7            /* call out of order (e.g. solve before assemble) */
#define OM_PENDING 8              /* om_server_poll: the request has not finished yet */

/* Harmonic selector */
#define OM_FF 0                   /* fundamental frequency */
#define OM_SH 1                   /* second harmonic (2 omega, eps_SH) */

/* Storage precision of the scattering matrix */
#define OM_C128 0                 /* complex FP64 */
#define OM_C64 1                  /* complex FP32 (precision form) */
#define OM_ACA 2                  /* complex FP64, admissible blocks ACA-compressed (GMRES only):
                                     Scattering_matrix_ACA_FF/_SH + ACA_compression,
                                     PreconditionedMatrix.cpp:402-551,760-890 */

/* Solve methods (Solver roles of the reference) */
#define OM_SOLVE_LU 0             /* dense LU, partial pivoting: ScalapackSolver pzgesv role */
#define OM_SOLVE_GMRES 1          /* restarted GMRES: MatrixBelosSolver / Gmres_Zcomp role */
#define OM_SOLVE_FGMRES_MIXED 2   /* FP64 outer FGMRES around FP32 inner GMRES on the C64 matrix */
#define OM_SOLVE_LU_MIXED 3       /* FP32 LU + FP64 iterative refinement (GMRES-IR: GMRES on the system
                                     left-preconditioned by the LU, FP64-accurate residuals) */

typedef struct om_context om_context;
typedef struct om_problem om_problem;

typedef struct {
  double x, y, z;        /* centre (XML <cartesian> times 1e-9) */
  double radius;         /* <properties radius> times 1e-9 */
  double eps_r[2];       /* relative permittivity at the fundamental */
  double mu_r[2];        /* relative permeability */
  double eps_r_sh[2];    /* relative permittivity at the second harmonic (<epsilon_SH>) */
  double ksippp[2];      /* surface chi(2), perp-perp-perp (<ksippp>) */
  double ksiparppar[2];  /* surface chi(2), par-perp-par (<ksiparppar>) */
  double gamma[2];       /* bulk chi(2) (<gamma>) */
  int nmax;              /* <harmonics nmax>; equal for all spheres */
  int reserved;
} om_sphere;

typedef struct {
  double eps_r[2];       /* background relative permittivity (<background>) */
  double mu_r[2];
} om_medium;

typedef struct {
  double wavelength;     /* <wavelength value> times 1e-9 */
  double theta, phi;     /* <propagation>, radians */
  double e_theta[2];     /* <polarization Etheta> */
  double e_phi[2];       /* <polarization Ephi> */
  int sh;                /* <SHsources condition="yes"> */
  int reserved;
} om_plane_wave;

typedef struct {
  int method;            /* OM_SOLVE_* */
  int max_iter;          /* Krylov dimension per restart cycle */
  int restarts;          /* restart cycles */
  int inner_iter;        /* inner FP32 GMRES iterations per outer step (mixed) */
  double tol;            /* relative residual ||b - S x|| / ||b|| */
  double inner_tol;      /* inner relative tolerance (mixed) */
} om_solve_options;

typedef struct {
  int iterations;        /* Krylov iterations; OM_SOLVE_FGMRES_MIXED: outer FGMRES steps;
                            OM_SOLVE_LU_MIXED: refinement steps */
  int inner_iterations;  /* OM_SOLVE_FGMRES_MIXED: inner FP32 GMRES iterations;
                            OM_SOLVE_LU_MIXED: GMRES iterations on the LU-preconditioned system */
  double rel_residual;   /* final FP64 relative residual */
  double seconds;        /* device time of the solve */
} om_solve_stats;

/* Device context: one GPU, one stream, a device-memory budget (0 = no limit).
 * Replaces the process-level state of mpi::init / scalapack::Context
 * (srcAna/mpi/Session.cpp:38-64, srcAna/scalapack/Context.h:32-169). */
int om_context_create(int device, size_t budget_bytes, om_context **out);
/* Also destroys the problems of the context that are still alive. */
void om_context_destroy(om_context *ctx);
const char *om_context_last_error(const om_context *ctx);
/* Number of kernels the last call on this context launched. */
int om_context_last_launches(const om_context *ctx);
/* Wait for all work queued on the context's stream (calls are asynchronous
 * with respect to the host unless they return data). */
int om_context_synchronize(om_context *ctx);
/* Kernel timers (CUDA events on the context's stream; no counterpart in the
 * reference, which has no profiling). Writes the totals accumulated since the
 * previous call to out[8] = {assembly ms, assembly launches, complex128 matvec
 * ms, launches, complex64 x complex64 matvec ms, launches, complex64 x
 * complex128 (compensated) matvec ms, launches} (out may be NULL), resets
 * them and switches timing on or off. */
int om_context_timers(om_context *ctx, int enable, double *out);
/* Timers of the inner FP32 GMRES products of OM_SOLVE_FGMRES_MIXED on the
 * bf16 copy (recorded while om_context_timers has switched timing on):
 * out[4] = {products on the bf16 copy ms, launches, complex64 products that
 * write the copy ms, launches}; resets them. */
int om_context_inner_timers(om_context *ctx, double *out);
/* LU phase timers, recorded while om_context_timers has switched timing on:
 * out[8] = {factorization ms, factorizations, panel ms, panels, trailing-
 * update ms, trailing updates, triangular-solve ms, solves (one forward and
 * one backward sweep each)} accumulated since the previous call (out may be
 * NULL); resets them. */
int om_context_lu_timers(om_context *ctx, double *out);
/* Launch tuning of a context (no counterpart in the reference). Fields below
 * zero keep the current value.
 *   matvec_ctas_per_sm / matvec_df_ctas_per_sm: grid caps of the complex64 /
 *     complex128 matvec and of the compensated complex64 x complex128 one, in
 *     CTAs per SM (defaults 8 and 8; servers with several slots start at 4
 *     and 2); the CTAs take tiles from a counter, so lower caps leave room on
 *     each SM for another context's work.
 *   assemble_carveout / matvec_carveout: preferred shared-memory carveout of
 *     the assembly and matvec kernels in percent (0-100; default: the
 *     driver's choice). The setting is per kernel for the whole process. */
typedef struct {
  int matvec_ctas_per_sm;
  int matvec_df_ctas_per_sm;
  int assemble_carveout;
  int matvec_carveout;
  int lu_tensor_cores;   /* complex64 LU updates on the tensor cores: 3 (default) the persistent
                            kernel (one CTA per SM) for the rank-256 trailing updates and one CTA
                            per 128 x 64 tile for the rank-32 in-block and U12 updates, 1 the
                            persistent kernel for all, 2 one CTA per tile for all (the same bits
                            in all three), 0 off */
  int matvec_tma;        /* complex64 x complex64 matvec with TMA-staged matrix tiles: 1 (default for
                            a context) / 0 (default for the slots of a server with several slots) */
  int assemble_rotation; /* complex64 assembly by rotated z-axis translations (one recurrence
                            chain per pair, FP32 rotation products): 1 (default) / 0 (the general
                            translation's 3 nMax + 1 chains per pair, FP32 block forming) */
  int lu_persistent;     /* LU kernels: 1 (default) one cooperative launch per panel of 8,192
                            rows or more (a grid-wide barrier per column) and one launch per
                            triangular sweep (solved blocks published through flags); 2 a pivot
                            launch and an update launch per panel column, one launch per
                            32-row block of a triangular sweep; 3 as 1 with the panel's rows
                            kept in global memory rather than shared memory */
  int batch_tiles;       /* tiles and schedule of the batched matvecs (om_batch_solve): 0 (default)
                            autotuned per size class at its first batch, 1..8 a fixed candidate
                            (rows per tile, tile order, CTAs per SM; see om_batch_tiles) */
  int batch_fused;       /* batched solves of the small size classes in one cooperative launch
                            per solve that runs every slot's cycles to the end (a group of one
                            CTA per 512 rows for each slot): 1 (default) for the classes of at
                            most 1,024 padded unknowns, 2 for those of at most 4,096, 0 never
                            (the lockstep Arnoldi steps of all slots as captured graphs); the
                            same bits either way */
  int inner_half;        /* the inner FP32 products of the precision form read a 4-byte copy of the
                            complex64 matrix when 1 (default), the complex64 matrix itself when 0;
                            the FP64 residuals always use the complex64 matrix. OM_SOLVE_FGMRES_MIXED:
                            a bf16 copy, written by the first inner product while it reads the
                            complex64 matrix. om_batch_solve (GMRES-based refinement): an fp16 copy
                            with a power-of-two scale per 256-row block and column, written by one
                            launch after the batch's assembly */
} om_tuning;
int om_context_tune(om_context *ctx, const om_tuning *t);
/* C (m x n) -= A (m x k) B (k x n), complex64 interleaved, column-major, any
 * k >= 1, host buffers: the tensor-core trailing update of the complex64 LU.
 * A's rows and B's columns are scaled by powers of two and split into fp16
 * hi / lo parts once; the products hi hi + hi lo + lo hi accumulate in FP32
 * over all of k (about 21 significant bits relative to the rows' and
 * columns' magnitudes). The role of the trailing pzgemm of pzgesv
 * (ScalapackSolver.cpp:54-130). */
/* y = S x, complex64 interleaved (S column-major n x n, host buffers), by the
 * inner FP32 GMRES product of OM_SOLVE_FGMRES_MIXED repeated `products`
 * times: the first on the complex64 matrix (writing its bf16 copy when the
 * context's inner_half tuning is on), the later ones on the copy; y is the
 * last product. The role of the FP32 matvecs inside the reference's GMRES
 * iterations (PreconditionedMatrix.cpp:892-1133). */
int om_matvec_inner_c64(om_context *ctx, long n, const float *S, const float *x, float *y, int products);
int om_cgemm_sub_c64(om_context *ctx, long m, long n, int k, const float *A, long lda,
                     const float *B, long ldb, float *C, long ldc);
/* Statistics of an ACA-compressed matrix (om_assemble with OM_ACA): device
 * bytes of the packed blocks, number of compressed / dense off-diagonal blocks,
 * mean and largest rank (the reference prints the compressed size in MB,
 * PreconditionedMatrix.cpp:548). */
int om_aca_info(om_problem *pr, int harmonic, double *store_bytes, int *compressed, int *dense,
                double *mean_rank, int *max_rank);
/* Record an event on the context's stream, wait for it and return in *ms the
 * device time since the previous mark (0 for the first). Device-side step
 * timing for benchmarks; no counterpart in the reference. */
int om_context_mark(om_context *ctx, double *ms);

/* Geometry + Excitation for one cluster at one wavelength. Mirrors
 * simulation_input (Reader.cpp:55-101,585-663,782-834): spheres are stored in
 * spherical coordinates, overlap is rejected, the plane wave is expanded
 * (Excitation::populate, Excitation.cpp:48-75). */
int om_problem_create(om_context *ctx, const om_sphere *spheres, int n_spheres,
                      const om_medium *background, const om_plane_wave *wave,
                      om_problem **out);
void om_problem_destroy(om_problem *pr);
/* Excitation::updateWavelength (Excitation.cpp:132-137) + Geometry::update. */
int om_problem_set_wavelength(om_problem *pr, double wavelength);
/* The whole plane wave at once (wavelength, direction, polarisation, SH flag):
 * Excitation::populate (Excitation.cpp:48-75) for a new excitation of the same
 * geometry; device buffers, including an assembled matrix's storage, are kept. */
int om_problem_set_wave(om_problem *pr, const om_plane_wave *wave);
/* Number of unknowns 2 P N (AbstractSolver::scattering_size, Solver.h:118-121). */
long om_problem_size(const om_problem *pr);

/* Coupling(relR, waveK, nMax, regular) (Coupling.h:29-41, Coupling.cpp:80-87):
 * A ("diagonal") and B ("offdiagonal"), P x P column-major, for `count`
 * displacements rel_xyz[3*count] (Cartesian, metres). `regular` keeps the
 * reference's inverted meaning: 1 -> Hankel (irregular), 0 -> Bessel. */
int om_coupling(om_context *ctx, const double *rel_xyz, int count, double k_re, double k_im,
                int nmax, int regular, double *A, double *B);

/* Diagonal T-matrices, N x 2P (Scatterer::getTLocal / getTLocalSH,
 * Scatterer.cpp:39-161). */
int om_tmatrix(om_problem *pr, int harmonic, double *T);
/* Plane-wave coefficients [a_p | b_p], 2P (Excitation::dataIncAp/Bp). */
int om_incident_coefficients(om_problem *pr, double *ab);

/* preconditioned_scattering_matrix[SH] (PreconditionedMatrix.cpp:350-400,555-610,
 * 1137-1184): S_ii = I, S_ij = -T_i [A^T B^T; B^T A^T](r_i - r_j), kept on the
 * device in the requested precision. */
int om_assemble(om_problem *pr, int harmonic, int precision);
/* Copy the assembled matrix to the host (complex128, column-major n x n). */
int om_copy_matrix(om_problem *pr, int harmonic, double *S);
/* source_vector (PreconditionedMatrix.cpp:1327-1345): Q_i = T_i IncLocal_i.
 * Q may be NULL (kept on the device). */
int om_source_vector(om_problem *pr, double *Q);
/* AbstractSolver::solve for the fundamental (PreconditionedMatrixSolver.h:45-79,
 * ScalapackSolver.cpp:54-130, MatrixBelosSolver.cpp:26-104), followed by
 * convertInternal (Solver.cpp:57-77). */
int om_solve(om_problem *pr, const om_solve_options *opts, om_solve_stats *stats);
/* Solve S x = b for a caller-supplied right-hand side with the assembled matrix. */
int om_solve_rhs(om_problem *pr, int harmonic, const om_solve_options *opts, const double *b,
                 double *x, om_solve_stats *stats);
/* The solve of om_solve_rhs (OM_SOLVE_GMRES only) without any device-memory
 * allocation. No counterpart in the reference. For callers that cannot call
 * cudaMalloc/cudaFree while they solve -- a serving loop that has given all of
 * HBM to resident matrices and its own arena, or latency-critical host code
 * that must not let an allocation synchronise the device. b and x are host
 * buffers of n complex values, as for om_solve_rhs.
 *   Limit: every device buffer of the solve (b, x, the Krylov basis of
 *   max_iter + 1 vectors, split-K partial sums) lives in one fixed 64 MiB
 *   array that each GPU loading the library holds until the process exits;
 *   a request that does not fit returns OM_ERR_INVALID with the bytes it needs.
 *   The first call on a device looks up that array's device address; make it
 *   before any stream capture on that device.
 *   All calls share the array and it keeps the previous call's contents (the
 *   solution vector is cleared at the start of every call); calls that overlap
 *   on the GPU, from any context on the same device, race.
 *   stats->seconds is the host wall-clock time of the call, copies included. */
int om_solve_rhs_noalloc(om_problem *pr, int harmonic, const om_solve_options *opts,
                         const double *b, double *x, om_solve_stats *stats);
/* Block rows of S for a solve sharded over several GPUs: the rows of spheres
 * sphere0 .. sphere1 - 1 (complex128, 2P (sphere1 - sphere0) x n, kept on the
 * device in place of a previous row block). The role of one MPI rank's rows
 * in the reference's distributed product (matvec_parallel,
 * PreconditionedMatrix.cpp:989-1054, rank r owning spheres gran1 .. gran2 - 1,
 * :1001-1007). Synchronous. */
int om_assemble_rows(om_problem *pr, int harmonic, int sphere0, int sphere1);
/* y = S_rows x for the row block of om_assemble_rows: x is n complex128 values
 * and y 2P (sphere1 - sphere0) values, both in DEVICE memory of the context's
 * GPU (e.g. tensors of the framework that runs the collective). The partial
 * product one rank contributes before the all-gather of the full vector
 * (MPI_Gatherv + MPI_Bcast, PreconditionedMatrix.cpp:1044-1051). Each row's sum
 * is formed in an order that does not depend on the row split. Synchronous. */
int om_matvec_rows(om_problem *pr, int harmonic, const double *x, double *y);
/* Scattered and internal coefficients (n each; either may be NULL). */
int om_get_coefficients(om_problem *pr, double *X_sca, double *X_int);
/* Result::getExtinctionCrossSection, getScatteringCrossSection,
 * getAbsorptionCrossSection (Result.cpp:541-631):
 * out = {C_ext, C_sca, C_ext - C_sca (the scan's absorption column,
 * Simulation.cpp:659), C_abs from the Mie factors (Geometry.cpp:86-145)}. */
int om_cross_sections(om_problem *pr, double out[4]);
/* Result::getEHFields at Cartesian points (Result.cpp:74-301), fundamental,
 * Cartesian components: E, H are 3 complex per point. */
int om_near_field(om_problem *pr, const double *xyz, int npts, double *E, double *H);

/* Second harmonic (the SH half of PreconditionedMatrix::solve,
 * PreconditionedMatrixSolver.h:62-78): source K and K1ana from the FF internal
 * coefficients (source_vectorSH / source_vectorSH_K1ana, PreconditionedMatrix.cpp:
 * 1347-1436, with the nine coupling tables of Symbol.cpp:1036-1451), solve with
 * the SH matrix (om_assemble(pr, OM_SH, ...) first), then convertInternal_SH
 * (Solver.cpp:95-116). Needs a fundamental solution (om_solve). */
int om_solve_sh(om_problem *pr, const om_solve_options *opts, om_solve_stats *stats);
/* SH source and its analytic part (K, K1ana; n each, either may be NULL) and SH
 * scattered / internal coefficients (either may be NULL). */
int om_get_sh_vectors(om_problem *pr, double *K, double *K1ana, double *X_sca_SH,
                      double *X_int_SH);
/* Result::getEHFields, second-harmonic half, at Cartesian points
 * (Result.cpp:166-199, 237-276, with the particular solution of
 * Result::setFields / Geometry::COEFFpartSH, Result.cpp:906-919,
 * Geometry.cpp:458-491): E_SH, H_SH, 3 complex per point. Needs om_solve_sh. */
int om_near_field_sh(om_problem *pr, const double *xyz, int npts, double *E, double *H);
/* Result::getScatteringCrossSection_SH and getAbsorptionCrossSection_SH
 * (Result.cpp:662-778, Symbol.cpp:358-477): out = {C_sca_SH, C_abs_SH}. */
int om_sh_cross_sections(om_problem *pr, double out[2]);
/* The nine SH coupling tables for nMaxS = nMax (9 x P^3 doubles, order C_10m1,
 * C_11m1, C_00m1, C_01m1, W_m1m1, W_11, W_00, W_10, W_01; [k][p][q]),
 * computed on the device (Geometry::Coefficients, Geometry.cpp:234-247). */
int om_clg_tables(om_context *ctx, int nmax, double *out);

/* One wavelength-solve from host buffers to host buffers: problem set-up,
 * source vector, FF assembly, solve, internal coefficients, cross sections
 * (the body of Simulation::scan_wavelengths' loop, Simulation.cpp:643-674,
 * fundamental part).
 * X_sca / X_int may be NULL. */
int om_wavelength_solve(om_context *ctx, const om_sphere *spheres, int n_spheres,
                        const om_medium *background, const om_plane_wave *wave,
                        const om_solve_options *opts, int precision, double xsec[4],
                        double *X_sca, double *X_int, om_solve_stats *stats);
/* As om_wavelength_solve, followed, when wave->sh is set, by the SH assembly
 * (same precision), om_solve_sh and om_sh_cross_sections into xsec_sh[2]. */
int om_wavelength_solve_sh(om_context *ctx, const om_sphere *spheres, int n_spheres,
                           const om_medium *background, const om_plane_wave *wave,
                           const om_solve_options *opts, int precision, double xsec[4],
                           double xsec_sh[2], om_solve_stats *stats);

/* ---------------------------------------------------------------------------
 * Serving and batching. No counterpart in the reference, whose
 * Simulation::scan_wavelengths (Simulation.cpp:604-685) runs one
 * wavelength-solve after another on one process.
 *
 * A server owns `slots` device contexts on one GPU, each driven by its own
 * host thread and stream. Requests are taken in arrival order by the first
 * free slot (continuous batching: a request that arrives while others run
 * starts as soon as a slot and device memory are free, and its kernels overlap
 * theirs on the device). Admission is against `hbm_budget` bytes: a request's
 * device memory (matrix, Krylov basis, solver workspace) is estimated from
 * N, nMax, the precision and the solve options, and it waits until the running
 * and resident requests leave room; one that cannot fit even on an empty
 * device fails with OM_ERR_BUDGET. A slot keeps its problem (matrix storage,
 * per-sphere state) resident after a request and reuses it for the next one
 * with the same non-zero cluster_key (a wavelength scan), releasing it under
 * memory pressure. Results do not depend on the slot or on what else runs:
 * every kernel reduces in a fixed order.
 * ------------------------------------------------------------------------- */
typedef struct om_server om_server;

typedef struct {
  const om_sphere *spheres;       /* copied by om_server_submit */
  int n_spheres;
  int precision;                  /* OM_C128 (plain form) or OM_C64 (precision form) */
  om_medium background;
  om_plane_wave wave;             /* wave.sh = 1 attaches the second-harmonic solve */
  om_solve_options opts;          /* used for the FF and the SH solve */
  unsigned long long cluster_key; /* non-zero: same spheres as earlier requests with this key */
} om_request;

typedef struct {
  int status;                     /* OM_OK or the first failing call's code */
  int slot;                       /* slot that served the request */
  double xsec[4];                 /* as om_cross_sections */
  double xsec_sh[2];              /* as om_sh_cross_sections (SH requests) */
  om_solve_stats ff, sh;          /* solve statistics */
  double queue_ms;                /* submit -> start of service (host clock) */
  double service_ms;              /* start of service -> result */
  double latency_ms;              /* submit -> result */
  size_t device_bytes;            /* admission estimate */
} om_result;

int om_server_create(int device, size_t hbm_budget, int slots, om_server **out);
/* Copies the request; returns its ticket. */
int om_server_submit(om_server *srv, const om_request *rq, unsigned long long *ticket);
/* OM_PENDING while the request runs (wait = 0) or blocks until it finishes
 * (wait != 0); on completion fills *out and forgets the ticket. */
int om_server_poll(om_server *srv, unsigned long long ticket, int wait, om_result *out);
/* Blocks until every submitted request has finished. */
int om_server_drain(om_server *srv);
/* Records an event on every slot's stream, waits for them and returns in *ms
 * the device time from the earliest event of the previous mark to the latest
 * of this one (0 for the first). */
int om_server_mark(om_server *srv, double *ms);
/* Batched service: with max_requests > 1, requests that om_batch_solve runs
 * (OM_C128 with OM_SOLVE_GMRES, OM_C64 with OM_SOLVE_FGMRES_MIXED) whose
 * batched footprint (FF and SH matrices together plus the slot's vectors) is
 * at most max_request_bytes (0 = any) are batchable. A free slot serves the
 * head of the queue on the single-request path when it is not batchable and
 * fits; otherwise it takes the batchable requests of the queue in arrival
 * order, at most max_requests and within the budget, and serves them in one
 * om_batch_solve call (arena_bytes as there; 0 = the run's own footprint).
 * max_requests <= 1 turns it off (the default). Each path's results are
 * fixed-order reductions (bitwise reproducible); the two paths agree within
 * the solver tolerance. */
int om_server_batching(om_server *srv, int max_requests, size_t arena_bytes,
                       size_t max_request_bytes);
/* om_context_tune on every slot; only while no request is outstanding. */
int om_server_tune(om_server *srv, const om_tuning *t);
/* Autotuner of the launch tuning: runs `count` requests like *rq (its cluster
 * key and options, successive wavelengths from rq->wave.wavelength in steps of
 * `step` metres) under each of a few built-in tunings (matvec grid caps,
 * shared-memory carveouts), keeps the one with the shortest device time and
 * returns it in *chosen (may be NULL). Results do not depend on the tuning. */
int om_server_autotune(om_server *srv, const om_request *rq, int count, double step,
                       om_tuning *chosen);
/* Kernels launched by all requests finished since the previous call. */
long om_server_launches(om_server *srv);
const char *om_server_last_error(om_server *srv);
void om_server_destroy(om_server *srv);

/* Batched wavelength solves (the batching form): runs `count` requests on the
 * context's stream and fills results[i] for reqs[i] (status, cross sections,
 * solve statistics; slot = the request's slot in its batch; queue_ms = call
 * start -> start of its batch; service_ms = its batch's time; latency_ms =
 * call start -> its results). Requests are grouped into size classes (same
 * precision, nMax and options; N padded up to 1, 2, 3, 4, 6, 8, 12, 16, ...)
 * and solved in batches whose device memory stays within `arena_bytes`
 * (0 = 40 % of the free device memory, at most 64 GiB). Per batch one
 * assembly launch builds the FF and SH matrices of all its requests, and the
 * systems are solved together by restarted GMRES whose steps are captured
 * CUDA graphs (one set per size class). Supported: OM_C128 with
 * OM_SOLVE_GMRES (restarts cycles of at most max_iter steps) and OM_C64 with
 * OM_SOLVE_FGMRES_MIXED, run as GMRES-based iterative refinement: at most
 * min(max_iter, 32) x restarts refinement steps, each with an FP64-accurate
 * residual and an FP32 GMRES of at most inner_iter steps that reduces it by
 * inner_tol. Other requests get OM_ERR_INVALID. A request's results do not
 * depend on the batch it runs in. cluster_key is not used.
 * Returns OM_OK unless a device error stopped the call; per-request failures
 * (overlap, not converged, budget) are in results[i].status. */
int om_batch_solve(om_context *ctx, const om_request *reqs, int count, size_t arena_bytes,
                   om_result *results);
/* The batched matvecs' tile configurations chosen so far on this context,
 * one per size class (the autotuner times each candidate on the class's
 * first batch and keeps the fastest): out[7 i .. 7 i + 6] = {precision,
 * nMax, padded N, rows per tile, tile order (0 slot by slot, 1 interleaved
 * across slots), CTAs per SM, microseconds of one Arnoldi matvec of that
 * batch}. Returns the number of classes (at most max_entries are written). */
int om_batch_tiles(om_context *ctx, int *out, int max_entries);

#ifdef __cplusplus
}
#endif

#endif /* OPTIMET_GPU_H */
