/*
 * dagtm_gb300.h -- C ABI of the GB300 (sm_103a) DA-GTM annealed EM step.
 *
 * One opaque context owns every device buffer of one GTM problem
 * (N data points T in D dimensions, K latent points, M1 = M + 1 basis
 * functions FI).  The data T stays resident on the GPU; the K x N distance
 * and responsibility matrices of the reference are never stored: the E-step
 * keeps two numbers per data point (the column log-sum-exp statistics) and
 * the M-step recomputes responsibilities tile by tile.
 *
 * Host arrays are row-major doubles with an explicit leading dimension
 * (GSL's tda is accepted as is) and are only borrowed for the call.
 * Every entry point is synchronous at the ABI edge, returns 0 on success or
 * one of the DGTM_E* codes, and never aborts; dgtm_last_error_string()
 * describes the last failure of the calling thread.  A context is used by
 * one host thread at a time; it runs on the CUDA device that was current
 * when it was created, on a stream of its own.
 *
 * Citations name the reference routine each entry point replaces
 * (jychoi-hpc/da-gtm, paths relative to the checkout).
 */
#ifndef DAGTM_GB300_H
#define DAGTM_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dgtm_ctx dgtm_ctx;

/* precision forms */
#define DGTM_FP64 0   /* plain FP64, as the reference computes               */
#define DGTM_FP32 1   /* FP32 arithmetic, FP64 reductions and M-step         */
#define DGTM_BF16X3 2 /* tensor-core split-BF16 distances, FP64 reductions  */

/* M-step solvers */
#define DGTM_SOLVE_CHOLESKY 0 /* FP64 Cholesky (default)                          */
#define DGTM_SOLVE_SVD 1      /* symmetric-eigen SVD, exactly-zero values dropped  */

/* status codes */
#define DGTM_OK 0
#define DGTM_EINVAL 1     /* bad argument or shape                              */
#define DGTM_ECUDA 2      /* CUDA runtime error                                 */
#define DGTM_ENOTSPD 3    /* A = FI^T diag(G) FI not positive definite         */
#define DGTM_ENONFINITE 4 /* a non-finite value where a finite one is required  */
#define DGTM_ETIMEOUT 5   /* a device-side wait gave up (kernel returned early) */
#define DGTM_ENOMEM 6     /* device allocation failed                           */
#define DGTM_ESTATE 7     /* call out of order (e.g. M-step before any E-step)  */
#define DGTM_ENOTSUP 8    /* form or size not supported on this device          */

/* Version of this ABI (major * 10000 + minor * 100 + patch). */
int dgtm_version(void);

/* Description of the calling thread's last error ("" if none). */
const char *dgtm_last_error_string(void);

/*
 * Create a context: uploads T (N x D, leading dimension ldT) and FI
 * (K x M1, leading dimension ldFI) to the current device.  precision is one
 * of DGTM_FP64, DGTM_FP32, DGTM_BF16X3.  DGTM_BF16X3 needs a Blackwell
 * (sm_10x) device and D <= 189; otherwise it returns DGTM_ENOTSUP.
 * Replaces the set-up of dagtm/dagtm.cxx:1031-1101 (allocation of the Kbar x
 * Nbar D and R blocks, hyperslab read of T) for a single process.
 */
int dgtm_ctx_create(int N, int D, int K, int M1, const double *T, int ldT,
                    const double *FI, int ldFI, int precision, dgtm_ctx **out);

/* Free every device buffer of the context (NULL is accepted). */
int dgtm_ctx_destroy(dgtm_ctx *ctx);

/* Choose the M-step solver (DGTM_SOLVE_*); Cholesky is the default.
 * The reference solves with a GSL SVD: comm/comm.c:1299-1348 (dagtm_solve2).
 * Limits on M1 (basis functions + bias): Cholesky 1024, SVD 1022; beyond
 * them dgtm_mstep returns DGTM_ENOTSUP. */
int dgtm_set_solver(dgtm_ctx *ctx, int solver);

/* Load the centres Y (K x D).  Replaces the distance pass that follows a
 * fresh set-up or a restart: dagtm/dagtm.cxx:1143,1232 (Y = FI W; dagtm_dist). */
int dgtm_set_Y(dgtm_ctx *ctx, const double *Y, int ldY);

/* Copy the current centres Y (K x D) and the last solved W (M1 x D) to the
 * host; either pointer may be NULL. */
int dgtm_get_Y(dgtm_ctx *ctx, double *Y, int ldY);
int dgtm_get_W(dgtm_ctx *ctx, double *W, int ldW);

/*
 * E-step at (beta, temp): responsibilities R_kn ∝ exp(-beta d_kn/2)^(1/temp)
 * normalised over k, without storing R.  Returns the two qualities of the
 * reference: *llh (log-likelihood, normalised by N) and *nfree (the
 * annealed quality, temp * sum_n log sum_k exp(-beta d/2)^(1/temp), same
 * normalisation; = -llh when isDA == 0).  Zero columns (every exp()
 * underflowing) follow the reference's fallback: R column = 1/K, llh term
 * log 0 = -inf, nfree term log K.
 * Replaces comm/mpicomm.c:316-414 (dagtm_mpi_resp) and the two
 * comm/mpicomm.c:463-500 (dagtm_mpi_qual) calls of dagtm/dagtm.cxx:1541-1563.
 */
int dgtm_estep(dgtm_ctx *ctx, double beta, int isDA, double temp, double *llh,
               double *nfree);

/*
 * M-step on the responsibilities of the last E-step:
 *   G = rowsum R, RT = R T, A = FI^T diag(G) FI, B = FI^T RT, A W = B,
 *   Y = FI W, beta = N D / sum_kn R_kn |y_k - t_n|^2  (with the new Y).
 * W (M1 x D) and Y (K x D) are copied out when non-NULL; *beta receives the
 * new beta.  The context keeps the new Y for the next E-step.
 * Replaces the inline M-step dagtm/dagtm.cxx:1715-1770 (with dagtm_solve2,
 * comm/comm.c:1299-1348) and comm/mpicomm.c:276-302 (dagtm_mpi_beta).
 */
int dgtm_mstep(dgtm_ctx *ctx, double *W, int ldW, double *Y, int ldY,
               double *beta);

/*
 * Row sums G (K) and the raw statistics RT = R T (K x D) of the last E-step's
 * responsibilities, as computed inside dgtm_mstep (for checking and for the
 * gradient of the free energy).  Either pointer may be NULL.
 */
int dgtm_get_stats(dgtm_ctx *ctx, double *G, double *RT, int ldRT);

/*
 * Posterior-mean projection M = R^T X (N x L) with the responsibilities of
 * the last E-step.  X is K x L (leading dimension L).
 * Replaces dagtm/dagtm.cxx:2348-2355 (MAP before the output is written) and
 * the -I interpolation pass of dagtm/dagtm.cxx:1247-1295.
 */
int dgtm_map(dgtm_ctx *ctx, const double *X, int L, double *M, int ldM);

/*
 * Responsibilities of the last E-step for the block k0..k0+nk-1 x
 * n0..n0+nn-1, written to R (nk x nn, leading dimension ldR).
 * Replaces the -R dump of dagtm/dagtm.cxx:2406-2414 (h5save_byblock of R).
 */
int dgtm_get_R_block(dgtm_ctx *ctx, int k0, int nk, int n0, int nn, double *R,
                     int ldR);

/*
 * The reference's output after a run that stopped on its iteration cap (-j):
 * there the break comes after dagtm_mpi_beta has multiplied R in place by
 * the squared distances to the new centres (comm/mpicomm.c:288), and the
 * MAP and the -R dump are computed from that R o D (dagtm/dagtm.cxx:2348-2355,
 * 2406-2414).  dgtm_map_rd and dgtm_get_RD_block give M = (R o D)^T X and
 * blocks of R o D: R of the last E-step (on the centres before the last
 * M-step, which the context keeps) times the squared distance of each point
 * to the current centres.  They need an M-step after the last E-step
 * (DGTM_ESTATE otherwise).  FP64 in every precision form.
 */
int dgtm_map_rd(dgtm_ctx *ctx, const double *X, int L, double *M, int ldM);
int dgtm_get_RD_block(dgtm_ctx *ctx, int k0, int nk, int n0, int nn, double *R, int ldR);

/*
 * Next critical temperature of the AUTO cooling schedule, from the
 * responsibilities R of the last E-step.  For each centre k, with
 * x_n = t_n - y_k:  S1 = sum_n R_kn x_n x_n^T, S2 = sum_n R_kn^2 x_n x_n^T,
 * H_k = [[2 S1 - S2, -S2], [-S2, 2 S1 - S2]]; the eigenvalues of H_k at or
 * above (temp - eps) gg_k 2 / beta count as 0, ctemp_k = beta / 2 / gg_k
 * times the largest (HUGE_VAL when gg_k = 0), and *ctemp = max_k ctemp_k.
 * gg: K weights on the host (the reference passes its G of the last M-step),
 * or NULL for the row sums of the current R.  The work is about K N D^2 FMA
 * plus 2K symmetric eigenproblems of size D.  The FP64 form computes in
 * FP64; the FP32 and split forms build S1 and S2 from FP32 products (sums
 * in FP64) and take the eigenvalues in FP32, within their stated 1e-4.
 * Scratch: DGTM_CTEMP_SCRATCH_MB (default 256) bounds the device memory of
 * one batch of centres, DGTM_CTEMP_CHUNK (default 16384) the points per chunk.
 * The split form on 0/1 data forms S1 and S2 instead as a tensor-core GEMM of
 * R and R^2 (split BF16) against the pair features (t_i t_j, t_i, 1), which
 * are exact in BF16, with DGTM_CTEMP_GEMM_MB (default 8192) of scratch;
 * DGTM_CTEMP_PAIRS=0 selects the CUDA-core scatter for those contexts too.
 * Replaces dagtm_mpi_next_ctemp and its helper (comm/mpicomm.c:562-674) with
 * dagtm_vector_max (comm/comm.c:2149-2161), called at dagtm/dagtm.cxx:1919-1934.
 */
int dgtm_next_ctemp(dgtm_ctx *ctx, double temp, double beta, double eps, const double *gg,
                    double *ctemp);

/*
 * dgtm_next_ctemp that also returns every centre's ctemp_k in ctemp_k[0..K)
 * (host, may be NULL): the reference's vctemp, which the hierarchical (HDA)
 * schedule writes as ctemp.<i> before it expands the latent grid
 * (dagtm/dagtm.cxx:1958-2067).
 */
int dgtm_next_ctemp_k(dgtm_ctx *ctx, double temp, double beta, double eps, const double *gg,
                      double *ctemp_k, double *ctemp);

/*
 * Per-phase device timers, the counterpart of the reference's LOG_TICTOC
 * phase counters (comm/log.h:35-75, printed by logfullWithPID at
 * dagtm/dagtm.cxx:2286).  When enabled, CUDA events bracket each phase on the
 * context's stream; times (ms), kernel launches and phase calls accumulate
 * until dgtm_reset_timing.  Phases:
 */
#define DGTM_PHASE_ESTEP 0        /* distance + column log-sum-exp kernel      */
#define DGTM_PHASE_ESTEP_REDUCE 1 /* quality reductions                        */
#define DGTM_PHASE_MSTEP_PASS 2   /* responsibility pass: G, RT                */
#define DGTM_PHASE_MSTEP_SOLVE 3  /* slice sums, A, B, solve, Y (and its copies), beta */
#define DGTM_NPHASES 4
int dgtm_set_timing(dgtm_ctx *ctx, int on);
int dgtm_reset_timing(dgtm_ctx *ctx);
int dgtm_get_timing(dgtm_ctx *ctx, double *ms, long long *launches, long long *calls);

/* The CUDA stream (cudaStream_t) the context launches on, for callers that
 * order their own work or events against it. */
int dgtm_get_stream(dgtm_ctx *ctx, void **stream);

/* Which implementation runs the context's E-step and responsibility pass
 * (informational; no reference counterpart).  DGTM_FP64 contexts on 0/1 data
 * (D <= 189, K <= 60000) on an sm_10x GPU use the exact-slice path: distance
 * products from fixed-point digit slices of the centres on the tensor cores
 * (exact integers), exponentials and sums in double-float and 2^-48 fixed
 * point.  Setting DGTM_X64=0 before dgtm_ctx_create keeps them on the
 * CUDA-core FP64 kernels. */
#define DGTM_PATH_CUDA_CORES 0
#define DGTM_PATH_SPLIT_BF16 1
#define DGTM_PATH_EXACT_SLICES 2
int dgtm_get_path(dgtm_ctx *ctx, int *path);

/*
 * Annealed free energy and its gradient on caller-owned device arrays, for
 * gradient-based refinement (torch.autograd) and the projection of new points:
 *   F = N (D/2 ln(beta/2pi) - ln K) + temp sum_n ln sum_k exp(-beta d_kn/(2 temp))
 * Y (K x D) and T (N x D) are row-major FP32 device arrays; reductions are
 * FP64.  F, gF and dbeta point to one device double each.  The workspace (a
 * 256-byte aligned device buffer of at least dgtm_fe_workspace_size bytes)
 * carries two numbers per point from the forward to the backward call, which
 * must receive the same Y, T, beta, temp and workspace.  Work is enqueued on
 * `stream` (a cudaStream_t) and not synchronised; any of dY, dT, dbeta may be
 * NULL.  The backward recomputes the responsibilities tile by tile:
 *   dY = -gF beta (G Y - R T),  dT = -gF beta (T - R^T Y),
 *   dbeta = gF (N D / (2 beta) - sum_kn R_kn d_kn / 2).
 * F is N times the reference's DA quality (comm/mpicomm.c:463-500); the
 * gradient has no counterpart in the reference.
 */
int dgtm_fe_workspace_size(int N, int K, int D, size_t *bytes);
int dgtm_fe_forward(const float *Y, const float *T, int N, int K, int D, double beta,
                    double temp, void *workspace, size_t ws_bytes, void *stream, double *F);
int dgtm_fe_backward(const float *Y, const float *T, int N, int K, int D, double beta,
                     double temp, void *workspace, size_t ws_bytes, void *stream,
                     const double *gF, float *dY, float *dT, double *dbeta);

/*
 * dgtm_fe_forward for callers that cannot allocate device memory at all, not
 * even a workspace: code running where cudaMalloc is forbidden or unwanted (a
 * host callback; a process whose device memory is all handed out by another
 * allocator; a latency-critical loop that cannot pay for the synchronisation
 * an allocation implies).  It computes the same F with the FP32 CUDA-core
 * kernels of the FP32 form and writes it (one device double) the same way,
 * but keeps its scratch in a fixed array of DGTM_FE_NOALLOC_BYTES inside this
 * library, which every GPU that loads the library holds until the process
 * exits.  It calls no allocator.  Limits and rules:
 *   - the scratch needs about 24 N + 8 K bytes (plus alignment); problems
 *     that need more than DGTM_FE_NOALLOC_BYTES are rejected with
 *     DGTM_EINVAL and a message giving the bytes needed;
 *   - set-up happens in the first call on each device (and again in the first
 *     call after that device's context was destroyed and recreated, e.g. by
 *     cudaDeviceReset): with the device current it looks up the array's
 *     device address (cudaGetSymbolAddress).  Under CUDA's lazy module loading
 *     that lookup is what makes the driver load this library's device code,
 *     so the array is reserved on the device at that moment and not before.
 *     Make that first call before any stream capture; from the second call on
 *     nothing is loaded or reserved;
 *   - all calls share the one array, so calls that may overlap on the GPU
 *     (other streams, other host threads) race with each other: serialise
 *     them; nothing in the array needs to start at zero.
 * No counterpart in the reference (which has no GPU code).
 */
#define DGTM_FE_NOALLOC_BYTES (8u << 20)
int dgtm_fe_forward_noalloc(const float *Y, const float *T, int N, int K, int D, double beta,
                            double temp, void *stream, double *F);

/*
 * Diagnostic: runs the three tensor-core operand configurations the split-BF16
 * kernels rely on (K-major x K-major from shared memory; K-major x MN-major;
 * tensor-memory A x MN-major) on small integer matrices and writes the largest
 * absolute error against a host product to errs[0..2] (0 when correct).  With
 * nerrs >= 4, errs[3] is the number of lanes in which the packed (f32x2)
 * double-float exp, add, mul and four-term sum of the exact-slice FP64 form
 * differ bitwise from the scalar ones over 2^20 argument pairs (0 when
 * correct).
 * No reference counterpart (the reference has no GPU code).
 */
int dgtm_selftest(double *errs, int nerrs);

/*
 * Diagnostic of the failure path: every wait in the tensor-core kernels is
 * bounded and, when it gives up, records a site code that the host turns into
 * DGTM_ETIMEOUT while the device stays usable.  This runs one such wait, with
 * limit_ms (1 .. 10000), on a barrier that nothing arrives at.  Returns
 * DGTM_ETIMEOUT with *site = 90 and the time the wait took in *waited_ms.
 * No reference counterpart (the reference has no GPU code).
 */
int dgtm_wait_probe(unsigned limit_ms, int *site, double *waited_ms);

#ifdef __cplusplus
}
#endif
#endif /* DAGTM_GB300_H */
