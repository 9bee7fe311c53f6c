/*
 * dagtm_oracle.h -- CPU FP64 restatement of DA-GTM's annealed EM step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU
 * implementation is compared against, and the timed CPU baseline of the
 * benchmark.  Nothing in the product path may link, load or call it.
 *
 * Every function restates one reference routine (cited file:line, paths
 * relative to the jychoi-hpc/da-gtm checkout) with the reference's own
 * semantics: dense K x N distance and responsibility matrices, no max-shift
 * inside exp(), the zero-column fallback, log applied in place, the
 * int-typed N*D product.  Matrices are dense row-major doubles (the
 * reference's tda padding is a CPU cache detail and is not reproduced).
 *
 * Third-party arithmetic the reference delegates to GSL (unpinned version)
 * is restated from the published algorithms:
 *   - gsl_linalg_SV_decomp/SV_solve  -> one-sided Jacobi SVD (Hestenes 1958),
 *     solve x = V diag(1/s) U^T b with exactly-zero singular values dropped;
 *   - gsl_eigen_symm                 -> cyclic Jacobi eigenvalue method;
 *   - gsl_rng_default (mt19937) + gsl_rng_uniform -> MT19937 of Matsumoto &
 *     Nishimura (2002 seeding), uniform = next32 / 2^32;
 *   - gsl_blas_dgemm/ddot/dger       -> plain loops, contraction index in
 *     increasing order.
 */
#ifndef DAGTM_ORACLE_H
#define DAGTM_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Threads used by the OpenMP loops (0 = OpenMP default). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* comm/comm.c:560-629 dagtm_dist_ws: Dm[k*N+n] = -2 y_k.t_n + |y_k|^2 + |t_n|^2 */
void orc_dist(int K, int N, int D, const double *Y, const double *T, double *Dm);

/* comm/mpicomm.c:316-414 dagtm_mpi_resp (single rank). */
void orc_resp(int K, int N, double beta, const double *Dm, int isDA,
              double temp, double *R, double *vgc, double *vgc2);

/* comm/mpicomm.c:463-500 dagtm_mpi_qual (single rank; log applied in place to v). */
double orc_qual(int N, int K, int D, double beta, double *v, int isDA, double temp);

/* dagtm/dagtm.cxx:1715-1761: G = rowsum R, A = FI^T diag(G) FI, B = (FI^T R) T. */
void orc_mstep_stats(int K, int N, int D, int M1, const double *R,
                     const double *FI, const double *T, double *G, double *A,
                     double *B);

/* comm/comm.c:1299-1348 dagtm_solve2: A X = B by SVD (n x n A, n x k B). */
int orc_solve2(int n, int k, const double *A, const double *B, double *X);

/* FP64 Cholesky solve of the same system (the GPU's default solver); pivots
 * keeping <= 1e-12 of their diagonal are dropped.  Returns the number dropped. */
int orc_solve_chol(int n, int k, const double *A, const double *B, double *X);

/* Y = FI W  (dagtm/dagtm.cxx:1769) */
void orc_fiw(int K, int M1, int D, const double *FI, const double *W, double *Y);

/* comm/mpicomm.c:276-302 dagtm_mpi_beta: Dm <- dist(Y,T); R <- R o Dm;
 * returns (N*D)/sum(R). */
double orc_beta(int K, int N, int D, const double *Y, const double *T,
                double *R, double *Dm);

/* ---- set-up (runs once on the host in the reference) ---- */
/* comm/comm.c:1453-1504 dagtm_rctg for L in {1,2,3}: regular grid in [-1,1]^L. */
void orc_rctg(int L, int gdim, double *X);
/* comm/comm.c:1506-1536 dagtm_gbf: FI = [exp(-|x-mu|^2/(2 sigma^2)) | 1]. */
void orc_gbf(int K, int M, int L, const double *MU, const double *X,
             double sigma, double *FI);
/* comm/comm.c:992-1103 dagtm_stp (GRID_SWEEP only): X (K x L), FI (K x (M+1)). */
int orc_stp(int L, int K, int M, double s, double *X, double *FI);
/* comm/comm.c:1401-1448 dagtm_yrnd2: uniform mu +- 6 sd from MT19937(seed). */
void orc_yrnd2(unsigned long seed, int K, int D, const double *mu,
               const double *sd, double *Yrnd);
/* comm/comm.c:1247-1294 dagtm_solve: least squares (A^T A) X = A^T B by SVD. */
int orc_solve_ls(int m, int n, int k, const double *A, const double *B, double *X);
/* comm/comm.c:1161-1185 dagtm_bi: 2 / mean nearest-neighbour squared distance. */
double orc_bi(int K, int D, const double *Y);
/* comm/comm.c:1118-1156 dagtm_stp3_rnd: X, FI, W, beta. */
int orc_stp3_rnd(unsigned long seed, const double *mu, const double *sd, int D,
                 int L, int K, int M, double s, double *X, double *FI,
                 double *W, double *beta);
/* comm/mpicomm.c:686-730 dagtm_mpi_mean / dagtm_mpi_sd. */
void orc_mean(int N, int D, const double *T, double *mu);
void orc_sd(int N, int D, const double *T, const double *mu, double *sd);
/* comm/mpicomm.c:511-559 dagtm_mpi_ctemp: first critical temperature. */
double orc_ctemp(int N, int D, const double *T);
/* Largest eigenvalue helper (cyclic Jacobi), exposed for tests. */
int orc_eig_sym(int n, const double *S, double *lambda);
/* Next critical temperature of the AUTO schedule (comm/mpicomm.c:562-674,
 * comm/comm.c:2149-2161); R is K x N, gg the K weights (vggsub). */
double orc_next_ctemp(int N, int D, int K, const double *T, const double *Y, const double *R,
                      const double *gg, double temp, double beta, double eps);
/* MT19937 stream helper for tests: n uniforms from gsl_rng_set(seed). */
void orc_mt_uniform(unsigned long seed, int n, double *out);

/* ---- one EM iteration and the annealing loop ---- */
/*
 * One iteration of dagtm/dagtm.cxx:1531-1795 without the convergence tests:
 * resp (on Dm) -> llh/nfree -> G, A, B -> W = solve -> Y = FI W -> beta.
 * Dm (K x N) holds dist(Y, T) on entry and dist(Y_new, T) on exit; R (K x N)
 * is workspace (left holding R o Dm, as the reference does).
 * solver: 0 = SVD (reference), 1 = Cholesky.
 */
int orc_em_iteration(int N, int D, int K, int M1, const double *T,
                     const double *FI, double *Y, double *W, double *beta,
                     int isDA, double temp, double *Dm, double *R, double *vgc,
                     double *vgc2, double *llh, double *nfree, int solver);

/*
 * The temperature loop of dagtm/dagtm.cxx:1508-1795,1910-2206 for the EXP and
 * LINEAR schedules (no HDA), started from a restart state (FI, Y, beta, temp)
 * as after dagtm/dagtm.cxx:1161-1232.  Per iteration it records temp, nfree,
 * llh and the beta used by that iteration's E-step.
 *   schedule: 0 = EXP (temp *= alpha), 1 = LINEAR (temp -= delta)
 *   maxloop : 0 = unlimited (counted from iter0, as after a restart)
 * On exit Y, W, beta, *temp_io hold the final state, R_out (optional, K x N)
 * the responsibilities as left by the reference (clean after a convergence
 * break, R o D after a maxloop break) and *n_out the number of iterations.
 */
int orc_run(int N, int D, int K, int M1, const double *T, const double *FI,
            double *Y, double *W, double *beta_io, double *temp_io, int isDA,
            int schedule, double alpha, double delta, double eps, int iter0,
            int maxloop, int solver, int cap, double *tr_temp,
            double *tr_nfree, double *tr_llh, double *tr_beta, int *n_out,
            double *R_out);

#ifdef __cplusplus
}
#endif
#endif
