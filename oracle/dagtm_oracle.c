/*
 * dagtm_oracle.c -- CPU FP64 restatement of DA-GTM's annealed EM step.
 *
 * TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline).  The
 * product path never links or calls this file.  See dagtm_oracle.h for the
 * list of reference routines restated here; each function below cites the
 * reference file:line it follows.  Built with -ffp-contract=off so that the
 * x86 container and the aarch64 GPU host produce the same bits.
 */
#include "dagtm_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int g_threads = 0;

void orc_set_threads(int n)
{
    g_threads = n;
#ifdef _OPENMP
    if (n > 0)
        omp_set_num_threads(n);
#endif
}

int orc_get_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ */
/* distances                                                           */
/* ------------------------------------------------------------------ */

/*
 * comm/comm.c:560-629 (dagtm_dist_ws, GSL branch):
 *   D = -2 * Y T^T               (gsl_blas_dgemm, alpha = -2, beta = 0)
 *   v1_k = y_k . y_k, v2_n = t_n . t_n   (gsl_blas_ddot)
 *   D += v1 (x) 1 ; D += 1 (x) v2        (two gsl_blas_dger)
 * Contraction indices run in increasing order.
 */
void orc_dist(int K, int N, int D, const double *Y, const double *T, double *Dm)
{
    double *v2 = (double *) malloc(sizeof(double) * (size_t) (N > 0 ? N : 1));
    int n;
#pragma omp parallel for schedule(static)
    for (n = 0; n < N; n++) {
        const double *t = T + (size_t) n * D;
        double s = 0.0;
        for (int l = 0; l < D; l++)
            s += t[l] * t[l];
        v2[n] = s;
    }
    int k;
#pragma omp parallel for schedule(dynamic, 4)
    for (k = 0; k < K; k++) {
        const double *y = Y + (size_t) k * D;
        double v1 = 0.0;
        for (int l = 0; l < D; l++)
            v1 += y[l] * y[l];
        double *row = Dm + (size_t) k * N;
        int nn = 0;
        /* four independent dot products per pass; each keeps the l order */
        for (; nn + 4 <= N; nn += 4) {
            const double *t0 = T + (size_t) nn * D;
            const double *t1 = t0 + D, *t2 = t1 + D, *t3 = t2 + D;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            for (int l = 0; l < D; l++) {
                double yl = y[l];
                a0 += yl * t0[l];
                a1 += yl * t1[l];
                a2 += yl * t2[l];
                a3 += yl * t3[l];
            }
            row[nn + 0] = -2.0 * a0;
            row[nn + 1] = -2.0 * a1;
            row[nn + 2] = -2.0 * a2;
            row[nn + 3] = -2.0 * a3;
        }
        for (; nn < N; nn++) {
            const double *t0 = T + (size_t) nn * D;
            double a0 = 0.0;
            for (int l = 0; l < D; l++)
                a0 += y[l] * t0[l];
            row[nn] = -2.0 * a0;
        }
        for (nn = 0; nn < N; nn++)
            row[nn] += v1;
        for (nn = 0; nn < N; nn++)
            row[nn] += v2[nn];
    }
    free(v2);
}

/* ------------------------------------------------------------------ */
/* E-step                                                              */
/* ------------------------------------------------------------------ */

/*
 * comm/mpicomm.c:316-414 (dagtm_mpi_resp), one rank:
 *   R = D; R *= -beta/2; R = exp(R); vgc = colsum(R)           (:324-344)
 *   if isDA: R = pow(R, 1/temp); vgc2 = colsum(R); v = vgc2     (:348-357)
 *   zero column j: v_j = K, R[:,j] = 1                          (:382-389)
 *   R[:,j] /= v_j                                               (:390)
 * Column sums run over k in increasing order (comm/vec.c:316-336).
 */
void orc_resp(int K, int N, double beta, const double *Dm, int isDA,
              double temp, double *R, double *vgc, double *vgc2)
{
    const double sc = -beta / 2.0;
    const double p = 1.0 / temp;
    int n;
#pragma omp parallel for schedule(static)
    for (n = 0; n < N; n++) {
        double s1 = 0.0, s2 = 0.0;
        for (int k = 0; k < K; k++) {
            size_t i = (size_t) k * N + n;
            double r = exp(Dm[i] * sc);
            s1 += r;
            if (isDA) {
                r = pow(r, p);
                s2 += r;
            }
            R[i] = r;
        }
        vgc[n] = s1;
        double v;
        if (isDA) {
            vgc2[n] = s2;
            v = s2;
        } else {
            v = s1;
        }
        if (v == 0.0) {
            v = (double) K;
            for (int k = 0; k < K; k++)
                R[(size_t) k * N + n] = 1.0;
            if (isDA)
                vgc2[n] = v;
            else
                vgc[n] = v;
        }
        for (int k = 0; k < K; k++)
            R[(size_t) k * N + n] /= v;
    }
}

/*
 * comm/mpicomm.c:463-500 (dagtm_mpi_qual), one rank:
 *   v = log(v) (in place); sum = sum_n v_n
 *   qual = N*((D/2) log(beta/(2 pi)) - log K) + (isDA ? temp*sum : sum); qual /= N
 */
double orc_qual(int N, int K, int D, double beta, double *v, int isDA, double temp)
{
    double sum = 0.0;
    for (int n = 0; n < N; n++) {
        v[n] = log(v[n]);
        sum += v[n];
    }
    double qual = N * ((D / 2.0) * log(beta / (2.0 * M_PI)) - log((double) K));
    if (isDA)
        qual += temp * sum;
    else
        qual += sum;
    return qual / (double) N;
}

/* ------------------------------------------------------------------ */
/* M-step                                                              */
/* ------------------------------------------------------------------ */

/*
 * dagtm/dagtm.cxx:1715-1761:
 *   G = rowsum(R)                                  (:1715, comm/vec.c:298-314)
 *   GFI = FI scaled by row with G; A = FI^T GFI    (:1729-1732, comm/comm.c:268-291)
 *   FIR = FI^T R; B = FIR T                        (:1746-1753)
 */
void orc_mstep_stats(int K, int N, int D, int M1, const double *R,
                     const double *FI, const double *T, double *G, double *A,
                     double *B)
{
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < K; k++) {
        const double *r = R + (size_t) k * N;
        double s = 0.0;
        for (int n = 0; n < N; n++)
            s += r[n];
        G[k] = s;
    }
    memset(A, 0, sizeof(double) * (size_t) M1 * M1);
    for (k = 0; k < K; k++) {
        const double *fi = FI + (size_t) k * M1;
        for (int i = 0; i < M1; i++) {
            double tmp = fi[i];
            for (int j = 0; j < M1; j++)
                A[(size_t) i * M1 + j] += tmp * (fi[j] * G[k]);
        }
    }
    double *FIR = (double *) calloc((size_t) M1 * N, sizeof(double));
    int n;
#pragma omp parallel for schedule(static)
    for (n = 0; n < N; n++) {
        for (int kk = 0; kk < K; kk++) {
            double r = R[(size_t) kk * N + n];
            const double *fi = FI + (size_t) kk * M1;
            for (int i = 0; i < M1; i++)
                FIR[(size_t) i * N + n] += fi[i] * r;
        }
    }
    int i;
#pragma omp parallel for schedule(static)
    for (i = 0; i < M1; i++) {
        double *b = B + (size_t) i * D;
        for (int d = 0; d < D; d++)
            b[d] = 0.0;
        const double *fr = FIR + (size_t) i * N;
        for (int nn = 0; nn < N; nn++) {
            double tmp = fr[nn];
            const double *t = T + (size_t) nn * D;
            for (int d = 0; d < D; d++)
                b[d] += tmp * t[d];
        }
    }
    free(FIR);
}

/*
 * One-sided Jacobi SVD (Hestenes): A (m x n, m >= n) = U diag(s) V^T.
 * U overwrites a copy of A; columns with zero norm keep s = 0.
 * Stands in for gsl_linalg_SV_decomp (called at comm/comm.c:1273,1329).
 */
static void svd_jacobi(int m, int n, double *U, double *V, double *s)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++)
            V[(size_t) i * n + j] = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; sweep++) {
        int rotated = 0;
        for (int p = 0; p < n - 1; p++) {
            for (int q = p + 1; q < n; q++) {
                double a = 0.0, b = 0.0, g = 0.0;
                for (int i = 0; i < m; i++) {
                    double up = U[(size_t) i * n + p], uq = U[(size_t) i * n + q];
                    a += up * up;
                    b += uq * uq;
                    g += up * uq;
                }
                if (g == 0.0 || fabs(g) <= DBL_EPSILON * sqrt(a * b))
                    continue;
                rotated = 1;
                double zeta = (b - a) / (2.0 * g);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                double c = 1.0 / sqrt(1.0 + t * t);
                double sn = c * t;
                for (int i = 0; i < m; i++) {
                    double up = U[(size_t) i * n + p], uq = U[(size_t) i * n + q];
                    U[(size_t) i * n + p] = c * up - sn * uq;
                    U[(size_t) i * n + q] = sn * up + c * uq;
                }
                for (int i = 0; i < n; i++) {
                    double vp = V[(size_t) i * n + p], vq = V[(size_t) i * n + q];
                    V[(size_t) i * n + p] = c * vp - sn * vq;
                    V[(size_t) i * n + q] = sn * vp + c * vq;
                }
            }
        }
        if (!rotated)
            break;
    }
    for (int j = 0; j < n; j++) {
        double nrm = 0.0;
        for (int i = 0; i < m; i++)
            nrm += U[(size_t) i * n + j] * U[(size_t) i * n + j];
        nrm = sqrt(nrm);
        s[j] = nrm;
        if (nrm != 0.0)
            for (int i = 0; i < m; i++)
                U[(size_t) i * n + j] /= nrm;
    }
}

/* gsl_linalg_SV_solve semantics (quoted in comm/comm.c:1188-1239):
 * x = V diag(1/s_i, or 0 where s_i == 0) U^T b */
static void sv_solve(int m, int n, const double *U, const double *V,
                     const double *s, const double *b, int ldb, double *x, int ldx)
{
    double *w = (double *) calloc((size_t) n, sizeof(double));
    for (int i = 0; i < n; i++) {
        double acc = 0.0;
        for (int r = 0; r < m; r++)
            acc += U[(size_t) r * n + i] * b[(size_t) r * ldb];
        double al = s[i];
        if (al != 0.0)
            al = 1.0 / al;
        w[i] = al * acc;
    }
    for (int r = 0; r < n; r++) {
        double acc = 0.0;
        for (int i = 0; i < n; i++)
            acc += V[(size_t) r * n + i] * w[i];
        x[(size_t) r * ldx] = acc;
    }
    free(w);
}

/* comm/comm.c:1299-1348 (dagtm_solve2): SVD of A, then one SV_solve per column of B. */
int orc_solve2(int n, int k, const double *A, const double *B, double *X)
{
    double *U = (double *) malloc(sizeof(double) * (size_t) n * n);
    double *V = (double *) malloc(sizeof(double) * (size_t) n * n);
    double *s = (double *) malloc(sizeof(double) * (size_t) n);
    memcpy(U, A, sizeof(double) * (size_t) n * n);
    svd_jacobi(n, n, U, V, s);
    for (int j = 0; j < k; j++)
        sv_solve(n, n, U, V, s, B + j, k, X + j, k);
    free(U);
    free(V);
    free(s);
    return 0;
}

/* Cholesky A = L L^T and two triangular solves per column (FP64).  A pivot
 * keeping no more than 1e-12 of its diagonal is dropped (that unknown is 0),
 * the same rule as the GPU solver.  Returns the number of dropped pivots, or
 * -1 on a non-finite pivot. */
int orc_solve_chol(int n, int k, const double *A, const double *B, double *X)
{
    double *L = (double *) calloc((size_t) n * n, sizeof(double));
    int ndrop = 0;
    for (int j = 0; j < n; j++) {
        double d = A[(size_t) j * n + j];
        for (int p = 0; p < j; p++)
            d -= L[(size_t) j * n + p] * L[(size_t) j * n + p];
        if (!isfinite(d)) {
            free(L);
            return -1;
        }
        if (!(d > 1e-12 * A[(size_t) j * n + j])) {
            ndrop++;
            L[(size_t) j * n + j] = 0.0;
            continue; /* column j below the diagonal stays 0 */
        }
        d = sqrt(d);
        L[(size_t) j * n + j] = d;
        for (int i = j + 1; i < n; i++) {
            double v = A[(size_t) i * n + j];
            for (int p = 0; p < j; p++)
                v -= L[(size_t) i * n + p] * L[(size_t) j * n + p];
            L[(size_t) i * n + j] = v / d;
        }
    }
    double *z = (double *) malloc(sizeof(double) * (size_t) n);
    for (int c = 0; c < k; c++) {
        for (int i = 0; i < n; i++) {
            double v = B[(size_t) i * k + c];
            for (int p = 0; p < i; p++)
                v -= L[(size_t) i * n + p] * z[p];
            double lii = L[(size_t) i * n + i];
            z[i] = (lii != 0.0) ? v / lii : 0.0;
        }
        for (int i = n - 1; i >= 0; i--) {
            double v = z[i];
            for (int p = i + 1; p < n; p++)
                v -= L[(size_t) p * n + i] * X[(size_t) p * k + c];
            double lii = L[(size_t) i * n + i];
            X[(size_t) i * k + c] = (lii != 0.0) ? v / lii : 0.0;
        }
    }
    free(z);
    free(L);
    return ndrop;
}

/* dagtm/dagtm.cxx:1769: Y = FI W (gsl_blas_dgemm NoTrans/NoTrans). */
void orc_fiw(int K, int M1, int D, const double *FI, const double *W, double *Y)
{
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < K; k++) {
        double *y = Y + (size_t) k * D;
        for (int d = 0; d < D; d++)
            y[d] = 0.0;
        for (int m = 0; m < M1; m++) {
            double f = FI[(size_t) k * M1 + m];
            const double *w = W + (size_t) m * D;
            for (int d = 0; d < D; d++)
                y[d] += f * w[d];
        }
    }
}

/*
 * comm/mpicomm.c:276-302 (dagtm_mpi_beta):
 *   D = dist(Y, T); R = R o D; sum = sum(R); beta = (N * D) / sum
 * N * D is an int product in the reference (undefined past 2^31).
 * The sum runs row by row; per-row partials keep the order deterministic.
 */
double orc_beta(int K, int N, int D, const double *Y, const double *T,
                double *R, double *Dm)
{
    orc_dist(K, N, D, Y, T, Dm);
    double *rows = (double *) malloc(sizeof(double) * (size_t) (K > 0 ? K : 1));
    int k;
#pragma omp parallel for schedule(static)
    for (k = 0; k < K; k++) {
        double *r = R + (size_t) k * N;
        const double *dd = Dm + (size_t) k * N;
        double s = 0.0;
        for (int n = 0; n < N; n++) {
            r[n] = r[n] * dd[n];
            s += r[n];
        }
        rows[k] = s;
    }
    double sum = 0.0;
    for (k = 0; k < K; k++)
        sum += rows[k];
    free(rows);
    int nd = N * D;
    return nd / sum;
}

/* ------------------------------------------------------------------ */
/* set-up                                                              */
/* ------------------------------------------------------------------ */

/* comm/comm.c:1453-1504 (dagtm_rctg): x fastest, then y, then z; scale 2/(g-1), shift -1. */
void orc_rctg(int L, int gdim, double *X)
{
    int idx = 0;
    int m = gdim - 1;
    if (L == 1) {
        for (int x = 0; x < gdim; x++, idx++)
            X[idx] = x;
    } else if (L == 2) {
        for (int y = 0; y < gdim; y++)
            for (int x = 0; x < gdim; x++, idx++) {
                X[idx * 2 + 0] = x;
                X[idx * 2 + 1] = y;
            }
    } else {
        for (int z = 0; z < gdim; z++)
            for (int y = 0; y < gdim; y++)
                for (int x = 0; x < gdim; x++, idx++) {
                    X[idx * 3 + 0] = x;
                    X[idx * 3 + 1] = y;
                    X[idx * 3 + 2] = z;
                }
    }
    int total = idx * L;
    for (int i = 0; i < total; i++)
        X[i] = X[i] * (2 / (double) m) + -1.0;
}

/* comm/comm.c:1506-1536 (dagtm_gbf): dist(X, MU) scaled by -0.5/sigma^2, exp, bias column 1. */
void orc_gbf(int K, int M, int L, const double *MU, const double *X,
             double sigma, double *FI)
{
    double *DI = (double *) malloc(sizeof(double) * (size_t) K * M);
    orc_dist(K, M, L, X, MU, DI);
    double sc = -0.5 / pow(sigma, 2);
    for (int k = 0; k < K; k++) {
        for (int j = 0; j < M; j++)
            FI[(size_t) k * (M + 1) + j] = exp(DI[(size_t) k * M + j] * sc);
        FI[(size_t) k * (M + 1) + M] = 1.0;
    }
    free(DI);
}

/* comm/comm.c:992-1103 (dagtm_stp), GRID_SWEEP branch (:1004-1035,1083-1087). */
int orc_stp(int L, int K, int M, double s, double *X, double *FI)
{
    if (s <= 0)
        return -1;
    if (L < 1 || L > 3)
        return -2;
    int gx = (int) rint(pow(K, 1 / (double) L));
    int gf = (int) rint(pow(M, 1 / (double) L));
    if (pow(gx, L) != K)
        return -3;
    if (pow(gf, L) != M)
        return -4;
    double *MU = (double *) malloc(sizeof(double) * (size_t) M * L);
    orc_rctg(L, gx, X);
    orc_rctg(L, gf, MU);
    double scale = (double) gf / (gf - 1);
    for (int i = 0; i < M * L; i++)
        MU[i] *= scale;
    double sigma = s * (MU[1 * L + 0] - MU[0 * L + 0]);
    orc_gbf(K, M, L, MU, X, sigma, FI);
    free(MU);
    return 0;
}

/* MT19937 (Matsumoto & Nishimura), seeded as gsl_rng_set does for mt19937
 * (seed 0 -> 4357; 2002 initialisation), uniform = next32 / 2^32. */
typedef struct {
    uint32_t mt[624];
    int mti;
} mt_state;

static void mt_seed(mt_state *st, unsigned long seed)
{
    if (seed == 0)
        seed = 4357;
    st->mt[0] = (uint32_t) (seed & 0xffffffffUL);
    for (int i = 1; i < 624; i++)
        st->mt[i] = (uint32_t) (1812433253UL * (st->mt[i - 1] ^ (st->mt[i - 1] >> 30)) + (uint32_t) i);
    st->mti = 624;
}

static uint32_t mt_next(mt_state *st)
{
    static const uint32_t mag01[2] = {0x0u, 0x9908b0dfu};
    if (st->mti >= 624) {
        int kk;
        uint32_t y;
        for (kk = 0; kk < 624 - 397; kk++) {
            y = (st->mt[kk] & 0x80000000u) | (st->mt[kk + 1] & 0x7fffffffu);
            st->mt[kk] = st->mt[kk + 397] ^ (y >> 1) ^ mag01[y & 1u];
        }
        for (; kk < 623; kk++) {
            y = (st->mt[kk] & 0x80000000u) | (st->mt[kk + 1] & 0x7fffffffu);
            st->mt[kk] = st->mt[kk + (397 - 624)] ^ (y >> 1) ^ mag01[y & 1u];
        }
        y = (st->mt[623] & 0x80000000u) | (st->mt[0] & 0x7fffffffu);
        st->mt[623] = st->mt[396] ^ (y >> 1) ^ mag01[y & 1u];
        st->mti = 0;
    }
    uint32_t y = st->mt[st->mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
}

void orc_mt_uniform(unsigned long seed, int n, double *out)
{
    mt_state st;
    mt_seed(&st, seed);
    for (int i = 0; i < n; i++)
        out[i] = mt_next(&st) / 4294967296.0;
}

/* comm/comm.c:1401-1448 (dagtm_yrnd2): dev = 6 sd; rnd = ceil(u/1e-15)*1e-15;
 * y = 2 dev rnd - dev + mu, row by row. */
void orc_yrnd2(unsigned long seed, int K, int D, const double *mu,
               const double *sd, double *Yrnd)
{
    mt_state st;
    mt_seed(&st, seed);
    const double roundoff = 1E-15;
    for (int i = 0; i < K; i++)
        for (int j = 0; j < D; j++) {
            double dev = sd[j] * 6;
            double rnd = ceil((mt_next(&st) / 4294967296.0) / roundoff) * roundoff;
            double m = mu[j];
            Yrnd[(size_t) i * D + j] = 2 * dev * rnd - dev + m;
        }
}

/* comm/comm.c:1247-1294 (dagtm_solve): U = A^T A; SVD(U); AB = A^T B; X = SV_solve per column. */
int orc_solve_ls(int m, int n, int k, const double *A, const double *B, double *X)
{
    double *U = (double *) calloc((size_t) n * n, sizeof(double));
    double *V = (double *) malloc(sizeof(double) * (size_t) n * n);
    double *s = (double *) malloc(sizeof(double) * (size_t) n);
    double *AB = (double *) calloc((size_t) n * k, sizeof(double));
    for (int r = 0; r < m; r++)
        for (int i = 0; i < n; i++) {
            double a = A[(size_t) r * n + i];
            for (int j = 0; j < n; j++)
                U[(size_t) i * n + j] += a * A[(size_t) r * n + j];
            for (int j = 0; j < k; j++)
                AB[(size_t) i * k + j] += a * B[(size_t) r * k + j];
        }
    svd_jacobi(n, n, U, V, s);
    for (int j = 0; j < k; j++)
        sv_solve(n, n, U, V, s, AB + j, k, X + j, k);
    free(U);
    free(V);
    free(s);
    free(AB);
    return 0;
}

/* comm/comm.c:1161-1185 (dagtm_bi): D = dist(Y,Y); diag = DBL_MAX; column minima;
 * m = gsl_stats_mean (running mean in long double); 2/m (m == 0 -> 1). */
double orc_bi(int K, int D, const double *Y)
{
    double *Dm = (double *) malloc(sizeof(double) * (size_t) K * K);
    orc_dist(K, K, D, Y, Y, Dm);
    for (int i = 0; i < K; i++)
        Dm[(size_t) i * K + i] = DBL_MAX;
    long double mean = 0;
    for (int j = 0; j < K; j++) {
        double mn = Dm[j];
        for (int i = 1; i < K; i++)
            if (Dm[(size_t) i * K + j] < mn)
                mn = Dm[(size_t) i * K + j];
        mean += (mn - mean) / (j + 1);
    }
    double m = (double) mean;
    free(Dm);
    if (m == 0)
        m = 1;
    return 2 / m;
}

/* comm/comm.c:1118-1156 (dagtm_stp3_rnd): stp, yrnd2, W = solve(FI, Yrnd),
 * beta = 0.1 when K > 1000 else dagtm_bi(Yrnd). */
int orc_stp3_rnd(unsigned long seed, const double *mu, const double *sd, int D,
                 int L, int K, int M, double s, double *X, double *FI,
                 double *W, double *beta)
{
    int ret = orc_stp(L, K, M, s, X, FI);
    if (ret != 0)
        return -1;
    double *Yr = (double *) malloc(sizeof(double) * (size_t) K * D);
    orc_yrnd2(seed, K, D, mu, sd, Yr);
    orc_solve_ls(K, M + 1, D, FI, Yr, W);
    if (K > 1000)
        *beta = 0.1;
    else
        *beta = orc_bi(K, D, Yr);
    free(Yr);
    return 0;
}

/* comm/mpicomm.c:686-703 (dagtm_mpi_mean): colsum * (1/N). */
void orc_mean(int N, int D, const double *T, double *mu)
{
    for (int d = 0; d < D; d++)
        mu[d] = 0.0;
    for (int n = 0; n < N; n++)
        for (int d = 0; d < D; d++)
            mu[d] += T[(size_t) n * D + d];
    for (int d = 0; d < D; d++)
        mu[d] *= 1.0 / N;
}

/* comm/mpicomm.c:705-730 (dagtm_mpi_sd): sqrt(colsum((T-mu)^2) * (1/(N-1))). */
void orc_sd(int N, int D, const double *T, const double *mu, double *sd)
{
    for (int d = 0; d < D; d++)
        sd[d] = 0.0;
    for (int n = 0; n < N; n++)
        for (int d = 0; d < D; d++) {
            double c = T[(size_t) n * D + d] - mu[d];
            sd[d] += pow(c, 2.0);
        }
    for (int d = 0; d < D; d++)
        sd[d] = sqrt(sd[d] * (1.0 / (N - 1)));
}

/* Cyclic Jacobi eigenvalues of a symmetric n x n matrix (stands in for
 * gsl_eigen_symm, comm/mpicomm.c:540). */
int orc_eig_sym(int n, const double *S, double *lambda)
{
    double *a = (double *) malloc(sizeof(double) * (size_t) n * n);
    memcpy(a, S, sizeof(double) * (size_t) n * n);
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; i++)
            for (int j = 0; j < n; j++) {
                double v = a[(size_t) i * n + j] * a[(size_t) i * n + j];
                tot += v;
                if (i != j)
                    off += v;
            }
        if (off <= DBL_EPSILON * DBL_EPSILON * tot)
            break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++) {
                double apq = a[(size_t) p * n + q];
                if (apq == 0.0)
                    continue;
                double app = a[(size_t) p * n + p], aqq = a[(size_t) q * n + q];
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; k++) {
                    double akp = a[(size_t) k * n + p], akq = a[(size_t) k * n + q];
                    a[(size_t) k * n + p] = c * akp - s * akq;
                    a[(size_t) k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; k++) {
                    double apk = a[(size_t) p * n + k], aqk = a[(size_t) q * n + k];
                    a[(size_t) p * n + k] = c * apk - s * aqk;
                    a[(size_t) q * n + k] = s * apk + c * aqk;
                }
            }
    }
    for (int i = 0; i < n; i++)
        lambda[i] = a[(size_t) i * n + i];
    free(a);
    return 0;
}

/* comm/mpicomm.c:511-559 (dagtm_mpi_ctemp): centre T, S = C^T C, lambda_max/N,
 * beta_T = N D / sum(C^2), ctemp = lambda_max * beta_T. */
double orc_ctemp(int N, int D, const double *T)
{
    double *c = (double *) calloc((size_t) D, sizeof(double));
    for (int n = 0; n < N; n++)
        for (int d = 0; d < D; d++)
            c[d] += T[(size_t) n * D + d];
    for (int d = 0; d < D; d++)
        c[d] *= 1.0 / N;
    double *S = (double *) calloc((size_t) D * D, sizeof(double));
    double csum = 0.0;
    double *row = (double *) malloc(sizeof(double) * (size_t) D);
    for (int n = 0; n < N; n++) {
        for (int d = 0; d < D; d++)
            row[d] = -1.0 * c[d] + T[(size_t) n * D + d];
        for (int i = 0; i < D; i++) {
            double ri = row[i];
            for (int j = 0; j < D; j++)
                S[(size_t) i * D + j] += ri * row[j];
        }
    }
    for (int n = 0; n < N; n++)
        for (int d = 0; d < D; d++) {
            double v = -1.0 * c[d] + T[(size_t) n * D + d];
            csum += pow(v, 2.0);
        }
    double *lam = (double *) malloc(sizeof(double) * (size_t) D);
    orc_eig_sym(D, S, lam);
    double lmax = lam[0];
    for (int d = 1; d < D; d++)
        if (lam[d] > lmax)
            lmax = lam[d];
    lmax /= N;
    double beta = (double) ((size_t) N * (size_t) D) / csum;
    free(c);
    free(S);
    free(row);
    free(lam);
    return lmax * beta;
}

/* comm/mpicomm.c:562-637 (dagtm_mpi_next_ctemp_helper) for every centre, the
 * maximum over centres of comm/mpicomm.c:640-674, and the limit filter of
 * dagtm_vector_max (comm/comm.c:2149-2161).  Written as the reference does it:
 * Xc = T - y_k, rows scaled by sqrt(r) (S1 = 2 Xc^T Xc), scaled again (S12 =
 * -Xc^T Xc), S11 = S1 + S12, H = [[S11, S12], [S12, S11]], eigenvalues of the
 * 2D x 2D H. */
double orc_next_ctemp(int N, int D, int K, const double *T, const double *Y, const double *R,
                      const double *gg, double temp, double beta, double eps)
{
    const double GG_MIN_ = 1e-250;
    double *Xc = (double *) malloc(sizeof(double) * (size_t) N * D);
    double *resp = (double *) malloc(sizeof(double) * (size_t) N);
    double *S1 = (double *) malloc(sizeof(double) * (size_t) D * D);
    double *S12 = (double *) malloc(sizeof(double) * (size_t) D * D);
    double *H = (double *) malloc(sizeof(double) * (size_t) 4 * D * D);
    double *lam = (double *) malloc(sizeof(double) * (size_t) 2 * D);
    double cmax = -HUGE_VAL;
    for (int k = 0; k < K; k++) {
        const double g = gg[k];
        double ck;
        if (g == 0) {
            ck = HUGE_VAL;
        } else {
            for (int n = 0; n < N; n++)
                for (int d = 0; d < D; d++)
                    Xc[(size_t) n * D + d] = T[(size_t) n * D + d] - Y[(size_t) k * D + d];
            for (int n = 0; n < N; n++)
                resp[n] = sqrt(R[(size_t) k * N + n]);
            for (int n = 0; n < N; n++)
                for (int d = 0; d < D; d++)
                    Xc[(size_t) n * D + d] *= resp[n];
            for (int i = 0; i < D; i++)
                for (int j = 0; j < D; j++) {
                    double acc = 0.0;
                    for (int n = 0; n < N; n++)
                        acc += Xc[(size_t) n * D + i] * Xc[(size_t) n * D + j];
                    S1[(size_t) i * D + j] = 2.0 * acc;
                }
            for (int n = 0; n < N; n++)
                for (int d = 0; d < D; d++)
                    Xc[(size_t) n * D + d] *= resp[n];
            for (int i = 0; i < D; i++)
                for (int j = 0; j < D; j++) {
                    double acc = 0.0;
                    for (int n = 0; n < N; n++)
                        acc += Xc[(size_t) n * D + i] * Xc[(size_t) n * D + j];
                    S12[(size_t) i * D + j] = -1.0 * acc;
                }
            const int D2 = 2 * D;
            for (int i = 0; i < D; i++)
                for (int j = 0; j < D; j++) {
                    const double s11 = S1[(size_t) i * D + j] + S12[(size_t) i * D + j];
                    const double s12 = S12[(size_t) i * D + j];
                    H[(size_t) i * D2 + j] = s11;
                    H[(size_t) (D + i) * D2 + D + j] = s11;
                    H[(size_t) i * D2 + D + j] = s12;
                    H[(size_t) (D + i) * D2 + j] = s12;
                }
            if (g < GG_MIN_)
                for (size_t e = 0; e < (size_t) D2 * D2; e++)
                    H[e] *= 1.0 / GG_MIN_;
            orc_eig_sym(D2, H, lam);
            if (g < GG_MIN_)
                for (int i = 0; i < D2; i++)
                    lam[i] *= GG_MIN_;
            const double limit = (temp - eps) * g * 2 / beta;
            double lmax = -HUGE_VAL;
            for (int i = 0; i < D2; i++) {
                if (lam[i] >= limit)
                    lam[i] = 0.0;
                if (lam[i] > lmax)
                    lmax = lam[i];
            }
            ck = beta / 2 / g * lmax;
        }
        if (ck > cmax)
            cmax = ck;
    }
    free(Xc);
    free(resp);
    free(S1);
    free(S12);
    free(H);
    free(lam);
    return cmax;
}

/* ------------------------------------------------------------------ */
/* EM iteration and the annealing loop                                 */
/* ------------------------------------------------------------------ */

static int solve_w(int solver, int M1, int D, const double *A, const double *B, double *W)
{
    if (solver == 1)
        return orc_solve_chol(M1, D, A, B, W) < 0 ? -1 : 0;
    return orc_solve2(M1, D, A, B, W);
}

int orc_em_iteration(int N, int D, int K, int M1, const double *T,
                     const double *FI, double *Y, double *W, double *beta,
                     int isDA, double temp, double *Dm, double *R, double *vgc,
                     double *vgc2, double *llh, double *nfree, int solver)
{
    orc_resp(K, N, *beta, Dm, isDA, temp, R, vgc, vgc2);
    *llh = orc_qual(N, K, D, *beta, vgc, 0, temp);
    if (isDA)
        *nfree = orc_qual(N, K, D, *beta, vgc2, 1, temp);
    else
        *nfree = -*llh;
    double *G = (double *) malloc(sizeof(double) * (size_t) K);
    double *A = (double *) malloc(sizeof(double) * (size_t) M1 * M1);
    double *B = (double *) malloc(sizeof(double) * (size_t) M1 * D);
    orc_mstep_stats(K, N, D, M1, R, FI, T, G, A, B);
    int ret = solve_w(solver, M1, D, A, B, W);
    orc_fiw(K, M1, D, FI, W, Y);
    *beta = orc_beta(K, N, D, Y, T, R, Dm);
    free(G);
    free(A);
    free(B);
    return ret;
}

#define ORC_QUEUE 50 /* dagtm/dagtm.cxx:45 INIT_QUEUE_SIZE */
#define ORC_ABS(a) (((a) > (0)) ? (a) : (-a)) /* comm/comm.h:43 */

int orc_run(int N, int D, int K, int M1, const double *T, const double *FI,
            double *Y, double *W, double *beta_io, double *temp_io, int isDA,
            int schedule, double alpha, double delta, double eps, int iter0,
            int maxloop, int solver, int cap, double *tr_temp,
            double *tr_nfree, double *tr_llh, double *tr_beta, int *n_out,
            double *R_out)
{
    size_t KN = (size_t) K * N;
    double *Dm = (double *) malloc(sizeof(double) * KN);
    double *R = R_out ? R_out : (double *) malloc(sizeof(double) * KN);
    double *vgc = (double *) malloc(sizeof(double) * (size_t) N);
    double *vgc2 = (double *) malloc(sizeof(double) * (size_t) N);
    double *G = (double *) malloc(sizeof(double) * (size_t) K);
    double *A = (double *) malloc(sizeof(double) * (size_t) M1 * M1);
    double *B = (double *) malloc(sizeof(double) * (size_t) M1 * D);
    double queue[ORC_QUEUE];
    int qnext = 0;
    double beta = *beta_io, temp = *temp_io;
    double llh = 0, nfree = 0, qual = 0, qual_old = 0, diff;
    int nloop = iter0, lloop, isLast = 0, ntr = 0, ret = 0;
    if (maxloop)
        maxloop = iter0 + maxloop; /* dagtm/dagtm.cxx:1208-1211 */

    orc_dist(K, N, D, Y, T, Dm); /* dagtm/dagtm.cxx:1232 */
    do {
        if (temp < 1.0) { /* :1510-1514 */
            temp = 1.0;
            isLast = 1;
        }
        for (int i = 0; i < ORC_QUEUE; i++) /* :1521 */
            queue[i] = DBL_MAX;
        qnext = 0;
        lloop = 0;
        while (1) {
            orc_resp(K, N, beta, Dm, isDA, temp, R, vgc, vgc2); /* :1541 */
            qual_old = qual;
            lloop++;
            nloop++;
            if (isDA) { /* :1555-1585 */
                llh = orc_qual(N, K, D, beta, vgc, 0, temp);
                nfree = orc_qual(N, K, D, beta, vgc2, 1, temp);
                qual = nfree;
            } else { /* :1586-1605 */
                llh = orc_qual(N, K, D, beta, vgc, 0, temp);
                nfree = -llh;
                qual = llh;
            }
            diff = qual - qual_old;
            if (ntr < cap) {
                tr_temp[ntr] = temp;
                tr_nfree[ntr] = nfree;
                tr_llh[ntr] = llh;
                tr_beta[ntr] = beta;
            }
            ntr++;
            if (ORC_ABS(diff) < eps) /* :1690-1694 */
                break;
            if (nloop > ORC_QUEUE) { /* :1696-1709 */
                double s0 = 0.0;
                for (int i = 0; i < ORC_QUEUE; i++)
                    s0 += queue[i];
                double avg_old = s0 / ORC_QUEUE;
                queue[qnext] = qual;
                qnext = (qnext + 1) % ORC_QUEUE;
                double s1 = 0.0;
                for (int i = 0; i < ORC_QUEUE; i++)
                    s1 += queue[i];
                double avg = s1 / ORC_QUEUE;
                double diffavg = avg - avg_old;
                if (ORC_ABS(diffavg) < eps)
                    break;
            }
            orc_mstep_stats(K, N, D, M1, R, FI, T, G, A, B); /* :1715-1761 */
            if (solve_w(solver, M1, D, A, B, W) != 0) /* :1767 */
                ret = -1;
            orc_fiw(K, M1, D, FI, W, Y); /* :1769 */
            beta = orc_beta(K, N, D, Y, T, R, Dm); /* :1779 */
            if (maxloop && (nloop >= maxloop)) { /* :1790-1795 */
                isLast = 1;
                break;
            }
        }
        if (isDA && !isLast) { /* :1915-2173, EXP and LINEAR only */
            if (schedule == 1)
                temp -= delta;
            else
                temp *= alpha;
        } else {
            break;
        }
    } while (!isLast);

    *beta_io = beta;
    *temp_io = temp;
    *n_out = ntr;
    free(Dm);
    if (!R_out)
        free(R);
    free(vgc);
    free(vgc2);
    free(G);
    free(A);
    free(B);
    return ret;
}
