/*
 * oracle_abi.c -- TEST INFRASTRUCTURE ONLY.  The C ABI of include/dagtm_gb300.h
 * served by the oracle's FP64 routines (oracle/dagtm_oracle.c: dense K x N
 * distances and responsibilities, the reference's semantics), so that the
 * `dagtm` driver's host loop can be run and checked on a machine without a
 * GPU.  The tests link the driver's sources against this file; the product
 * library never contains it.
 *
 * Only the entry points the driver calls are served, with the product's
 * state rules (an M-step, a MAP, a critical temperature or an R block needs
 * an E-step on the current centres; W needs an M-step).  The M-step is the
 * reference's: G, A, B (orc_mstep_stats), the solve, Y = FI W, beta with the
 * new distances (orc_beta), and RT = R T for dgtm_get_stats.
 */
#include "dagtm_gb300.h"
#include "dagtm_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

struct dgtm_ctx {
    int N, D, K, M1, solver, precision;
    double *T, *FI, *Y, *W, *Dm, *R, *Rc, *vgc, *vgc2, *G, *RT, *A, *B;
    int stats_valid, w_valid, rt_valid, rd_valid;
};

static char g_err[256] = "";

static int fail(int code, const char *msg)
{
    snprintf(g_err, sizeof(g_err), "[%d] %s", code, msg);
    return code;
}

int dgtm_version(void) { return 10000; }

const char *dgtm_last_error_string(void) { return g_err; }

static double *alloc(size_t n) { return (double *) calloc(n ? n : 1, sizeof(double)); }

int dgtm_ctx_create(int N, int D, int K, int M1, const double *T, int ldT, const double *FI,
                    int ldFI, int precision, dgtm_ctx **out)
{
    if (!out || N < 1 || D < 1 || K < 1 || M1 < 1 || !T || !FI || ldT < D || ldFI < M1)
        return fail(DGTM_EINVAL, "bad shape");
    dgtm_ctx *c = (dgtm_ctx *) calloc(1, sizeof(dgtm_ctx));
    const size_t KN = (size_t) K * N;
    c->N = N, c->D = D, c->K = K, c->M1 = M1, c->precision = precision;
    c->T = alloc((size_t) N * D), c->FI = alloc((size_t) K * M1), c->Y = alloc((size_t) K * D);
    c->W = alloc((size_t) M1 * D), c->Dm = alloc(KN), c->R = alloc(KN), c->Rc = alloc(KN);
    c->vgc = alloc(N), c->vgc2 = alloc(N), c->G = alloc(K), c->RT = alloc((size_t) K * D);
    c->A = alloc((size_t) M1 * M1), c->B = alloc((size_t) M1 * D);
    for (int n = 0; n < N; n++)
        memcpy(c->T + (size_t) n * D, T + (size_t) n * ldT, sizeof(double) * D);
    for (int k = 0; k < K; k++)
        memcpy(c->FI + (size_t) k * M1, FI + (size_t) k * ldFI, sizeof(double) * M1);
    *out = c;
    return DGTM_OK;
}

int dgtm_ctx_destroy(dgtm_ctx *c)
{
    if (!c)
        return DGTM_OK;
    double *p[] = {c->T, c->FI, c->Y, c->W, c->Dm, c->R, c->Rc, c->vgc, c->vgc2, c->G, c->RT,
                   c->A, c->B};
    for (size_t i = 0; i < sizeof(p) / sizeof(p[0]); i++)
        free(p[i]);
    free(c);
    return DGTM_OK;
}

int dgtm_set_solver(dgtm_ctx *c, int solver)
{
    if (!c || (solver != DGTM_SOLVE_CHOLESKY && solver != DGTM_SOLVE_SVD))
        return fail(DGTM_EINVAL, "unknown solver");
    c->solver = solver;
    return DGTM_OK;
}

int dgtm_set_Y(dgtm_ctx *c, const double *Y, int ldY)
{
    if (!c || !Y || ldY < c->D)
        return fail(DGTM_EINVAL, "bad Y");
    for (int k = 0; k < c->K; k++)
        memcpy(c->Y + (size_t) k * c->D, Y + (size_t) k * ldY, sizeof(double) * c->D);
    orc_dist(c->K, c->N, c->D, c->Y, c->T, c->Dm);
    c->stats_valid = 0;
    c->rt_valid = 0;
    c->rd_valid = 0;
    return DGTM_OK;
}

int dgtm_get_Y(dgtm_ctx *c, double *Y, int ldY)
{
    for (int k = 0; k < c->K; k++)
        memcpy(Y + (size_t) k * ldY, c->Y + (size_t) k * c->D, sizeof(double) * c->D);
    return DGTM_OK;
}

int dgtm_get_W(dgtm_ctx *c, double *W, int ldW)
{
    if (!c->w_valid)
        return fail(DGTM_ESTATE, "no M-step has run yet");
    for (int m = 0; m < c->M1; m++)
        memcpy(W + (size_t) m * ldW, c->W + (size_t) m * c->D, sizeof(double) * c->D);
    return DGTM_OK;
}

int dgtm_estep(dgtm_ctx *c, double beta, int isDA, double temp, double *llh, double *nfree)
{
    if (!c || !(beta > 0.0) || !(temp > 0.0))
        return fail(DGTM_EINVAL, "bad beta or temp");
    orc_resp(c->K, c->N, beta, c->Dm, isDA ? 1 : 0, temp, c->R, c->vgc, c->vgc2);
    memcpy(c->Rc, c->R, sizeof(double) * (size_t) c->K * c->N);
    const double l = orc_qual(c->N, c->K, c->D, beta, c->vgc, 0, temp);
    const double f = isDA ? orc_qual(c->N, c->K, c->D, beta, c->vgc2, 1, temp) : -l;
    if (llh)
        *llh = l;
    if (nfree)
        *nfree = f;
    c->stats_valid = 1;
    c->rt_valid = 0;
    c->rd_valid = 0;
    return DGTM_OK;
}

int dgtm_mstep(dgtm_ctx *c, double *W, int ldW, double *Y, int ldY, double *beta)
{
    if (!c->stats_valid)
        return fail(DGTM_ESTATE, "dgtm_mstep needs an E-step on the current centres first");
    const int N = c->N, D = c->D, K = c->K, M1 = c->M1;
    orc_mstep_stats(K, N, D, M1, c->R, c->FI, c->T, c->G, c->A, c->B);
    for (int k = 0; k < K; k++)
        for (int d = 0; d < D; d++) {
            double s = 0.0;
            for (int n = 0; n < N; n++)
                s += c->R[(size_t) k * N + n] * c->T[(size_t) n * D + d];
            c->RT[(size_t) k * D + d] = s;
        }
    const int r = c->solver == DGTM_SOLVE_SVD ? orc_solve2(M1, D, c->A, c->B, c->W)
                                              : (orc_solve_chol(M1, D, c->A, c->B, c->W) < 0);
    if (r)
        return fail(DGTM_ENOTSPD, "solve failed");
    orc_fiw(K, M1, D, c->FI, c->W, c->Y);
    const double b = orc_beta(K, N, D, c->Y, c->T, c->R, c->Dm);
    if (W)
        for (int m = 0; m < M1; m++)
            memcpy(W + (size_t) m * ldW, c->W + (size_t) m * D, sizeof(double) * D);
    if (Y)
        dgtm_get_Y(c, Y, ldY);
    if (beta)
        *beta = b;
    c->stats_valid = 0;
    c->w_valid = 1;
    c->rt_valid = 1;
    c->rd_valid = 1;  /* orc_beta left R o D in c->R, as dagtm_mpi_beta does */
    return DGTM_OK;
}

int dgtm_get_stats(dgtm_ctx *c, double *G, double *RT, int ldRT)
{
    if (!c->rt_valid)
        return fail(DGTM_ESTATE, "no statistics of the current centres");
    if (G)
        memcpy(G, c->G, sizeof(double) * c->K);
    if (RT)
        for (int k = 0; k < c->K; k++)
            memcpy(RT + (size_t) k * ldRT, c->RT + (size_t) k * c->D, sizeof(double) * c->D);
    return DGTM_OK;
}

int dgtm_map(dgtm_ctx *c, const double *X, int L, double *M, int ldM)
{
    if (!c->stats_valid)
        return fail(DGTM_ESTATE, "dgtm_map needs an E-step on the current centres first");
    for (int n = 0; n < c->N; n++)
        for (int l = 0; l < L; l++) {
            double s = 0.0;
            for (int k = 0; k < c->K; k++)
                s += c->Rc[(size_t) k * c->N + n] * X[(size_t) k * L + l];
            M[(size_t) n * ldM + l] = s;
        }
    return DGTM_OK;
}

int dgtm_map_rd(dgtm_ctx *c, const double *X, int L, double *M, int ldM)
{
    if (!c->rd_valid)
        return fail(DGTM_ESTATE, "dgtm_map_rd needs an M-step after the last E-step");
    for (int n = 0; n < c->N; n++)
        for (int l = 0; l < L; l++) {
            double s = 0.0;
            for (int k = 0; k < c->K; k++)
                s += c->R[(size_t) k * c->N + n] * X[(size_t) k * L + l];
            M[(size_t) n * ldM + l] = s;
        }
    return DGTM_OK;
}

int dgtm_get_RD_block(dgtm_ctx *c, int k0, int nk, int n0, int nn, double *R, int ldR)
{
    if (!c->rd_valid)
        return fail(DGTM_ESTATE, "dgtm_get_RD_block needs an M-step after the last E-step");
    for (int k = 0; k < nk; k++)
        memcpy(R + (size_t) k * ldR, c->R + (size_t) (k0 + k) * c->N + n0, sizeof(double) * nn);
    return DGTM_OK;
}

int dgtm_get_R_block(dgtm_ctx *c, int k0, int nk, int n0, int nn, double *R, int ldR)
{
    if (!c->stats_valid)
        return fail(DGTM_ESTATE, "dgtm_get_R_block needs an E-step on the current centres first");
    for (int k = 0; k < nk; k++)
        memcpy(R + (size_t) k * ldR, c->Rc + (size_t) (k0 + k) * c->N + n0, sizeof(double) * nn);
    return DGTM_OK;
}

int dgtm_next_ctemp_k(dgtm_ctx *c, double temp, double beta, double eps, const double *gg,
                      double *ctemp_k, double *ctemp)
{
    if (!c->stats_valid)
        return fail(DGTM_ESTATE, "dgtm_next_ctemp needs an E-step on the current centres first");
    double cmax = -HUGE_VAL;
    for (int k = 0; k < c->K; k++) {
        const double *Rk = c->Rc + (size_t) k * c->N;
        double g = 0.0;
        if (gg) {
            g = gg[k];
        } else {
            for (int n = 0; n < c->N; n++)
                g += Rk[n];
        }
        const double ck = orc_next_ctemp(c->N, c->D, 1, c->T, c->Y + (size_t) k * c->D, Rk, &g,
                                         temp, beta, eps);
        if (ctemp_k)
            ctemp_k[k] = ck;
        if (ck > cmax)
            cmax = ck;
    }
    *ctemp = cmax;
    return DGTM_OK;
}

int dgtm_next_ctemp(dgtm_ctx *c, double temp, double beta, double eps, const double *gg,
                    double *ctemp)
{
    return dgtm_next_ctemp_k(c, temp, beta, eps, gg, NULL, ctemp);
}
