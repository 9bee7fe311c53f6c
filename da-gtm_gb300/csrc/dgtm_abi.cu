// dgtm_abi.cu -- the C ABI: context life cycle and the order of launches of one
// EM iteration.  The host side mirrors the reference's loop body
// (dagtm/dagtm.cxx:1531-1795): E-step -> qualities -> (caller's convergence
// test) -> M-step -> beta; every MPI_Allreduce of comm/mpicomm.c becomes a
// fixed-order on-device reduction and only scalars cross to the host.
#include "common.cuh"
#include "kernels.cuh"
#include "tc.cuh"
#include "x64.cuh"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <utility>
#include <vector>

// Row-block copy.  When both pitches equal the row width the block is
// contiguous and goes through a plain 1D copy: the 2D host-to-device path
// costs several times as long for the same bytes (0.33 ms against 0.06 ms for
// an 8000 x 166 FP64 block on GB300).
static cudaError_t copy_rows(void *dst, size_t dpitch, const void *src, size_t spitch,
                             size_t width, size_t height, cudaMemcpyKind kind, cudaStream_t s)
{
    if (dpitch == width && spitch == width)
        return cudaMemcpyAsync(dst, src, width * height, kind, s);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, width, height, kind, s);
}

namespace dgtm {

static thread_local char g_err[512] = "";

void set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    int n = snprintf(g_err, sizeof(g_err), "[%d] ", code);
    if (n < 0)
        n = 0;
    vsnprintf(g_err + n, sizeof(g_err) - (size_t) n, fmt, ap);
    va_end(ap);
}

}  // namespace dgtm

using namespace dgtm;

struct dgtm_ctx {
    int N, D, K, M1, precision, solver, device, sms;
    cudaStream_t stream;
    // data (device)
    double *T64;       // N x D (all forms: exact distances, norms)
    float *T32;        // N x D (FP32 form)
    double *tt;        // N
    double sum_tt;
    double *FI;        // K x M1
    float2 *FIp;       // K x M1 FP32 (hi, lo) pairs for update_y (FP32 / split forms)
    double *Y64;       // K x D (master copy of the centres)
    double *Yprev;     // K x D: the centres before the last M-step (swapped, not copied)
    double *yyprev;    // K
    float *Y32;        // K x D (FP32 form)
    double *yy;        // K
    double *W;         // M1 x D
    // E-step
    double2 *colstat;  // N
    double *part;      // 2 x nblk1
    int nblk1;
    // M-step
    int nsplit, n_per_split;
    double *Gpart, *RTpart;
    double *G, *RT, *A, *B, *work, *bterm, *abpart;
    double *scal;      // device scalars
    int *flag;         // device status: [0..1] the solver's, [2] update_y's pair counter
    double *hscal;     // pinned host scalars
    int *hflag;
    // split-BF16 form
    TcState *tc;
    // exact-slice FP64 form (0/1 data on sm_10x; otherwise the CUDA-core form)
    XState *x64;
    // phase timers (dgtm_set_timing)
    int timing;
    cudaEvent_t ev[DGTM_NPHASES][2];
    int pending[DGTM_NPHASES];
    double ms[DGTM_NPHASES];
    long long launches[DGTM_NPHASES], calls[DGTM_NPHASES];
    // state
    int stats_valid;   // colstat belongs to the current Y
    int prev_valid;    // colstat belongs to Yprev (an M-step since the last E-step)
    int rt_valid;      // G / RT computed
    int w_valid;
    int dropped;       // pivots dropped by the last Cholesky solve
    double beta, temp;
    int isDA;
};

namespace {

template <typename P>
int dev_alloc(P **p, size_t count)
{
    *p = nullptr;
    if (count == 0)
        count = 1;
    cudaError_t e = cudaMalloc((void **) p, sizeof(P) * count);
    if (e != cudaSuccess) {
        set_error(DGTM_ENOMEM, "cudaMalloc(%zu bytes): %s", sizeof(P) * count,
                  cudaGetErrorString(e));
        *p = nullptr;
        return DGTM_ENOMEM;
    }
    return DGTM_OK;
}

#define DGTM_TRY(expr)              \
    do {                            \
        int _r = (expr);            \
        if (_r != DGTM_OK)          \
            return _r;              \
    } while (0)

// an integer from the environment, or dflt when unset or out of [lo, hi]
int env_int(const char *name, int dflt, int lo, int hi)
{
    const char *v = getenv(name);
    if (!v || !*v)
        return dflt;
    char *end = nullptr;
    const long x = strtol(v, &end, 10);
    if (*end || x < lo || x > hi)
        return dflt;
    return (int) x;
}

int check_ctx(dgtm_ctx *c)
{
    if (!c) {
        set_error(DGTM_EINVAL, "null context");
        return DGTM_EINVAL;
    }
    int dev = -1;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != c->device)
        DGTM_CUDA_TRY(cudaSetDevice(c->device));
    return DGTM_OK;
}

int sync_and_check(dgtm_ctx *c)
{
    DGTM_CUDA_TRY(cudaStreamSynchronize(c->stream));
    for (int p = 0; p < DGTM_NPHASES; p++) {
        if (!c->pending[p])
            continue;
        float t = 0.f;
        DGTM_CUDA_TRY(cudaEventElapsedTime(&t, c->ev[p][0], c->ev[p][1]));
        c->ms[p] += t;
        c->pending[p] = 0;
    }
    return DGTM_OK;
}

int phase_begin(dgtm_ctx *c, int p)
{
    if (c->timing)
        DGTM_CUDA_TRY(cudaEventRecord(c->ev[p][0], c->stream));
    return DGTM_OK;
}

int phase_end(dgtm_ctx *c, int p, int nlaunch)
{
    c->launches[p] += nlaunch;
    c->calls[p] += 1;
    if (c->timing) {
        DGTM_CUDA_TRY(cudaEventRecord(c->ev[p][1], c->stream));
        c->pending[p] = 1;
    }
    return DGTM_OK;
}

// returns the number of kernels launched through *n
int refresh_y_copies(dgtm_ctx *c, int *n)
{
    *n = 0;
    if (c->precision == DGTM_FP32) {
        DGTM_TRY(launch_to_f32(c->Y64, (size_t) c->K * c->D, c->Y32, c->stream));
        *n = 1;
    }
    if (c->precision == DGTM_BF16X3) {
        DGTM_TRY(tc_prepare_y(c->tc, c->Y64, c->stream));
        *n = 1;
    }
    return DGTM_OK;
}

void free_ctx(dgtm_ctx *c)
{
    if (!c)
        return;
    void *ptrs[] = {c->T64, c->T32, c->tt, c->FI, c->FIp, c->Y64, c->Yprev, c->yyprev, c->Y32, c->yy,
                    c->W, c->colstat,
                    c->part, c->Gpart, c->RTpart, c->G, c->RT, c->A, c->B, c->work, c->bterm, c->abpart,
                    c->scal, c->flag};
    for (void *p : ptrs)
        if (p)
            cudaFree(p);
    if (c->hscal)
        cudaFreeHost(c->hscal);
    if (c->hflag)
        cudaFreeHost(c->hflag);
    if (c->tc)
        tc_destroy(c->tc);
    if (c->x64)
        x64_destroy(c->x64);
    for (int p = 0; p < DGTM_NPHASES; p++)
        for (int q = 0; q < 2; q++)
            if (c->ev[p][q])
                cudaEventDestroy(c->ev[p][q]);
    if (c->stream)
        cudaStreamDestroy(c->stream);
    free(c);
}

}  // namespace

extern "C" {

int dgtm_version(void) { return 10000; }

const char *dgtm_last_error_string(void) { return g_err; }

int dgtm_ctx_create(int N, int D, int K, int M1, const double *T, int ldT, const double *FI,
                    int ldFI, int precision, dgtm_ctx **out)
{
    g_err[0] = 0;
    if (!out) {
        set_error(DGTM_EINVAL, "out is null");
        return DGTM_EINVAL;
    }
    *out = nullptr;
    if (N < 1 || D < 1 || K < 1 || M1 < 1 || !T || !FI || ldT < D || ldFI < M1) {
        set_error(DGTM_EINVAL, "bad shape: N=%d D=%d K=%d M1=%d ldT=%d ldFI=%d", N, D, K, M1,
                  ldT, ldFI);
        return DGTM_EINVAL;
    }
    if (precision != DGTM_FP64 && precision != DGTM_FP32 && precision != DGTM_BF16X3) {
        set_error(DGTM_EINVAL, "unknown precision form %d", precision);
        return DGTM_EINVAL;
    }
    if (D > 256) {
        set_error(DGTM_ENOTSUP, "D = %d > 256 is not supported", D);
        return DGTM_ENOTSUP;
    }
    if ((long long) K * D > (1LL << 31) || (long long) N * D > (1LL << 40)) {
        set_error(DGTM_ENOTSUP, "problem too large: N=%d K=%d D=%d", N, K, D);
        return DGTM_ENOTSUP;
    }
    dgtm_ctx *c = (dgtm_ctx *) calloc(1, sizeof(dgtm_ctx));
    if (!c) {
        set_error(DGTM_ENOMEM, "host allocation failed");
        return DGTM_ENOMEM;
    }
    c->N = N;
    c->D = D;
    c->K = K;
    c->M1 = M1;
    c->precision = precision;
    c->solver = DGTM_SOLVE_CHOLESKY;
    int r = DGTM_OK;
#define CK(expr)               \
    do {                       \
        r = (expr);            \
        if (r != DGTM_OK) {    \
            free_ctx(c);       \
            return r;          \
        }                      \
    } while (0)
#define CKC(expr)                                                                       \
    do {                                                                                \
        cudaError_t _e = (expr);                                                        \
        if (_e != cudaSuccess) {                                                        \
            set_error(DGTM_ECUDA, "%s: %s", #expr, cudaGetErrorString(_e));              \
            free_ctx(c);                                                                \
            return DGTM_ECUDA;                                                          \
        }                                                                               \
    } while (0)
    CKC(cudaGetDevice(&c->device));
    CKC(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device));
    CKC(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));

    const size_t ND = (size_t) N * D, KD = (size_t) K * D;
    CK(dev_alloc(&c->T64, ND));
    CK(dev_alloc(&c->tt, N));
    CK(dev_alloc(&c->FI, (size_t) K * M1));
    CK(dev_alloc(&c->Y64, KD));
    CK(dev_alloc(&c->yy, K));
    CK(dev_alloc(&c->Yprev, KD));
    CK(dev_alloc(&c->yyprev, K));
    CK(dev_alloc(&c->W, (size_t) M1 * D));
    CK(dev_alloc(&c->colstat, N));
    CK(dev_alloc(&c->G, K));
    CK(dev_alloc(&c->RT, KD));
    CK(dev_alloc(&c->A, (size_t) M1 * M1));
    CK(dev_alloc(&c->B, (size_t) M1 * D));
    CK(dev_alloc(&c->work, 2 * (size_t) M1 * M1 + (size_t) M1 * D));
    CK(dev_alloc(&c->bterm, K));
    CK(dev_alloc(&c->abpart, form_ab_scratch_doubles(M1, D)));
    CK(dev_alloc(&c->scal, 8));
    CK(dev_alloc(&c->flag, 4));
    CKC(cudaMallocHost((void **) &c->hscal, 8 * sizeof(double)));
    CKC(cudaMallocHost((void **) &c->hflag, 4 * sizeof(int)));

    CKC(copy_rows(c->T64, sizeof(double) * D, T, sizeof(double) * (size_t) ldT,
                          sizeof(double) * D, N, cudaMemcpyHostToDevice, c->stream));
    CKC(copy_rows(c->FI, sizeof(double) * M1, FI, sizeof(double) * (size_t) ldFI,
                          sizeof(double) * M1, K, cudaMemcpyHostToDevice, c->stream));
    if (precision != DGTM_FP64) {
        CK(dev_alloc(&c->FIp, (size_t) K * M1));
        CK(launch_to_pairs(c->FI, (size_t) K * M1, c->FIp, c->stream));
    }
    CK(launch_norms(c->T64, N, D, c->tt, c->stream));
    CK(launch_sum_ratio(c->tt, N, 0.0, 1.0, c->scal, c->stream));
    CKC(cudaMemcpyAsync(c->hscal, c->scal, sizeof(double), cudaMemcpyDeviceToHost, c->stream));

    if (precision == DGTM_FP64 || precision == DGTM_FP32) {
        c->nblk1 = pass1_simt_blocks(N);
        const int kt = pass2_simt_ktiles(K);
        int nsplit = (2 * c->sms + kt - 1) / kt;
        const int max_split = ceil_div(N, 64);
        if (nsplit > max_split)
            nsplit = max_split;
        if (nsplit < 1)
            nsplit = 1;
        c->nsplit = nsplit;
        c->n_per_split = ceil_div(ceil_div(N, nsplit), 64) * 64;
        c->nsplit = ceil_div(N, c->n_per_split);
        if (precision == DGTM_FP64) {
            const int xr = x64_create(&c->x64, N, D, K, c->sms, c->T64, c->stream);
            if (xr != DGTM_ENOTSUP)
                CK(xr);
            if (c->x64)
                c->nblk1 = x64_pass1_blocks(c->x64);
        }
        CK(dev_alloc(&c->part, 2 * (size_t) c->nblk1));
        CK(dev_alloc(&c->Gpart, (size_t) c->nsplit * K));
        CK(dev_alloc(&c->RTpart, (size_t) c->nsplit * KD));
        if (precision == DGTM_FP32) {
            CK(dev_alloc(&c->T32, ND));
            CK(dev_alloc(&c->Y32, KD));
            CK(launch_to_f32(c->T64, ND, c->T32, c->stream));
        }
    } else {
        CK(tc_create(&c->tc, N, D, K, c->sms, c->T64, c->tt, c->stream));
        c->nblk1 = tc_pass1_blocks(c->tc);
        CK(dev_alloc(&c->part, 2 * (size_t) c->nblk1));
    }
    CKC(cudaStreamSynchronize(c->stream));
    c->sum_tt = c->hscal[0];
    *out = c;
    return DGTM_OK;
#undef CK
#undef CKC
}

int dgtm_ctx_destroy(dgtm_ctx *ctx)
{
    if (!ctx)
        return DGTM_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    free_ctx(ctx);
    return DGTM_OK;
}

int dgtm_set_solver(dgtm_ctx *ctx, int solver)
{
    DGTM_TRY(check_ctx(ctx));
    if (solver != DGTM_SOLVE_CHOLESKY && solver != DGTM_SOLVE_SVD) {
        set_error(DGTM_EINVAL, "unknown solver %d", solver);
        return DGTM_EINVAL;
    }
    ctx->solver = solver;
    return DGTM_OK;
}

int dgtm_set_Y(dgtm_ctx *ctx, const double *Y, int ldY)
{
    DGTM_TRY(check_ctx(ctx));
    if (!Y || ldY < ctx->D) {
        set_error(DGTM_EINVAL, "bad Y (ldY=%d, D=%d)", ldY, ctx->D);
        return DGTM_EINVAL;
    }
    DGTM_CUDA_TRY(copy_rows(ctx->Y64, sizeof(double) * ctx->D, Y,
                                    sizeof(double) * (size_t) ldY, sizeof(double) * ctx->D,
                                    ctx->K, cudaMemcpyHostToDevice, ctx->stream));
    DGTM_TRY(launch_norms(ctx->Y64, ctx->K, ctx->D, ctx->yy, ctx->stream));
    int nl = 0;
    DGTM_TRY(refresh_y_copies(ctx, &nl));
    ctx->stats_valid = 0;
    ctx->prev_valid = 0;
    ctx->rt_valid = 0;
    return sync_and_check(ctx);
}

int dgtm_get_Y(dgtm_ctx *ctx, double *Y, int ldY)
{
    DGTM_TRY(check_ctx(ctx));
    if (!Y || ldY < ctx->D) {
        set_error(DGTM_EINVAL, "bad Y (ldY=%d, D=%d)", ldY, ctx->D);
        return DGTM_EINVAL;
    }
    DGTM_CUDA_TRY(copy_rows(Y, sizeof(double) * (size_t) ldY, ctx->Y64,
                                    sizeof(double) * ctx->D, sizeof(double) * ctx->D, ctx->K,
                                    cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

int dgtm_get_W(dgtm_ctx *ctx, double *W, int ldW)
{
    DGTM_TRY(check_ctx(ctx));
    if (!W || ldW < ctx->D) {
        set_error(DGTM_EINVAL, "bad W (ldW=%d, D=%d)", ldW, ctx->D);
        return DGTM_EINVAL;
    }
    if (!ctx->w_valid) {
        set_error(DGTM_ESTATE, "no M-step has run yet");
        return DGTM_ESTATE;
    }
    DGTM_CUDA_TRY(copy_rows(W, sizeof(double) * (size_t) ldW, ctx->W,
                                    sizeof(double) * ctx->D, sizeof(double) * ctx->D, ctx->M1,
                                    cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

int dgtm_estep(dgtm_ctx *ctx, double beta, int isDA, double temp, double *llh, double *nfree)
{
    DGTM_TRY(check_ctx(ctx));
    if (!(beta > 0.0) || !isfinite(beta) || !(temp > 0.0) || !isfinite(temp)) {
        set_error(DGTM_EINVAL, "beta (%g) and temp (%g) must be positive and finite", beta, temp);
        return DGTM_EINVAL;
    }
    isDA = isDA ? 1 : 0;
    const double c1 = beta / 2.0, c2 = beta / (2.0 * temp);
    int r, nl = 1;
    DGTM_TRY(phase_begin(ctx, DGTM_PHASE_ESTEP));
    if (ctx->x64) {
        r = x64_estep(ctx->x64, ctx->Y64, ctx->yy, ctx->tt, c1, c2, isDA, ctx->colstat, ctx->part,
                      ctx->stream, &nl);
    } else if (ctx->precision == DGTM_FP64) {
        Pass1Args<double> a{ctx->T64, ctx->Y64, ctx->tt, ctx->yy, ctx->N, ctx->D, ctx->K,
                            c1, c2, isDA, ctx->colstat, ctx->part};
        r = launch_pass1_simt<double>(a, ctx->stream);
    } else if (ctx->precision == DGTM_FP32) {
        Pass1Args<float> a{ctx->T32, ctx->Y32, ctx->tt, ctx->yy, ctx->N, ctx->D, ctx->K,
                           c1, c2, isDA, ctx->colstat, ctx->part};
        r = launch_pass1_simt<float>(a, ctx->stream);
    } else {
        r = tc_estep(ctx->tc, ctx->Y64, c1, c2, isDA, ctx->colstat, ctx->part, ctx->stream, &nl);
    }
    DGTM_TRY(r);
    DGTM_TRY(phase_end(ctx, DGTM_PHASE_ESTEP, nl));
    DGTM_TRY(phase_begin(ctx, DGTM_PHASE_ESTEP_REDUCE));
    DGTM_TRY(launch_sum_pairs(ctx->part, ctx->nblk1, ctx->scal, ctx->stream));
    DGTM_TRY(phase_end(ctx, DGTM_PHASE_ESTEP_REDUCE, 1));
    DGTM_CUDA_TRY(cudaMemcpyAsync(ctx->hscal, ctx->scal, 2 * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->tc)
        DGTM_TRY(tc_fetch_status(ctx->tc, ctx->stream));
    if (ctx->x64)
        DGTM_TRY(x64_fetch_status(ctx->x64, ctx->stream));
    DGTM_TRY(sync_and_check(ctx));
    if (ctx->tc)
        DGTM_TRY(tc_check_status(ctx->tc));
    if (ctx->x64)
        DGTM_TRY(x64_check_status(ctx->x64));
    const double S1 = ctx->hscal[0], S2 = ctx->hscal[1];
    // comm/mpicomm.c:483-497
    const int N = ctx->N, K = ctx->K, D = ctx->D;
    const double base = N * ((D / 2.0) * log(beta / (2.0 * M_PI)) - log((double) K));
    const double q_llh = (base + S1) / (double) N;
    const double q_free = isDA ? (base + temp * S2) / (double) N : -q_llh;
    if (llh)
        *llh = q_llh;
    if (nfree)
        *nfree = q_free;
    ctx->beta = beta;
    ctx->temp = temp;
    ctx->prev_valid = 0;
    ctx->isDA = isDA;
    ctx->stats_valid = 1;
    ctx->rt_valid = 0;
    return DGTM_OK;
}

int dgtm_mstep(dgtm_ctx *ctx, double *W, int ldW, double *Y, int ldY, double *beta)
{
    DGTM_TRY(check_ctx(ctx));
    if (!ctx->stats_valid) {
        set_error(DGTM_ESTATE, "dgtm_mstep needs an E-step on the current centres first");
        return DGTM_ESTATE;
    }
    if ((W && ldW < ctx->D) || (Y && ldY < ctx->D)) {
        set_error(DGTM_EINVAL, "bad leading dimension (ldW=%d ldY=%d D=%d)", ldW, ldY, ctx->D);
        return DGTM_EINVAL;
    }
    const int N = ctx->N, K = ctx->K, D = ctx->D, M1 = ctx->M1;
    const double c = ctx->isDA ? ctx->beta / (2.0 * ctx->temp) : ctx->beta / 2.0;
    // kernels of the solve phase: form_ab (2), the solver (Cholesky and the
    // substitution, or one eigen kernel), update_y, the beta sum, the reduction
    int npass = 1, nsmall = 4 + solve_launches(M1, ctx->solver);
    DGTM_TRY(phase_begin(ctx, DGTM_PHASE_MSTEP_PASS));
    if (ctx->x64) {
        DGTM_TRY(x64_mstep_pass(ctx->x64, c, ctx->G, ctx->RT, ctx->stream, &npass));  // cut: pass 1
    } else if (ctx->precision == DGTM_FP64) {
        Pass2Args<double> a{ctx->T64, ctx->Y64, ctx->tt, ctx->yy, ctx->colstat, N, D, K, c,
                            ctx->n_per_split, ctx->Gpart, ctx->RTpart, ref_dcut(ctx->beta)};
        DGTM_TRY(launch_pass2_simt<double>(a, ctx->nsplit, ctx->stream));
    } else if (ctx->precision == DGTM_FP32) {
        Pass2Args<float> a{ctx->T32, ctx->Y32, ctx->tt, ctx->yy, ctx->colstat, N, D, K, c,
                           ctx->n_per_split, ctx->Gpart, ctx->RTpart, ref_dcut(ctx->beta)};
        DGTM_TRY(launch_pass2_simt<float>(a, ctx->nsplit, ctx->stream));
    } else {
        DGTM_TRY(tc_mstep_pass(ctx->tc, ctx->colstat, c, ctx->stream, &npass));
    }
    DGTM_TRY(phase_end(ctx, DGTM_PHASE_MSTEP_PASS, npass));
    DGTM_TRY(phase_begin(ctx, DGTM_PHASE_MSTEP_SOLVE));
    if (ctx->precision == DGTM_BF16X3) {
        int nr = 0;
        DGTM_TRY(tc_mstep_reduce(ctx->tc, ctx->G, ctx->RT, ctx->stream, &nr));
        nsmall += nr;
    } else if (!ctx->x64) {
        DGTM_TRY(launch_reduce_slices(ctx->Gpart, ctx->RTpart, ctx->nsplit, K, D, ctx->G,
                                      ctx->RT, ctx->stream));
        nsmall += 1;
    }
    DGTM_TRY(launch_form_ab(ctx->FI, ctx->G, ctx->RT, K, M1, D, ctx->A, ctx->B, ctx->abpart,
                            ctx->stream));
    DGTM_TRY(launch_solve(ctx->A, ctx->B, M1, D, ctx->solver, ctx->W, ctx->work, ctx->flag,
                          ctx->stream));
    // the E-step's copies of the new centres come out of the same kernel
    YCopies cp;
    if (ctx->precision == DGTM_FP32)
        cp.Y32 = ctx->Y32;
    else if (ctx->precision == DGTM_BF16X3)
        tc_y_copies(ctx->tc, &cp);
    // the new centres go to the spare buffers, which then become the current
    // ones: the centres of the last E-step stay on the device (dgtm_map_rd)
    std::swap(ctx->Y64, ctx->Yprev);
    std::swap(ctx->yy, ctx->yyprev);
    // work (the solver's factor, no longer needed once W is out) holds W as
    // FP32 pairs when update_y cannot keep W in shared memory
    int nuy = 1;
    DGTM_TRY(launch_update_y(ctx->FI, ctx->FIp, ctx->W, ctx->G, ctx->RT, K, M1, D, ctx->Y64,
                             ctx->yy, ctx->bterm, cp, ctx->flag + 2, ctx->work,
                             2 * (size_t) M1 * M1 + (size_t) M1 * D, &nuy, ctx->stream));
    nsmall += nuy - 1;
    DGTM_TRY(launch_sum_ratio(ctx->bterm, K, ctx->sum_tt, (double) ((long long) N * D),
                              ctx->scal, ctx->stream));
    DGTM_TRY(phase_end(ctx, DGTM_PHASE_MSTEP_SOLVE, nsmall));
    DGTM_CUDA_TRY(cudaMemcpyAsync(ctx->hscal, ctx->scal, 2 * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    DGTM_CUDA_TRY(cudaMemcpyAsync(ctx->hflag, ctx->flag, 2 * sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    if (W)
        DGTM_CUDA_TRY(copy_rows(W, sizeof(double) * (size_t) ldW, ctx->W,
                                        sizeof(double) * D, sizeof(double) * D, M1,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    if (Y)
        DGTM_CUDA_TRY(copy_rows(Y, sizeof(double) * (size_t) ldY, ctx->Y64,
                                        sizeof(double) * D, sizeof(double) * D, K,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    if (ctx->tc)
        DGTM_TRY(tc_fetch_status(ctx->tc, ctx->stream));
    DGTM_TRY(sync_and_check(ctx));
    if (ctx->tc)
        DGTM_TRY(tc_check_status(ctx->tc));
    ctx->stats_valid = 0;
    ctx->prev_valid = 1;
    ctx->rt_valid = 1;
    ctx->w_valid = 1;
    ctx->dropped = ctx->hflag[1];
    if (ctx->hflag[0] != 0) {
        set_error(ctx->hflag[0], "M-step solve failed: A = FI^T diag(G) FI has non-finite entries");
        return ctx->hflag[0];
    }
    const double b = ctx->hscal[1];
    if (!isfinite(b)) {
        set_error(DGTM_ENONFINITE, "beta update is not finite (sum R o D = %g)", ctx->hscal[0]);
        return DGTM_ENONFINITE;
    }
    if (beta)
        *beta = b;
    return DGTM_OK;
}

int dgtm_get_stats(dgtm_ctx *ctx, double *G, double *RT, int ldRT)
{
    DGTM_TRY(check_ctx(ctx));
    if (!ctx->rt_valid) {
        set_error(DGTM_ESTATE, "no M-step statistics available");
        return DGTM_ESTATE;
    }
    if (RT && ldRT < ctx->D) {
        set_error(DGTM_EINVAL, "bad ldRT %d", ldRT);
        return DGTM_EINVAL;
    }
    if (G)
        DGTM_CUDA_TRY(cudaMemcpyAsync(G, ctx->G, sizeof(double) * ctx->K, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    if (RT)
        DGTM_CUDA_TRY(copy_rows(RT, sizeof(double) * (size_t) ldRT, ctx->RT,
                                        sizeof(double) * ctx->D, sizeof(double) * ctx->D,
                                        ctx->K, cudaMemcpyDeviceToHost, ctx->stream));
    return sync_and_check(ctx);
}

int dgtm_set_timing(dgtm_ctx *ctx, int on)
{
    DGTM_TRY(check_ctx(ctx));
    if (on && !ctx->ev[0][0]) {
        for (int p = 0; p < DGTM_NPHASES; p++)
            for (int q = 0; q < 2; q++)
                DGTM_CUDA_TRY(cudaEventCreate(&ctx->ev[p][q]));
    }
    DGTM_TRY(sync_and_check(ctx));
    ctx->timing = on ? 1 : 0;
    return DGTM_OK;
}

int dgtm_reset_timing(dgtm_ctx *ctx)
{
    DGTM_TRY(check_ctx(ctx));
    DGTM_TRY(sync_and_check(ctx));
    for (int p = 0; p < DGTM_NPHASES; p++) {
        ctx->ms[p] = 0.0;
        ctx->launches[p] = 0;
        ctx->calls[p] = 0;
    }
    return DGTM_OK;
}

int dgtm_get_timing(dgtm_ctx *ctx, double *ms, long long *launches, long long *calls)
{
    DGTM_TRY(check_ctx(ctx));
    DGTM_TRY(sync_and_check(ctx));
    for (int p = 0; p < DGTM_NPHASES; p++) {
        if (ms)
            ms[p] = ctx->ms[p];
        if (launches)
            launches[p] = ctx->launches[p];
        if (calls)
            calls[p] = ctx->calls[p];
    }
    return DGTM_OK;
}

int dgtm_get_stream(dgtm_ctx *ctx, void **stream)
{
    DGTM_TRY(check_ctx(ctx));
    if (!stream) {
        set_error(DGTM_EINVAL, "stream is null");
        return DGTM_EINVAL;
    }
    *stream = (void *) ctx->stream;
    return DGTM_OK;
}

int dgtm_get_path(dgtm_ctx *ctx, int *path)
{
    DGTM_TRY(check_ctx(ctx));
    if (!path) {
        set_error(DGTM_EINVAL, "path is null");
        return DGTM_EINVAL;
    }
    *path = ctx->x64 ? DGTM_PATH_EXACT_SLICES : ctx->tc ? DGTM_PATH_SPLIT_BF16 : DGTM_PATH_CUDA_CORES;
    return DGTM_OK;
}

}  // extern "C"

namespace {

// M = R^T X, or with rd (R o D)^T X: R of the last E-step, which an M-step has
// followed, times the squared distances to the new centres.
int map_impl(dgtm_ctx *ctx, const double *X, int L, double *M, int ldM, bool rd)
{
    DGTM_TRY(check_ctx(ctx));
    if (!rd && !ctx->stats_valid) {
        set_error(DGTM_ESTATE, "dgtm_map needs an E-step on the current centres first");
        return DGTM_ESTATE;
    }
    if (rd && !ctx->prev_valid) {
        set_error(DGTM_ESTATE, "dgtm_map_rd needs an M-step after the last E-step");
        return DGTM_ESTATE;
    }
    if (!X || !M || L < 1 || L > 8 || ldM < L) {
        set_error(DGTM_EINVAL, "bad MAP arguments (L=%d ldM=%d)", L, ldM);
        return DGTM_EINVAL;
    }
    const double c = ctx->isDA ? ctx->beta / (2.0 * ctx->temp) : ctx->beta / 2.0;
    double *dX = nullptr, *dM = nullptr;
    DGTM_TRY(dev_alloc(&dX, (size_t) ctx->K * L));
    int r = dev_alloc(&dM, (size_t) ctx->N * L);
    if (r != DGTM_OK) {
        cudaFree(dX);
        return r;
    }
    r = DGTM_OK;
    cudaError_t e = cudaMemcpyAsync(dX, X, sizeof(double) * ctx->K * L, cudaMemcpyHostToDevice,
                                    ctx->stream);
    if (e == cudaSuccess) {
        if (rd)
            r = launch_map(ctx->T64, ctx->Yprev, ctx->tt, ctx->yyprev, ctx->colstat, ctx->N, ctx->D,
                           ctx->K, c, dX, L, dM, ctx->stream, ctx->Y64, ctx->yy);
        else
            r = launch_map(ctx->T64, ctx->Y64, ctx->tt, ctx->yy, ctx->colstat, ctx->N, ctx->D,
                           ctx->K, c, dX, L, dM, ctx->stream);
        if (r == DGTM_OK)
            e = copy_rows(M, sizeof(double) * (size_t) ldM, dM, sizeof(double) * L,
                                  sizeof(double) * L, ctx->N, cudaMemcpyDeviceToHost,
                                  ctx->stream);
    }
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dX);
    cudaFree(dM);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "dgtm_map: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    return r;
}

int r_block_impl(dgtm_ctx *ctx, int k0, int nk, int n0, int nn, double *R, int ldR, bool rd)
{
    DGTM_TRY(check_ctx(ctx));
    if (!rd && !ctx->stats_valid) {
        set_error(DGTM_ESTATE, "dgtm_get_R_block needs an E-step on the current centres first");
        return DGTM_ESTATE;
    }
    if (rd && !ctx->prev_valid) {
        set_error(DGTM_ESTATE, "dgtm_get_RD_block needs an M-step after the last E-step");
        return DGTM_ESTATE;
    }
    if (!R || k0 < 0 || n0 < 0 || nk < 1 || nn < 1 || k0 + nk > ctx->K || n0 + nn > ctx->N ||
        ldR < nn) {
        set_error(DGTM_EINVAL, "bad R block k0=%d nk=%d n0=%d nn=%d ldR=%d", k0, nk, n0, nn, ldR);
        return DGTM_EINVAL;
    }
    const double c = ctx->isDA ? ctx->beta / (2.0 * ctx->temp) : ctx->beta / 2.0;
    double *dR = nullptr;
    DGTM_TRY(dev_alloc(&dR, (size_t) nk * nn));
    // R_kn = 0 where the reference's exp(-beta d / 2) underflows
    const double dcut = ref_dcut(ctx->beta);
    int r = rd ? launch_r_block(ctx->T64, ctx->Yprev, ctx->tt, ctx->yyprev, ctx->colstat, ctx->D,
                                ctx->K, c, k0, nk, n0, nn, dR, ctx->stream, ctx->Y64, ctx->yy, dcut)
               : launch_r_block(ctx->T64, ctx->Y64, ctx->tt, ctx->yy, ctx->colstat, ctx->D, ctx->K,
                                c, k0, nk, n0, nn, dR, ctx->stream, nullptr, nullptr, dcut);
    cudaError_t e = cudaSuccess;
    if (r == DGTM_OK)
        e = copy_rows(R, sizeof(double) * (size_t) ldR, dR, sizeof(double) * nn,
                              sizeof(double) * nn, nk, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    cudaFree(dR);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "dgtm_get_R_block: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    return r;
}

}  // namespace

extern "C" {

int dgtm_map(dgtm_ctx *ctx, const double *X, int L, double *M, int ldM)
{
    return map_impl(ctx, X, L, M, ldM, false);
}

int dgtm_map_rd(dgtm_ctx *ctx, const double *X, int L, double *M, int ldM)
{
    return map_impl(ctx, X, L, M, ldM, true);
}

int dgtm_get_RD_block(dgtm_ctx *ctx, int k0, int nk, int n0, int nn, double *R, int ldR)
{
    return r_block_impl(ctx, k0, nk, n0, nn, R, ldR, true);
}

int dgtm_next_ctemp(dgtm_ctx *ctx, double temp, double beta, double eps, const double *gg,
                    double *ctemp)
{
    return dgtm_next_ctemp_k(ctx, temp, beta, eps, gg, nullptr, ctemp);
}

int dgtm_next_ctemp_k(dgtm_ctx *ctx, double temp, double beta, double eps, const double *gg,
                      double *ctemp_k, double *ctemp)
{
    DGTM_TRY(check_ctx(ctx));
    if (!ctemp || !(beta > 0.0)) {
        set_error(DGTM_EINVAL, "dgtm_next_ctemp: bad arguments (beta=%g)", beta);
        return DGTM_EINVAL;
    }
    if (!ctx->stats_valid) {
        set_error(DGTM_ESTATE, "dgtm_next_ctemp needs an E-step on the current centres first");
        return DGTM_ESTATE;
    }
    const int N = ctx->N, D = ctx->D, K = ctx->K;
    const double c = ctx->isDA ? ctx->beta / (2.0 * ctx->temp) : ctx->beta / 2.0;
    // eigenvalues at or above (temp - eps) gg 2 / beta are dropped (comm/mpicomm.c:624)
    const double lim_scale = (temp - eps) * 2.0 / beta;
    bool pairs = false;
    if (ctx->precision == DGTM_BF16X3 && ctx->tc && env_int("DGTM_CTEMP_PAIRS", 1, 0, 1)) {
        TcView v;
        tc_view(ctx->tc, &v);
        pairs = v.binary && v.nT == 1;
    }
    // scratch budget and points per chunk: DGTM_CTEMP_SCRATCH_MB (default 256)
    // and DGTM_CTEMP_CHUNK (default 16384) override them; the pair-feature
    // GEMM (split form, 0/1 data) takes DGTM_CTEMP_GEMM_MB (default 8192)
    const size_t budget = (size_t) env_int("DGTM_CTEMP_SCRATCH_MB", 256, 1, 1 << 20) << 20;
    const int nn_max = env_int("DGTM_CTEMP_CHUNK", 16384, 1, 1 << 30);
    const CtempPlan pl = ctemp_plan(N, D, K, ctx->precision != DGTM_FP64, ctx->T32 != nullptr,
                                    budget, nn_max);
    const int kb = pl.kb;
    double *scratch = nullptr, *dgg = nullptr, *dgsum = nullptr, *dout = nullptr;
    std::vector<double> out((size_t) 2 * K), gsum(K);
    int rc = pairs ? DGTM_OK
                   : dev_alloc(&scratch, (pl.scratch_bytes + sizeof(double) - 1) / sizeof(double));
    if (rc == DGTM_OK)
        rc = dev_alloc(&dgsum, K);
    if (rc == DGTM_OK)
        rc = dev_alloc(&dout, (size_t) 2 * K);
    if (rc == DGTM_OK && gg)
        rc = dev_alloc(&dgg, K);
    cudaError_t e = cudaSuccess;
    if (rc == DGTM_OK && gg)
        e = cudaMemcpyAsync(dgg, gg, sizeof(double) * K, cudaMemcpyHostToDevice, ctx->stream);
    // centres redone by the CUDA-core scatter (below), and their results
    std::vector<int> redo;
    std::vector<double> out_sel, gsum_sel;
    const double dcut = ref_dcut(ctx->beta);
    if (pairs && rc == DGTM_OK && e == cudaSuccess) {
        TcView v;
        tc_view(ctx->tc, &v);
        const size_t gbudget = (size_t) env_int("DGTM_CTEMP_GEMM_MB", 8192, 64, 1 << 22) << 20;
        float *ddmin = nullptr;
        std::vector<float> dmin(K);
        rc = dev_alloc(&ddmin, (size_t) v.Kpad);
        if (rc == DGTM_OK)
            rc = tc_ctemp_pairs(v, ctx->Y64, gg ? dgg : nullptr, lim_scale, gbudget, dcut, dgsum, dout,
                                ddmin, ctx->stream);
        if (rc == DGTM_OK)
            rc = tc_fetch_status(ctx->tc, ctx->stream);
        if (rc == DGTM_OK)
            e = cudaMemcpyAsync(gsum.data(), dgsum, sizeof(double) * K, cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (rc == DGTM_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(dmin.data(), ddmin, sizeof(float) * K, cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (rc == DGTM_OK && e == cudaSuccess && (e = cudaStreamSynchronize(ctx->stream)) == cudaSuccess)
            rc = tc_check_status(ctx->tc);
        cudaFree(ddmin);
        // A centre far from every point can have all its responsibilities below
        // the FP32 planes' 2^-126: its scatter there is zero (row sum 0) while
        // the FP64 reference still forms it.  Such centres (row sum below 1e-25:
        // a flushed tail is then 1e-13 of the rest) are redone by the CUDA-core
        // scatter, whose R is FP64, unless every point is beyond the reference's
        // own cut (then its row sum is 0 there too: HUGE_VAL).  FP32 distances
        // carry ~1e-5: centres within 1e-3 of the cut are redone.
        for (int k = 0; rc == DGTM_OK && e == cudaSuccess && k < K; k++)
            if (!(gsum[k] >= 1e-25) && (double) dmin[k] <= dcut * (1.0 + 1e-3))
                redo.push_back(k);
    }
    if (!redo.empty()) {
        // the redone centres packed into one batch (one pass over the points)
        const int ns = (int) redo.size();
        int *didx = nullptr;
        double *Ys = nullptr, *yys = nullptr, *ggs = nullptr, *gs = nullptr, *os = nullptr;
        rc = dev_alloc(&scratch, (pl.scratch_bytes + sizeof(double) - 1) / sizeof(double));
        if (rc == DGTM_OK)
            rc = dev_alloc(&didx, (size_t) ns);
        if (rc == DGTM_OK)
            rc = dev_alloc(&Ys, (size_t) ns * D);
        if (rc == DGTM_OK)
            rc = dev_alloc(&yys, (size_t) ns);
        if (rc == DGTM_OK && gg)
            rc = dev_alloc(&ggs, (size_t) ns);
        if (rc == DGTM_OK)
            rc = dev_alloc(&gs, (size_t) ns);
        if (rc == DGTM_OK)
            rc = dev_alloc(&os, (size_t) 2 * ns);
        if (rc == DGTM_OK)
            e = cudaMemcpyAsync(didx, redo.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, ctx->stream);
        if (rc == DGTM_OK && e == cudaSuccess)
            rc = launch_gather_centres(ctx->Y64, ctx->yy, gg ? dgg : nullptr, didx, ns, D, Ys, yys,
                                       ggs, ctx->stream);
        for (int k0 = 0; rc == DGTM_OK && e == cudaSuccess && k0 < ns; k0 += kb) {
            const int nb = (ns - k0 < kb) ? ns - k0 : kb;
            // these centres' responsibilities can lie below FP32's range: scaled
            rc = launch_ctemp_batch(pl, ctx->T64, ctx->T32, Ys, ctx->tt, yys, ctx->colstat, N, D, K,
                                    c, k0, nb, ggs ? ggs + k0 : nullptr, lim_scale, scratch, gs + k0,
                                    os + (size_t) 2 * k0, dcut, true, ctx->stream);
        }
        out_sel.resize((size_t) 2 * ns);
        gsum_sel.resize((size_t) ns);
        if (rc == DGTM_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(out_sel.data(), os, sizeof(double) * 2 * ns, cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (rc == DGTM_OK && e == cudaSuccess)
            e = cudaMemcpyAsync(gsum_sel.data(), gs, sizeof(double) * ns, cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (rc == DGTM_OK && e == cudaSuccess)
            e = cudaStreamSynchronize(ctx->stream);
        cudaFree(didx);
        cudaFree(Ys);
        cudaFree(yys);
        cudaFree(ggs);
        cudaFree(gs);
        cudaFree(os);
    }
    for (int k0 = 0; !pairs && rc == DGTM_OK && e == cudaSuccess && k0 < K; k0 += kb) {
        const int nb = (K - k0 < kb) ? K - k0 : kb;
        rc = launch_ctemp_batch(pl, ctx->T64, ctx->T32, ctx->Y64, ctx->tt, ctx->yy, ctx->colstat,
                                N, D, K, c, k0, nb, gg ? dgg + k0 : nullptr, lim_scale, scratch,
                                dgsum + k0, dout + (size_t) 2 * k0, dcut, false, ctx->stream);
    }
    if (rc == DGTM_OK && e == cudaSuccess)
        e = cudaMemcpyAsync(out.data(), dout, sizeof(double) * 2 * K, cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (rc == DGTM_OK && e == cudaSuccess)
        e = cudaMemcpyAsync(gsum.data(), dgsum, sizeof(double) * K, cudaMemcpyDeviceToHost,
                            ctx->stream);
    if (rc == DGTM_OK && e == cudaSuccess)
        e = cudaStreamSynchronize(ctx->stream);
    cudaFree(scratch);
    cudaFree(dgsum);
    cudaFree(dout);
    cudaFree(dgg);
    if (rc != DGTM_OK)
        return rc;
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "dgtm_next_ctemp: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    for (size_t i = 0; i < redo.size(); i++) {
        const size_t k = (size_t) redo[i];
        out[2 * k] = out_sel[2 * i];
        out[2 * k + 1] = out_sel[2 * i + 1];
        gsum[k] = gsum_sel[i];
    }
    // comm/mpicomm.c:582-585, 625-627, 664-669
    double cmax = -HUGE_VAL;
    for (int k = 0; k < K; k++) {
        const double g = gg ? gg[k] : gsum[k];
        double ck;
        if (g == 0.0) {
            ck = HUGE_VAL;
        } else {
            const double lmax = out[(size_t) 2 * k] > out[(size_t) 2 * k + 1] ? out[(size_t) 2 * k]
                                                                              : out[(size_t) 2 * k + 1];
            ck = beta / 2 / g * lmax;
        }
        if (ctemp_k)
            ctemp_k[k] = ck;
        if (ck > cmax)
            cmax = ck;
    }
    *ctemp = cmax;
    return DGTM_OK;
}

int dgtm_get_R_block(dgtm_ctx *ctx, int k0, int nk, int n0, int nn, double *R, int ldR)
{
    return r_block_impl(ctx, k0, nk, n0, nn, R, ldR, false);
}

}  // extern "C"
