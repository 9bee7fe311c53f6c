// freeenergy.cu -- the annealed free energy of a GTM and its gradient on
// caller-owned device arrays (FP32 data, FP64 reductions), for autograd.
//
//   F(Y, T, beta, temp) = N (D/2 ln(beta / 2 pi) - ln K)
//                         + temp sum_n ln sum_k exp(-beta d_kn / (2 temp))
// (N times the reference's normalised DA quality, comm/mpicomm.c:463-500).
// With R the tempered responsibilities (columns sum to one):
//   dF/dy_k  = -beta (G_k y_k - (R T)_k)
//   dF/dt_n  = -beta (t_n - sum_k R_kn y_k)
//   dF/dbeta = N D / (2 beta) - 1/2 sum_kn R_kn d_kn
// The backward pass recomputes R tile by tile from the forward's per-point
// statistics (two numbers per point); nothing of size K x N is stored.
//
// On a Blackwell GPU with D <= 189 every contraction runs on the tensor cores
// in the split-BF16 form (Y and T each as two BF16 pieces, FP32 accumulation):
// pass 1 gives the per-point log-sum-exp statistics and F; pass 2 gives G and
// R T for dF/dY and dF/dbeta; pass 3 gives sum_k R_kn y_k for dF/dT.  Other
// shapes use the FP32 CUDA-core kernels of the FP32 form.
#include "common.cuh"
#include "kernels.cuh"
#include "tc.cuh"

#include <math.h>

namespace dgtm {

namespace {

struct FeLayout {
    size_t tt, yy, colstat, part, Gpart, RTpart, G, RT, Cpart, C, bterm, scal, tc, total;
    int nblk1, nsplit_k, n_per_split_k, nsplit_n, k_per_split_n;
    bool use_tc;
    TcFeLayout tcl;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

FeLayout fe_layout(int N, int K, int D, int sms)
{
    FeLayout L{};
    L.use_tc = tc_fe_layout(N, K, D, sms, &L.tcl) == DGTM_OK;
    if (L.use_tc) {
        // tensor-core passes: their operand pieces and slots, plus the
        // per-point statistics, the pass-1 partial sums and G, RT here
        size_t o = 0;
        auto take = [&](size_t bytes) {
            const size_t at = o;
            o += align256(bytes);
            return at;
        };
        L.nblk1 = L.tcl.pass1_blocks;
        L.tt = take(sizeof(double) * N);
        L.yy = take(sizeof(double) * K);
        L.colstat = take(sizeof(double2) * N);
        L.part = take(sizeof(double) * 2 * L.nblk1);
        L.G = take(sizeof(double) * K);
        L.RT = take(sizeof(double) * (size_t) K * D);
        L.bterm = take(sizeof(double) * K);
        L.scal = take(sizeof(double) * 8);
        L.tc = take(L.tcl.total);
        L.total = o;
        return L;
    }
    L.nblk1 = pass1_simt_blocks(N);
    const int kt = pass2_simt_ktiles(K);
    int ns = (2 * sms + kt - 1) / kt;
    const int maxs = (N + 63) / 64;
    ns = ns < 1 ? 1 : (ns > maxs ? maxs : ns);
    L.n_per_split_k = ((N + ns - 1) / ns + 63) / 64 * 64;
    L.nsplit_k = (N + L.n_per_split_k - 1) / L.n_per_split_k;
    const int nt = pass2_simt_ktiles(N);
    int nsn = (2 * sms + nt - 1) / nt;
    const int maxn = (K + 63) / 64;
    nsn = nsn < 1 ? 1 : (nsn > maxn ? maxn : nsn);
    L.k_per_split_n = ((K + nsn - 1) / nsn + 63) / 64 * 64;
    L.nsplit_n = (K + L.k_per_split_n - 1) / L.k_per_split_n;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += align256(bytes);
        return at;
    };
    L.tt = take(sizeof(double) * N);
    L.yy = take(sizeof(double) * K);
    L.colstat = take(sizeof(double2) * N);
    L.part = take(sizeof(double) * 2 * L.nblk1);
    L.Gpart = take(sizeof(double) * (size_t) L.nsplit_k * K);
    L.RTpart = take(sizeof(double) * (size_t) L.nsplit_k * K * D);
    L.G = take(sizeof(double) * K);
    L.RT = take(sizeof(double) * (size_t) K * D);
    L.Cpart = take(sizeof(double) * (size_t) L.nsplit_n * ((size_t) N * D + N));
    L.C = take(sizeof(double) * ((size_t) N * D + N));
    L.bterm = take(sizeof(double) * K);
    L.scal = take(sizeof(double) * 8);
    L.total = o;
    return L;
}

__global__ void norms_f32_kernel(const float *__restrict__ X, int rows, int D,
                                 double *__restrict__ out)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + (threadIdx.x >> 5); r < rows; r += gridDim.x * wpb) {
        double s = 0.0;
        for (int d = lane; d < D; d += 32) {
            const double v = (double) X[(size_t) r * D + d];
            s += v * v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0)
            out[r] = s;
    }
}

// Non-zero when a bounded wait of the tensor-core passes gave up: the
// outputs of the call are then NaN.
__device__ __forceinline__ bool fe_failed(const int *status) { return status && *status != 0; }

// F = base + temp * S2 (S2 = sum of the per-point tempered log-sum-exp terms)
__global__ void fe_value_kernel(const double *__restrict__ S, double base, double temp,
                                const int *__restrict__ status, double *__restrict__ F)
{
    F[0] = fe_failed(status) ? NAN : base + temp * S[1];
}

// bterm_k = G_k |y_k|^2 - 2 y_k . RT_k ; dY = -g beta (G_k y_k - RT_k)
__global__ void fe_dy_kernel(const float *__restrict__ Y, const double *__restrict__ G,
                             const double *__restrict__ RT, const double *__restrict__ yy, int K,
                             int D, double beta, const double *__restrict__ gF,
                             const int *__restrict__ status, float *__restrict__ dY,
                             double *__restrict__ bterm)
{
    const int lane = threadIdx.x & 31, wpb = blockDim.x >> 5;
    const double g = fe_failed(status) ? NAN : (gF ? gF[0] : 1.0);
    for (int k = blockIdx.x * wpb + (threadIdx.x >> 5); k < K; k += gridDim.x * wpb) {
        double yrt = 0.0;
        for (int d = lane; d < D; d += 32) {
            const double y = (double) Y[(size_t) k * D + d], rt = RT[(size_t) k * D + d];
            yrt += y * rt;
            if (dY)
                dY[(size_t) k * D + d] = (float) (-g * beta * (G[k] * y - rt));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            yrt += __shfl_xor_sync(0xffffffffu, yrt, o);
        if (lane == 0)
            bterm[k] = G[k] * yy[k] - 2.0 * yrt;
    }
}

// dT = -g beta (t_n - sum_k R_kn y_k); C FP64 (CUDA-core path) ...
__global__ void fe_dt_kernel(const float *__restrict__ T, const double *__restrict__ C, int N,
                             int D, double beta, const double *__restrict__ gF,
                             float *__restrict__ dT)
{
    const double g = gF ? gF[0] : 1.0;
    const size_t total = (size_t) N * D;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x)
        dT[i] = (float) (-g * beta * ((double) T[i] - C[i]));
}

// ... or FP32 in dT itself (tensor-core path), overwritten in place
__global__ void fe_dt_inplace_kernel(const float *__restrict__ T, int N, int D, double beta,
                                     const double *__restrict__ gF, const int *__restrict__ status,
                                     float *__restrict__ dT)
{
    const float gb = (float) (-(fe_failed(status) ? NAN : (gF ? gF[0] : 1.0)) * beta);
    const size_t total = (size_t) N * D;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x)
        dT[i] = gb * (T[i] - dT[i]);
}

// dbeta = g (N D / (2 beta) - sum R o D / 2), sum R o D = S[0]
__global__ void fe_dbeta_kernel(const double *__restrict__ S, double ND, double beta,
                                const double *__restrict__ gF, const int *__restrict__ status,
                                double *__restrict__ dbeta)
{
    const double g = fe_failed(status) ? NAN : (gF ? gF[0] : 1.0);
    dbeta[0] = g * (ND / (2.0 * beta) - 0.5 * S[0]);
}

int grid_rows(int rows)
{
    int b = (rows + 7) / 8;
    return b > 4864 ? 4864 : (b < 1 ? 1 : b);
}

}  // namespace

int launch_norms_f32(const float *X, int rows, int D, double *out, cudaStream_t s)
{
    norms_f32_kernel<<<grid_rows(rows), 256, 0, s>>>(X, rows, D, out);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

namespace {

int check_args(const float *Y, const float *T, int N, int K, int D, double beta, double temp,
               void *ws, size_t ws_bytes, size_t need)
{
    if (!Y || !T || N < 1 || K < 1 || D < 1 || D > 256) {
        set_error(DGTM_EINVAL, "bad free-energy arguments (N=%d K=%d D=%d)", N, K, D);
        return DGTM_EINVAL;
    }
    if (!(beta > 0.0) || !isfinite(beta) || !(temp > 0.0) || !isfinite(temp)) {
        set_error(DGTM_EINVAL, "beta (%g) and temp (%g) must be positive and finite", beta, temp);
        return DGTM_EINVAL;
    }
    if (!ws || ws_bytes < need) {
        set_error(DGTM_EINVAL, "workspace of %zu bytes is smaller than the %zu needed", ws_bytes,
                  need);
        return DGTM_EINVAL;
    }
    if (((uintptr_t) ws & 255) != 0) {
        set_error(DGTM_EINVAL, "workspace must be 256-byte aligned");
        return DGTM_EINVAL;
    }
    return DGTM_OK;
}

int sm_count()
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 148;
    return sms;
}

#define WS(ptr_t, field) reinterpret_cast<ptr_t>(static_cast<char *>(ws) + L.field)

}  // namespace

}  // namespace dgtm

using namespace dgtm;

extern "C" {

int dgtm_fe_workspace_size(int N, int K, int D, size_t *bytes)
{
    if (!bytes || N < 1 || K < 1 || D < 1) {
        set_error(DGTM_EINVAL, "bad sizes N=%d K=%d D=%d", N, K, D);
        return DGTM_EINVAL;
    }
    *bytes = fe_layout(N, K, D, sm_count()).total;
    return DGTM_OK;
}

int dgtm_fe_forward(const float *Y, const float *T, int N, int K, int D, double beta,
                    double temp, void *ws, size_t ws_bytes, void *stream, double *F)
{
    const int sms = sm_count();
    const FeLayout L = fe_layout(N, K, D, sms);
    int r = check_args(Y, T, N, K, D, beta, temp, ws, ws_bytes, L.total);
    if (r != DGTM_OK)
        return r;
    if (!F) {
        set_error(DGTM_EINVAL, "F is null");
        return DGTM_EINVAL;
    }
    cudaStream_t s = (cudaStream_t) stream;
    double *tt = WS(double *, tt), *yy = WS(double *, yy);
    if ((r = launch_norms_f32(T, N, D, tt, s)) != DGTM_OK ||
        (r = launch_norms_f32(Y, K, D, yy, s)) != DGTM_OK)
        return r;
    const int *status = nullptr;
    if (L.use_tc) {
        void *tcws = static_cast<char *>(ws) + L.tc;
        if ((r = tc_fe_estep(L.tcl, tcws, Y, T, N, K, D, sms, beta / 2.0, beta / (2.0 * temp),
                             WS(double2 *, colstat), WS(double *, part), s)) != DGTM_OK)
            return r;
        status = tc_fe_status(L.tcl, tcws);
    } else {
        Pass1Args<float> a{T, Y, tt, yy, N, D, K, beta / 2.0, beta / (2.0 * temp), 1,
                           WS(double2 *, colstat), WS(double *, part)};
        if ((r = launch_pass1_simt<float>(a, s)) != DGTM_OK)
            return r;
    }
    double *S = WS(double *, scal);
    if ((r = launch_sum_pairs(WS(double *, part), L.nblk1, S, s)) != DGTM_OK)
        return r;
    const double base = N * ((D / 2.0) * log(beta / (2.0 * M_PI)) - log((double) K));
    fe_value_kernel<<<1, 1, 0, s>>>(S, base, temp, status, F);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int dgtm_fe_backward(const float *Y, const float *T, int N, int K, int D, double beta,
                     double temp, void *ws, size_t ws_bytes, void *stream, const double *gF,
                     float *dY, float *dT, double *dbeta)
{
    const int sms = sm_count();
    const FeLayout L = fe_layout(N, K, D, sms);
    int r = check_args(Y, T, N, K, D, beta, temp, ws, ws_bytes, L.total);
    if (r != DGTM_OK)
        return r;
    cudaStream_t s = (cudaStream_t) stream;
    const double c = beta / (2.0 * temp);
    double *tt = WS(double *, tt), *yy = WS(double *, yy), *G = WS(double *, G),
           *RT = WS(double *, RT), *S = WS(double *, scal);
    const double2 *cs = WS(double2 *, colstat);
    void *tcws = L.use_tc ? static_cast<char *>(ws) + L.tc : nullptr;
    const int *status = L.use_tc ? tc_fe_status(L.tcl, tcws) : nullptr;
    if (dY || dbeta) {
        // G, R T: centres own the rows, points are streamed
        if (L.use_tc) {
            if ((r = tc_fe_stats(L.tcl, tcws, N, K, D, sms, G, RT, s)) != DGTM_OK)
                return r;
        } else {
            Pass2Args<float> a{T, Y, tt, yy, cs, N, D, K, c, L.n_per_split_k, WS(double *, Gpart),
                               WS(double *, RTpart)};
            if ((r = launch_pass2_simt<float>(a, L.nsplit_k, s, false)) != DGTM_OK)
                return r;
            if ((r = launch_reduce_slices(WS(double *, Gpart), WS(double *, RTpart), L.nsplit_k, K,
                                          D, G, RT, s)) != DGTM_OK)
                return r;
        }
        fe_dy_kernel<<<grid_rows(K), 256, 0, s>>>(Y, G, RT, yy, K, D, beta, gF, status, dY,
                                                   WS(double *, bterm));
        DGTM_CUDA_TRY(cudaGetLastError());
        if (dbeta) {
            // sum_kn R_kn d_kn = sum_k (G_k |y_k|^2 - 2 y_k.RT_k) + sum_n |t_n|^2
            double *tsum = S + 4;
            if ((r = launch_sum_ratio(tt, N, 0.0, 1.0, tsum, s)) != DGTM_OK)
                return r;
            if ((r = launch_sum_ratio_dev(WS(double *, bterm), K, tsum, S, s)) != DGTM_OK)
                return r;
            fe_dbeta_kernel<<<1, 1, 0, s>>>(S, (double) N * D, beta, gF, status, dbeta);
            DGTM_CUDA_TRY(cudaGetLastError());
        }
    }
    if (dT) {
        const size_t total = (size_t) N * D;
        size_t blocks = (total + 255) / 256;
        if (blocks > 8192)
            blocks = 8192;
        if (L.use_tc) {
            // sum_k R_kn y_k into dT itself, then dT = -g beta (t_n - that)
            if ((r = tc_fe_rty(L.tcl, tcws, N, K, D, sms, dT, s)) != DGTM_OK)
                return r;
            fe_dt_inplace_kernel<<<(unsigned) blocks, 256, 0, s>>>(T, N, D, beta, gF, status, dT);
            DGTM_CUDA_TRY(cudaGetLastError());
            return DGTM_OK;
        }
        // sum_k R_kn y_k: points own the rows (with their statistics), centres streamed
        Pass2Args<float> a{Y, T, yy, tt, cs, K, D, N, c, L.k_per_split_n,
                           WS(double *, Cpart), WS(double *, Cpart) + (size_t) L.nsplit_n * N};
        if ((r = launch_pass2_simt<float>(a, L.nsplit_n, s, true)) != DGTM_OK)
            return r;
        double *C = WS(double *, C);
        if ((r = launch_reduce_slices(WS(double *, Cpart), WS(double *, Cpart) + (size_t) L.nsplit_n * N,
                                      L.nsplit_n, N, D, C + (size_t) N * D, C, s)) != DGTM_OK)
            return r;
        fe_dt_kernel<<<(unsigned) blocks, 256, 0, s>>>(T, C, N, D, beta, gF, dT);
        DGTM_CUDA_TRY(cudaGetLastError());
    }
    return DGTM_OK;
}

}  // extern "C"
