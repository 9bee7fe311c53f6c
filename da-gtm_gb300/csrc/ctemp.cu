// ctemp.cu -- the next critical temperature of the AUTO cooling schedule
// (comm/mpicomm.c:562-674, dagtm_mpi_next_ctemp and its helper; the limit
// filter of dagtm_vector_max, comm/comm.c:2149-2161).
//
// For centre k, with x_n = t_n - y_k and R_kn the responsibilities of the last
// E-step, the reference forms
//     S1 = sum_n R_kn x_n x_n^T,  S2 = sum_n R_kn^2 x_n x_n^T,
//     H  = [[2 S1 - S2, -S2], [-S2, 2 S1 - S2]]            (2D x 2D)
// and takes its eigenvalues.  H = [[A, B], [B, A]] is block-diagonalised by the
// orthogonal (1/sqrt 2)[[I, I], [I, -I]], so its spectrum is that of
// A + B = 2 (S1 - S2) together with that of A - B = 2 S1: two D x D symmetric
// problems per centre instead of one of size 2D.  Eigenvalues at or above
// limit_k = (temp - eps) gg_k 2 / beta count as 0 (as dagtm_vector_max sets
// them), the largest remaining value gives ctemp_k = beta / (2 gg_k) lambda.
//
// Centres go in batches; inside a batch the points go in chunks small enough
// that the chunk's data and responsibilities stay in L2:
//   r_block_kernel  : R of the batch's centres over the chunk (FP64, once)
//   scatter_kernel  : one CTA per (centre, 64 x 64 tile of the upper
//                     triangle), 4 x 4 entries of S1 and of S2 per thread,
//                     added over the chunk's points in a fixed order and into
//                     the running sums of the earlier chunks
//   eig_kernel      : one CTA per (centre, block); Householder reduction of
//                     the D x D block to tridiagonal form, then the largest
//                     eigenvalue below the limit by Sturm-count bisection
// Arithmetic type F: FP64 for the FP64 form.  The FP32 and split forms form
// x and the products in FP32 (partial sums over 128 points go into FP64) and
// reduce and bisect in FP32: their stated error is 1e-4, and GB300's FP32
// pipe is about 64 times its FP64 pipe.
#include "common.cuh"
#include "kernels.cuh"

#include <float.h>
#include <math.h>
#include <type_traits>

namespace dgtm {

namespace {

constexpr int SC_THREADS = 256;  // 16 x 16 threads, 4 x 4 entries each
constexpr int SC_TILE = 64;      // output tile (rows x cols of S)
constexpr int SC_PTS = 32;       // points per staged sub-chunk
constexpr int SC_FLUSH = 4;      // FP32 partial sums go into FP64 every 4 sub-chunks
// threads of the eigen kernel: 256 for small matrices (several blocks per SM),
// 512 above that
constexpr int EIG_SMALL_D = 96;
// largest dynamic shared memory a block may opt into on sm_10x (227 KB), less
// room for the kernel's static arrays
constexpr size_t EIG_SMEM_MAX = 232448 - 1024;
constexpr double GG_MIN = 1e-250;  // comm/mpicomm.c:601-612
constexpr size_t ALIGN = 256;

size_t align_up(size_t b) { return (b + ALIGN - 1) / ALIGN * ALIGN; }

// The power of two that brings a centre's largest responsibility into
// [1, 2): FP32 weights keep full precision however small the FP64 ones are
// (a centre far from every point); S1, S2 scale by it, its eigenvalues are
// scaled back.  rmax: the largest R of each centre of the batch as bits (a
// positive double orders as its bit pattern), or null for no scaling.
__device__ __forceinline__ double r_scale(const unsigned long long *rmax, int kl)
{
    if (!rmax)
        return 1.0;
    const double m = __longlong_as_double((long long) rmax[kl]);
    if (!(m > 0.0))
        return 1.0;
    const int e = -ilogb(m);
    return ldexp(1.0, e > 1000 ? 1000 : (e < -1000 ? -1000 : e));
}

// rmax[kl] = max(rmax[kl], the largest R of centre kl over the chunk)
__global__ void r_rowmax_kernel(const double *__restrict__ Rb, int nn,
                                unsigned long long *__restrict__ rmax)
{
    __shared__ double wm[8];
    const int kl = blockIdx.x;
    double m = 0.0;
    for (int p = threadIdx.x; p < nn; p += blockDim.x)
        m = fmax(m, Rb[(size_t) kl * nn + p]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0)
        wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int) (blockDim.x >> 5); w++)
            m = fmax(m, wm[w]);
        m = fmax(m, wm[0]);
        atomicMax(&rmax[kl], (unsigned long long) __double_as_longlong(m));
    }
}

// blockIdx.x = centre in the batch, blockIdx.y = tile pair (ti <= tj).
// Tc: the chunk's points (nn x D, row-major); Rb: kb x nn responsibilities.
// S (per centre: S1 then S2, D x D) holds the entries i <= j only.
template <typename F>
__global__ void __launch_bounds__(SC_THREADS, 2) scatter_kernel(
    const F *__restrict__ Tc, const double *__restrict__ Y, const double *__restrict__ Rb, int nn,
    int D, int k0, int first, double *__restrict__ S, double *__restrict__ gsum,
    const unsigned long long *__restrict__ rmax)
{
    __shared__ __align__(16) F xr[SC_PTS][SC_TILE];
    __shared__ __align__(16) F xc[SC_PTS][SC_TILE];
    __shared__ F yr[SC_TILE], yc[SC_TILE], w1[SC_PTS], w2[SC_PTS];
    const int kl = blockIdx.x, k = k0 + kl;
    int ti = 0, rem = blockIdx.y;
    const int nb = (D + SC_TILE - 1) / SC_TILE;
    while (rem >= nb - ti) {
        rem -= nb - ti;
        ti++;
    }
    const int tj = ti + rem;
    const int i0 = ti * SC_TILE, j0 = tj * SC_TILE;
    const int tr = threadIdx.x >> 4, tc = threadIdx.x & 15;
    const double *yk = Y + (size_t) k * D;
    if (threadIdx.x < SC_TILE) {
        const int d = i0 + threadIdx.x;
        yr[threadIdx.x] = d < D ? (F) yk[d] : F(0);
    } else if (threadIdx.x < 2 * SC_TILE) {
        const int d = j0 + threadIdx.x - SC_TILE;
        yc[threadIdx.x - SC_TILE] = d < D ? (F) yk[d] : F(0);
    }
    constexpr bool F32 = std::is_same<F, float>::value;
    F a1[4][4], a2[4][4];
    double d1[4][4], d2[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            a1[i][j] = a2[i][j] = F(0), d1[i][j] = d2[i][j] = 0.0;
    const double *rk = Rb + (size_t) kl * nn;
    const double rs = r_scale(rmax, kl);  // the weights only; g stays unscaled
    double g = 0.0;  // lanes of warp 0: every 32nd point, summed at the end
    int sub = 0;
    for (int p0 = 0; p0 < nn; p0 += SC_PTS) {
        __syncthreads();
        if (threadIdx.x < SC_PTS) {
            const int p = p0 + threadIdx.x;
            const double r = p < nn ? rk[p] : 0.0;
            g += r;
            const F wf = (F) (r * rs);
            w1[threadIdx.x] = wf;
            w2[threadIdx.x] = wf * wf;
        }
        for (int e = threadIdx.x; e < SC_PTS * SC_TILE; e += SC_THREADS) {
            const int p = e / SC_TILE, j = e % SC_TILE;
            const bool ok = p0 + p < nn;
            const F *tp = Tc + (size_t) (ok ? p0 + p : 0) * D;
            xr[p][j] = (ok && i0 + j < D) ? tp[i0 + j] - yr[j] : F(0);
            xc[p][j] = (ok && j0 + j < D) ? tp[j0 + j] - yc[j] : F(0);
        }
        __syncthreads();
#pragma unroll 4
        for (int p = 0; p < SC_PTS; p++) {
            F a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                a[i] = xr[p][tr * 4 + i];
                b[i] = xc[p][tc * 4 + i];
            }
            const F u = w1[p], v = w2[p];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const F ua = u * a[i], va = v * a[i];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    a1[i][j] = fma(ua, b[j], a1[i][j]);
                    a2[i][j] = fma(va, b[j], a2[i][j]);
                }
            }
        }
        if (F32 && ++sub == SC_FLUSH) {
            sub = 0;
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    d1[i][j] += (double) a1[i][j];
                    d2[i][j] += (double) a2[i][j];
                    a1[i][j] = a2[i][j] = F(0);
                }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            d1[i][j] += (double) a1[i][j];
            d2[i][j] += (double) a2[i][j];
        }
    if (blockIdx.y == 0 && threadIdx.x < 32) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            g += __shfl_down_sync(0xffffffffu, g, o);
        if (threadIdx.x == 0)
            gsum[kl] = first ? g : gsum[kl] + g;
    }
    double *S1 = S + (size_t) kl * 2 * D * D, *S2 = S1 + (size_t) D * D;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int row = i0 + tr * 4 + i;
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int col = j0 + tc * 4 + j;
            if (row < D && col < D && row <= col) {
                const size_t at = (size_t) row * D + col;
                S1[at] = first ? d1[i][j] : S1[at] + d1[i][j];
                S2[at] = first ? d2[i][j] : S2[at] + d2[i][j];
            }
        }
    }
}

template <typename F>
size_t eig_smem_bytes(int D)
{
    // the matrix, then the Householder vector, M v (then w), the diagonal,
    // the off-diagonal and 32 + 2 reduction slots
    return sizeof(F) * ((size_t) D * D + 4 * (size_t) D + 34);
}

template <typename F>
__device__ __forceinline__ F warp_sum(F a)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
}

// sum over the block (every thread gets it); red: NT / 32 slots
template <int NT, typename F>
__device__ __forceinline__ F block_sum(F a, F *red)
{
    a = warp_sum(a);
    if ((threadIdx.x & 31) == 0)
        red[threadIdx.x >> 5] = a;
    __syncthreads();
    F s = F(0);
#pragma unroll
    for (int w = 0; w < NT / 32; w++)
        s += red[w];
    __syncthreads();
    return s;
}

// number of eigenvalues below x of the symmetric tridiagonal matrix with
// diagonal dg and squared off-diagonal od2 (Sturm sequence count; a zero pivot
// is replaced by -pivmin)
template <typename F>
__device__ int count_below(const F *dg, const F *od2, int D, F x, F pivmin)
{
    int c = 0;
    F q = dg[0] - x;
    if (fabs(q) < pivmin)
        q = -pivmin;
    c += q < F(0);
    for (int i = 1; i < D; i++) {
        q = (dg[i] - x) - od2[i - 1] / q;
        if (fabs(q) < pivmin)
            q = -pivmin;
        c += q < F(0);
    }
    return c;
}

// blockIdx.x = centre in the batch, blockIdx.y = 0: 2 S1, 1: 2 (S1 - S2).
// Only the largest eigenvalue below the limit is wanted, so instead of a full
// eigendecomposition the block is reduced to tridiagonal form by Householder
// reflections (Golub and Van Loan, Matrix Computations, algorithm 8.3.1: the
// reduction gsl_eigen_symm starts with too), and that eigenvalue is found by
// bisection on the Sturm sequence count (32-point multisection in one warp).
template <int EIG_THREADS, typename F>
__global__ void __launch_bounds__(EIG_THREADS) eig_kernel(const double *__restrict__ S, int D,
                                                          int in_smem, F *__restrict__ Mg,
                                                          const double *__restrict__ gg,
                                                          double lim_scale, double *__restrict__ out,
                                                          const unsigned long long *__restrict__ rmax)
{
    constexpr int NW = EIG_THREADS / 32;
    extern __shared__ __align__(16) unsigned char sh_raw[];
    F *sh = reinterpret_cast<F *>(sh_raw);
    const int kl = blockIdx.x, which = blockIdx.y;
    F *M = in_smem ? sh : Mg + ((size_t) kl * 2 + which) * D * D;
    F *v = in_smem ? sh + (size_t) D * D : sh;  // Householder vector
    F *p = v + D;                                // tau M v, then w
    F *dg = p + D;                               // diagonal
    F *od = dg + D;                              // off-diagonal, then its squares
    F *red = od + D;                             // reduction slots
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double *S1 = S + (size_t) kl * 2 * D * D, *S2 = S1 + (size_t) D * D;
    const double gk = gg[kl];
    if (gk == 0.0) {
        // the reference returns HUGE_VAL before any eigen work (comm/mpicomm.c:582-585)
        if (threadIdx.x == 0)
            out[(size_t) kl * 2 + which] = 0.0;
        return;
    }
    // gg < GG_MIN: the reference scales H by 1 / GG_MIN before gsl_eigen_symm
    // and the eigenvalues back.  The FP32 arithmetic takes H / gg (1e250 is
    // outside FP32) and multiplies the eigenvalues by gg; H was formed with
    // weights scaled by r_scale, which the matrix scale takes back out.
    double sc = 1.0, back = 1.0;
    if (sizeof(F) == 8) {
        if (gk < GG_MIN)
            sc = 1.0 / GG_MIN, back = GG_MIN;
    } else {
        sc = 1.0 / (gk * r_scale(rmax, kl)), back = gk;
    }
    for (int e = threadIdx.x; e < D * D; e += EIG_THREADS) {
        const int i = e / D, j = e - i * D;
        const size_t at = i <= j ? (size_t) i * D + j : (size_t) j * D + i;
        M[e] = (F) ((which == 0 ? 2.0 * S1[at] : 2.0 * (S1[at] - S2[at])) * sc);
    }
    __syncthreads();
    // column k: x = M[k + 1 .., k] (row k, by symmetry) goes to alpha e_1 by
    // H = I - tau v v^T, v = x - alpha e_1, alpha = -sign(x_0) |x|; the
    // trailing block A becomes H A H = A - v w^T - w v^T, p = tau A v,
    // w = p - (tau / 2)(p^T v) v
    for (int k = 0; k + 2 < D; k++) {
        const int m = D - k - 1;
        const F *x = M + (size_t) k * D + k + 1;
        F part = F(0);
        for (int i = 1 + threadIdx.x; i < m; i += EIG_THREADS)
            part += x[i] * x[i];
        const F sigma = block_sum<EIG_THREADS>(part, red);
        const F x0 = x[0];
        if (threadIdx.x == 0)
            dg[k] = M[(size_t) k * D + k];
        if (sigma == F(0)) {  // the column is already reduced (the same in every thread)
            if (threadIdx.x == 0)
                od[k] = x0;
            continue;
        }
        const F mu = sqrt(x0 * x0 + sigma);
        const F alpha = x0 <= F(0) ? mu : -mu;
        const F v0 = x0 - alpha;  // |v0| = |x0| + mu: no cancellation
        const F tau = F(2) / (v0 * v0 + sigma);
        if (!isfinite(tau)) {  // |x| underflows: the column counts as reduced
            if (threadIdx.x == 0)
                od[k] = x0;
            continue;
        }
        for (int i = threadIdx.x; i < m; i += EIG_THREADS)
            v[i] = i == 0 ? v0 : x[i];
        if (threadIdx.x == 0)
            od[k] = alpha;
        __syncthreads();
        F *A = M + (size_t) (k + 1) * D + (k + 1);
        for (int i = warp; i < m; i += NW) {
            const F *ri = A + (size_t) i * D;
            F acc = F(0);
            for (int j = lane; j < m; j += 32)
                acc += ri[j] * v[j];
            acc = warp_sum(acc);
            if (lane == 0)
                p[i] = tau * acc;
        }
        __syncthreads();
        part = F(0);
        for (int i = threadIdx.x; i < m; i += EIG_THREADS)
            part += p[i] * v[i];
        const F half_k = F(0.5) * tau * block_sum<EIG_THREADS>(part, red);
        for (int i = threadIdx.x; i < m; i += EIG_THREADS)
            p[i] -= half_k * v[i];
        __syncthreads();
        for (int i = warp; i < m; i += NW) {
            F *ri = A + (size_t) i * D;
            const F vi = v[i], wi = p[i];
            for (int j = lane; j < m; j += 32)
                ri[j] -= vi * p[j] + wi * v[j];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (D >= 2) {
            dg[D - 2] = M[(size_t) (D - 2) * D + (D - 2)];
            od[D - 2] = M[(size_t) (D - 2) * D + (D - 1)];
        }
        dg[D - 1] = M[(size_t) (D - 1) * D + (D - 1)];
    }
    __syncthreads();
    if (warp != 0)
        return;
    // Gershgorin bounds and the pivot floor (od becomes od^2)
    F lo = F(INFINITY), hi = F(-INFINITY), emax = F(0);
    for (int i = lane; i < D; i += 32) {
        const F el = i > 0 ? fabs(od[i - 1]) : F(0), er = i + 1 < D ? fabs(od[i]) : F(0);
        lo = fmin(lo, dg[i] - el - er);
        hi = fmax(hi, dg[i] + el + er);
        emax = fmax(emax, er);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
    }
    __syncwarp();
    for (int i = lane; i + 1 < D; i += 32)
        od[i] = od[i] * od[i];
    __syncwarp();
    const F tiny = sizeof(F) == 8 ? (F) DBL_MIN : (F) FLT_MIN;
    const F epsf = sizeof(F) == 8 ? (F) DBL_EPSILON : (F) FLT_EPSILON;
    const F pivmin = tiny * fmax(F(1), emax * emax);
    const double limit = lim_scale * gk;
    const F lim_s = (F) (limit / back);
    // eigenvalues at or above the limit count as 0, then the largest
    const int c = count_below(dg, od, D, lim_s, pivmin);
    double mx = 0.0;
    if (c > 0) {
        // the c-th smallest eigenvalue lies in [lo, min(hi, lim_s)]
        const F pad = epsf * fmax(fabs(lo), fabs(hi)) + pivmin;
        lo -= pad;
        hi = fmin(hi + pad, lim_s);
        for (int it = 0; it < 64 && hi - lo > F(2) * epsf * fmax(fabs(lo), fabs(hi)) + pivmin; it++) {
            const F xl = lo + (hi - lo) * (F) (lane + 1) / F(33);
            const unsigned up = __ballot_sync(0xffffffffu, count_below(dg, od, D, xl, pivmin) >= c);
            // the first point with at least c eigenvalues below it
            const int f = up ? __ffs(up) - 1 : 32;
            const F nlo = f == 0 ? lo : __shfl_sync(0xffffffffu, xl, f - 1 < 0 ? 0 : f - 1);
            const F nhi = f == 32 ? hi : __shfl_sync(0xffffffffu, xl, f == 32 ? 0 : f);
            lo = nlo;
            hi = nhi;
        }
        const double lam = (double) (F(0.5) * (lo + hi)) * back;
        mx = (c < D) ? fmax(lam, 0.0) : lam;
    }
    if (lane == 0)
        out[(size_t) kl * 2 + which] = mx;
}

template <int NT, typename F>
int launch_eig(int kb, int D, bool in_smem, const double *S, F *Mg, const double *gg,
               double lim_scale, double *out, cudaStream_t s,
               const unsigned long long *rmax = nullptr)
{
    const size_t smem = in_smem ? eig_smem_bytes<F>(D)
                                : eig_smem_bytes<F>(D) - sizeof(F) * (size_t) D * D;
    DGTM_CUDA_TRY(cudaFuncSetAttribute(eig_kernel<NT, F>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
    eig_kernel<NT, F><<<dim3(kb, 2), NT, smem, s>>>(S, D, in_smem ? 1 : 0, Mg, gg, lim_scale, out,
                                                    rmax);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

template <typename F>
int run_batch(const CtempPlan &pl, const double *T64, const float *T32, const double *Y,
              const double *tt, const double *yy, const double2 *colstat, int N, int D, int K,
              double c, int k0, int kb, const double *gg_dev, double lim_scale, void *scratch,
              double *gsum_dev, double *out_dev, double dcut, bool scale_r, cudaStream_t s)
{
    unsigned char *base = (unsigned char *) scratch;
    double *S = (double *) base;
    base += align_up(sizeof(double) * (size_t) pl.kb * 2 * D * D);
    F *Mg = nullptr;
    if (!pl.eig_in_smem) {
        Mg = (F *) base;
        base += align_up(sizeof(F) * (size_t) pl.kb * 2 * D * D);
    }
    double *Rb = (double *) base;
    base += align_up(sizeof(double) * (size_t) pl.kb * pl.nn);
    unsigned long long *rmax = (unsigned long long *) base;
    base += align_up(sizeof(unsigned long long) * (size_t) pl.kb);
    float *Tbuf = (float *) base;  // FP32 copy of a chunk when the context has none
    const int ntp = ((D + SC_TILE - 1) / SC_TILE) * ((D + SC_TILE - 1) / SC_TILE + 1) / 2;
    // FP32 weights of centres whose responsibilities may lie below FP32's
    // range: a first pass over the points for each centre's largest R
    const bool scaled = scale_r && !std::is_same<F, double>::value;
    if (scaled) {
        DGTM_CUDA_TRY(cudaMemsetAsync(rmax, 0, sizeof(unsigned long long) * (size_t) kb, s));
        for (int n0 = 0; n0 < N; n0 += pl.nn) {
            const int nn = (N - n0 < pl.nn) ? N - n0 : pl.nn;
            const int r = launch_r_block(T64, Y, tt, yy, colstat, D, K, c, k0, kb, n0, nn, Rb, s,
                                         nullptr, nullptr, dcut);
            if (r != DGTM_OK)
                return r;
            r_rowmax_kernel<<<kb, 256, 0, s>>>(Rb, nn, rmax);
            DGTM_CUDA_TRY(cudaGetLastError());
        }
    } else {
        rmax = nullptr;
    }
    for (int n0 = 0; n0 < N; n0 += pl.nn) {
        const int nn = (N - n0 < pl.nn) ? N - n0 : pl.nn;
        int r = launch_r_block(T64, Y, tt, yy, colstat, D, K, c, k0, kb, n0, nn, Rb, s, nullptr,
                               nullptr, dcut);
        if (r != DGTM_OK)
            return r;
        const F *Tc;
        if constexpr (std::is_same<F, double>::value) {
            Tc = T64 + (size_t) n0 * D;
        } else if (T32) {
            Tc = T32 + (size_t) n0 * D;
        } else {
            r = launch_to_f32(T64 + (size_t) n0 * D, (size_t) nn * D, Tbuf, s);
            if (r != DGTM_OK)
                return r;
            Tc = Tbuf;
        }
        scatter_kernel<F><<<dim3(kb, ntp), SC_THREADS, 0, s>>>(Tc, Y, Rb, nn, D, k0, n0 == 0 ? 1 : 0,
                                                                S, gsum_dev, rmax);
        DGTM_CUDA_TRY(cudaGetLastError());
    }
    const double *gg = gg_dev ? gg_dev : gsum_dev;
    if (D <= EIG_SMALL_D)
        return launch_eig<256, F>(kb, D, pl.eig_in_smem, S, Mg, gg, lim_scale, out_dev, s, rmax);
    return launch_eig<512, F>(kb, D, pl.eig_in_smem, S, Mg, gg, lim_scale, out_dev, s, rmax);
}

}  // namespace

CtempPlan ctemp_plan(int N, int D, int K, bool f32, bool have_t32, size_t budget, int nn_max)
{
    CtempPlan pl;
    pl.f32 = f32;
    pl.nn = N < nn_max ? N : nn_max;
    if (pl.nn < 1)
        pl.nn = 1;
    const size_t fsz = f32 ? sizeof(float) : sizeof(double);
    pl.eig_in_smem = (f32 ? eig_smem_bytes<float>(D) : eig_smem_bytes<double>(D)) <= EIG_SMEM_MAX;
    const size_t dd = (size_t) D * D;
    const size_t per = sizeof(double) * 2 * dd + (pl.eig_in_smem ? 0 : fsz * 2 * dd) +
                       sizeof(double) * (size_t) pl.nn;
    const size_t fixed = (f32 && !have_t32) ? sizeof(float) * (size_t) pl.nn * D : 0;
    size_t kb = budget > fixed + per ? (budget - fixed) / per : 1;
    if (kb > (size_t) K)
        kb = (size_t) K;
    pl.kb = (int) kb;
    pl.scratch_bytes = align_up(sizeof(double) * (size_t) pl.kb * 2 * dd) +
                       (pl.eig_in_smem ? 0 : align_up(fsz * (size_t) pl.kb * 2 * dd)) +
                       align_up(sizeof(double) * (size_t) pl.kb * pl.nn) +
                       align_up(sizeof(unsigned long long) * (size_t) pl.kb) + align_up(fixed) + ALIGN;
    return pl;
}

int launch_ctemp_eig(const CtempPlan &pl, int kb, int D, const double *S, void *Mg,
                     const double *gg, double lim_scale, double *out, cudaStream_t s)
{
    if (pl.f32) {
        float *M = static_cast<float *>(Mg);
        if (D <= EIG_SMALL_D)
            return launch_eig<256, float>(kb, D, pl.eig_in_smem, S, M, gg, lim_scale, out, s);
        return launch_eig<512, float>(kb, D, pl.eig_in_smem, S, M, gg, lim_scale, out, s);
    }
    double *M = static_cast<double *>(Mg);
    if (D <= EIG_SMALL_D)
        return launch_eig<256, double>(kb, D, pl.eig_in_smem, S, M, gg, lim_scale, out, s);
    return launch_eig<512, double>(kb, D, pl.eig_in_smem, S, M, gg, lim_scale, out, s);
}

namespace {

__global__ void gather_centres_kernel(const double *__restrict__ Y, const double *__restrict__ yy,
                                      const double *__restrict__ gg, const int *__restrict__ idx,
                                      int n, int D, double *__restrict__ Ys, double *__restrict__ yys,
                                      double *__restrict__ ggs)
{
    const size_t total = (size_t) n * D;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int r = (int) (i / D), d = (int) (i % D);
        const int k = idx[r];
        Ys[i] = Y[(size_t) k * D + d];
        if (d == 0) {
            yys[r] = yy[k];
            if (gg)
                ggs[r] = gg[k];
        }
    }
}

}  // namespace

int launch_gather_centres(const double *Y, const double *yy, const double *gg, const int *idx,
                          int n, int D, double *Ys, double *yys, double *ggs, cudaStream_t s)
{
    size_t blocks = ((size_t) n * D + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    gather_centres_kernel<<<(unsigned) (blocks ? blocks : 1), 256, 0, s>>>(Y, yy, gg, idx, n, D, Ys,
                                                                          yys, ggs);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int launch_ctemp_batch(const CtempPlan &pl, const double *T64, const float *T32, const double *Y,
                       const double *tt, const double *yy, const double2 *colstat, int N, int D,
                       int K, double c, int k0, int kb, const double *gg_dev, double lim_scale,
                       void *scratch, double *gsum_dev, double *out_dev, double dcut,
                       bool scale_r, cudaStream_t s)
{
    if (pl.f32)
        return run_batch<float>(pl, T64, T32, Y, tt, yy, colstat, N, D, K, c, k0, kb, gg_dev,
                                lim_scale, scratch, gsum_dev, out_dev, dcut, scale_r, s);
    return run_batch<double>(pl, T64, T32, Y, tt, yy, colstat, N, D, K, c, k0, kb, gg_dev,
                             lim_scale, scratch, gsum_dev, out_dev, dcut, false, s);
}

}  // namespace dgtm
