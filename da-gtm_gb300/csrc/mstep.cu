// mstep.cu -- the small FP64 kernels of the M-step, shared by every form.
//
//   reduce_slices : G_k = sum_s Gpart[s][k], RT = sum_s RTpart[s] (fixed order)
//   form_ab       : A = FI^T diag(G) FI, B = FI^T RT     (dagtm/dagtm.cxx:1715-1761),
//                   K-sliced 4 x 4 register tiles, slice partials summed in order
//   solve         : A W = B, FP64 Cholesky (numerically dependent pivots dropped;
//                   one block for M1 <= 110, panels over the GPU above that; one
//                   warp per right-hand side in the substitution)
//                   or symmetric-eigen pseudo-inverse
//                   with exactly-zero eigenvalues dropped (the semantics of
//                   gsl_linalg_SV_solve used by dagtm_solve2, comm/comm.c:1299-1348)
//   update_y      : Y = FI W (dagtm/dagtm.cxx:1769), |y_k|^2, the beta terms, and
//                   the copies of Y the E-step of the FP32 / split form reads
//   sum_ratio     : beta = N D / (sum_k G_k|y_k|^2 - 2 y_k.RT_k + sum_n |t_n|^2)
//                   = N D / sum_kn R_kn |y_k - t_n|^2 (comm/mpicomm.c:276-302
//                   evaluates the same sum over an explicit K x N distance matrix;
//                   every column of R sums to one, which gives the closed form)
//
// Every reduction runs in a fixed order, so repeated runs are bit-identical.
#include "common.cuh"
#include "kernels.cuh"

#include <cuda_bf16.h>

#include <math.h>

namespace dgtm {

__global__ void reduce_slices_kernel(const double *__restrict__ Gpart,
                                     const double *__restrict__ RTpart, int nsplit, int K, int D,
                                     double *__restrict__ G, double *__restrict__ RT)
{
    const size_t KD = (size_t) K * D;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < KD + K;
         i += (size_t) gridDim.x * blockDim.x) {
        double s = 0.0;
        if (i < KD) {
            for (int p = 0; p < nsplit; p++)
                s += RTpart[(size_t) p * KD + i];
            RT[i] = s;
        } else {
            const size_t k = i - KD;
            for (int p = 0; p < nsplit; p++)
                s += Gpart[(size_t) p * K + k];
            G[k] = s;
        }
    }
}

int launch_reduce_slices(const double *Gpart, const double *RTpart, int nsplit, int K, int D,
                         double *G, double *RT, cudaStream_t s)
{
    const size_t n = (size_t) K * D + K;
    int blocks = (int) ((n + 255) / 256);
    if (blocks > 4096)
        blocks = 4096;
    reduce_slices_kernel<<<blocks, 256, 0, s>>>(Gpart, RTpart, nsplit, K, D, G, RT);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

// C = FI^T [RT | diag(G) FI] (M1 x (D + M1)): B = C[:, :D], A = C[:, D:]
// (the upper triangle of A and its diagonal tiles only).
// The K rows are cut into slices; each thread keeps a 4 x 4 FP64 tile of C
// over its slice, fed from shared-memory copies of KC rows of FI and of the
// right operand; the slices' partial tiles are then summed in slice order.
// The FP64 pipe (about 2 FMA per clock per SM on this part) bounds this.
constexpr int AB_THREADS = 256;
constexpr int AB_SLICES = 76;

__global__ void __launch_bounds__(AB_THREADS) form_ab_partial_kernel(
    const double *__restrict__ FI, const double *__restrict__ G, const double *__restrict__ RT,
    int K, int M1, int D, int M1p, int Wp, int kc, int slice_len, double *__restrict__ Cpart)
{
    extern __shared__ double sh[];
    double *FIs = sh;                       // kc x M1p
    double *Rs = sh + (size_t) kc * M1p;    // kc x Wp
    const int W = D + M1;
    const int nct = Wp / 4;
    const int tile = blockIdx.y * AB_THREADS + threadIdx.x;
    const bool in_range = tile < (M1p / 4) * nct;
    const int m0 = in_range ? (tile / nct) * 4 : 0, c0 = in_range ? (tile % nct) * 4 : 0;
    // a tile of A strictly below the diagonal is not formed: the reduction
    // takes A from its upper triangle and mirrors it
    const bool active = in_range && !(c0 >= D && c0 + 3 - D < m0);
    const int kb = blockIdx.x * slice_len, ke = min(K, kb + slice_len);
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            acc[i][j] = 0.0;
    for (int k0 = kb; k0 < ke; k0 += kc) {
        const int nk = min(kc, ke - k0);
        __syncthreads();
        for (int e = threadIdx.x; e < kc * M1p; e += AB_THREADS) {
            const int r = e / M1p, m = e % M1p;
            FIs[e] = (r < nk && m < M1) ? FI[(size_t) (k0 + r) * M1 + m] : 0.0;
        }
        for (int e = threadIdx.x; e < kc * Wp; e += AB_THREADS) {
            const int r = e / Wp, c = e % Wp;
            double v = 0.0;
            if (r < nk) {
                const int k = k0 + r;
                if (c < D)
                    v = RT[(size_t) k * D + c];
                else if (c < W)
                    v = G[k] * FI[(size_t) k * M1 + (c - D)];
            }
            Rs[e] = v;
        }
        __syncthreads();
        if (active) {
            for (int r = 0; r < nk; r++) {
                const double2 a01 = *(const double2 *) &FIs[(size_t) r * M1p + m0];
                const double2 a23 = *(const double2 *) &FIs[(size_t) r * M1p + m0 + 2];
                const double2 b01 = *(const double2 *) &Rs[(size_t) r * Wp + c0];
                const double2 b23 = *(const double2 *) &Rs[(size_t) r * Wp + c0 + 2];
                const double av[4] = {a01.x, a01.y, a23.x, a23.y};
                const double bv[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        acc[i][j] = fma(av[i], bv[j], acc[i][j]);
            }
        }
    }
    if (!active)
        return;
    double *dst = Cpart + (size_t) blockIdx.x * M1 * W;
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++)
            if (m0 + i < M1 && c0 + j < W)
                dst[(size_t) (m0 + i) * W + c0 + j] = acc[i][j];
}

// sum over slices in slice order; A is written from its upper triangle and
// mirrored, so it is exactly symmetric
__global__ void form_ab_reduce_kernel(const double *__restrict__ Cpart, int nslice, int M1, int D,
                                      double *__restrict__ A, double *__restrict__ B)
{
    const int W = D + M1;
    const size_t total = (size_t) M1 * W;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int m = (int) (i / W), c = (int) (i % W);
        if (c >= D && c - D < m)
            continue;
        double sum = 0.0;
        for (int sl = 0; sl < nslice; sl++)
            sum += Cpart[(size_t) sl * total + i];
        if (c < D) {
            B[(size_t) m * D + c] = sum;
        } else {
            const int j = c - D;
            A[(size_t) m * M1 + j] = sum;
            A[(size_t) j * M1 + m] = sum;
        }
    }
}

size_t form_ab_scratch_doubles(int M1, int D) { return (size_t) AB_SLICES * M1 * (D + M1); }

int launch_form_ab(const double *FI, const double *G, const double *RT, int K, int M1, int D,
                   double *A, double *B, double *scratch, cudaStream_t s)
{
    const int M1p = (M1 + 3) / 4 * 4, Wp = (D + M1 + 3) / 4 * 4;
    int kc = (int) ((48 * 1024) / (sizeof(double) * (size_t) (M1p + Wp)));
    if (kc > 16)
        kc = 16;
    if (kc < 1) {
        set_error(DGTM_ENOTSUP, "form_ab: M1 + D too large (%d)", M1 + D);
        return DGTM_ENOTSUP;
    }
    const int slice_len = ceil_div(K, AB_SLICES);
    const int nslice = ceil_div(K, slice_len);
    const int ntiles = (M1p / 4) * (Wp / 4);
    const dim3 grid(nslice, ceil_div(ntiles, AB_THREADS));
    const size_t smem = sizeof(double) * (size_t) kc * (M1p + Wp);
    form_ab_partial_kernel<<<grid, AB_THREADS, smem, s>>>(FI, G, RT, K, M1, D, M1p, Wp, kc,
                                                          slice_len, scratch);
    DGTM_CUDA_TRY(cudaGetLastError());
    const size_t total = (size_t) M1 * (D + M1);
    int blocks = (int) ((total + 255) / 256);
    form_ab_reduce_kernel<<<blocks, 256, 0, s>>>(scratch, nslice, M1, D, A, B);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

// ---------------------------------------------------------------------------
// solvers
// ---------------------------------------------------------------------------
constexpr int SOLVE_THREADS = 512;
constexpr int SMEM_SOLVE_MAX = 110;  // M1 up to which L lives in shared memory
constexpr int TRI_MAXR = 32;  // registers per lane in the substitution: M1 <= 1024

// 1/sqrt(d) for a positive normal d: an FP32 estimate refined by two
// Newton-Raphson steps for f(r) = 1/r^2 - d, r <- r (3 - d r^2) / 2 (each
// step doubles the correct bits: 23 -> 46 -> full FP64).  Outside the FP32
// exponent range the FP64 library square root is used.
__device__ __forceinline__ double rsqrt_nr(double d)
{
    if (!(d > 1e-30 && d < 1e30))
        return 1.0 / sqrt(d);
    double r = (double) rsqrtf((float) d);
#pragma unroll
    for (int it = 0; it < 2; it++)
        r = r * fma(-0.5 * d * r, r, 1.5);
    return r;
}

// Cholesky with pivot drops.  A pivot that keeps less than CHOL_DROP of its
// diagonal (the column adds no new direction at FP64 precision) is dropped:
// its diagonal and column are stored as 0 and that unknown is fixed at 0,
// which keeps the solve defined when A = FI^T diag(G) FI is numerically
// singular (wide basis functions).  L (lower triangle) goes to
// work[0 .. M1*M1), the reciprocal diagonal to work[M1*M1 .. M1*M1 + M1) (0
// for a dropped pivot); flag[1] counts the drops.
constexpr double CHOL_DROP = 1e-12;
constexpr int CHOL_THREADS = 256;

__device__ __forceinline__ void chol_pivot(double *L, const double *adiag, int M1, int j,
                                           double *rinv, int *bad, int *ndrop)
{
    const size_t jj = (size_t) j * M1 + j;
    const double d = L[jj], ajj = adiag[j];
    double r = 0.0;
    if (!isfinite(d)) {
        *bad = 1;
        L[jj] = 0.0;
    } else if (!(d > CHOL_DROP * ajj)) {
        (*ndrop)++;
        L[jj] = 0.0;  // marks a dropped unknown
    } else {
        r = rsqrt_nr(d);
        L[jj] = d * r;
    }
    rinv[j] = r;
}

// Blocked right-looking Cholesky for M1 > SMEM_SOLVE_MAX, in panels of CHB
// columns, so that the O(M1^3) part runs on the whole GPU: chol_panel_kernel
// (one CTA) factorises a panel's columns one after the other over every row
// below them, with chol_pivot's drop rule, and chol_update_kernel (one CTA per
// 32 x 32 tile) subtracts the panel's L21 L21^T from the trailing lower
// triangle.  The layout is that of the shared-memory kernel below: the
// scaled L (L_ij = a_ij / sqrt(d_j)) in the lower
// triangle of work, the reciprocal diagonal after it (0 for a dropped pivot),
// flag[0] for a non-finite pivot and flag[1] counting the drops.
constexpr int CHB = 32;
constexpr int CHB_THREADS = 256;

__global__ void __launch_bounds__(CHB_THREADS) chol_panel_kernel(const double *__restrict__ A,
                                                                 int M1, int p0, int w,
                                                                 double *__restrict__ work,
                                                                 int *flag)
{
    double *L = work;
    double *rinv = work + (size_t) M1 * M1;
    __shared__ double r_sh;
    __shared__ double colj[CHB];  // the scaled column j in the panel's later rows
    __shared__ int bad, ndrop;
    const int tid = threadIdx.x;
    const int kend = p0 + w;
    if (tid == 0) {
        bad = 0;
        ndrop = 0;
    }
    for (int j = p0; j < kend; j++) {
        __syncthreads();
        if (tid == 0) {
            const size_t jj = (size_t) j * M1 + j;
            const double d = L[jj], ajj = A[jj];
            double r = 0.0;
            if (!isfinite(d)) {
                bad = 1;
                L[jj] = 0.0;
            } else if (!(d > CHOL_DROP * ajj)) {
                ndrop++;
                L[jj] = 0.0;  // marks a dropped unknown
            } else {
                r = rsqrt_nr(d);
                L[jj] = d * r;
            }
            rinv[j] = r;
            r_sh = r;
        }
        __syncthreads();
        const double r = r_sh;
        for (int i = j + 1 + tid; i < M1; i += CHB_THREADS)
            L[(size_t) i * M1 + j] *= r;
        __syncthreads();
        if (tid < kend - j - 1)
            colj[tid] = L[(size_t) (j + 1 + tid) * M1 + j];
        __syncthreads();
        // the panel's later columns k (j < k < kend), rows i >= k
        for (int i = j + 1 + tid; i < M1; i += CHB_THREADS) {
            double *Li = L + (size_t) i * M1;
            const double lij = Li[j];
            const int kmax = min(i, kend - 1);
            for (int k = j + 1; k <= kmax; k++)
                Li[k] = fma(-lij, colj[k - j - 1], Li[k]);
        }
    }
    __syncthreads();
    if (tid == 0) {
        if (bad)
            flag[0] = DGTM_ENONFINITE;
        flag[1] += ndrop;
    }
}

// L[i][k] -= sum_q L[i][p0 + q] L[k][p0 + q] over the panel's w columns, for
// i >= k >= p0 + w: tile (ti, tk), tk <= ti, from the block index
__global__ void __launch_bounds__(256) chol_update_kernel(int M1, int p0, int w,
                                                          double *__restrict__ work)
{
    __shared__ double Li[32][CHB + 1], Lk[32][CHB + 1];
    const int t0 = p0 + w;
    int x = blockIdx.x, ti = 0;
    while (x > ti) {
        x -= ti + 1;
        ti++;
    }
    const int tk = x;
    const int i0 = t0 + 32 * ti, k0 = t0 + 32 * tk;
    double *L = work;
    for (int e = threadIdx.x; e < 32 * w; e += 256) {
        const int r = e / w, q = e - (e / w) * w;
        Li[r][q] = (i0 + r < M1) ? L[(size_t) (i0 + r) * M1 + p0 + q] : 0.0;
        Lk[r][q] = (k0 + r < M1) ? L[(size_t) (k0 + r) * M1 + p0 + q] : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x >> 3, c0 = threadIdx.x & 7;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (int q = 0; q < w; q++) {
        const double a = Li[r][q];
#pragma unroll
        for (int m = 0; m < 4; m++)
            acc[m] = fma(a, Lk[c0 + 8 * m][q], acc[m]);
    }
    const int i = i0 + r;
#pragma unroll
    for (int m = 0; m < 4; m++) {
        const int k = k0 + c0 + 8 * m;
        if (i < M1 && k <= i)
            L[(size_t) i * M1 + k] -= acc[m];
    }
}

// The same factorisation with L in shared memory (M1 <= SMEM_SOLVE_MAX),
// balanced over the threads.  The trailing triangle of step j, the (i, k) with
// j < k <= i < M1, is the first n_j (n_j + 1) / 2 entries of a table ordered by
// k, then i, both descending (entry a (a + 1) / 2 + b holds k = M1 - 1 - a,
// i = M1 - 1 - b), so each step's elements spread evenly.  Per column j: the
// scaled column u_i = a_ij r_j goes to a shared vector (and to the free upper
// triangle), then every element takes one FMA, L[i][k] -= u_i u_k.  The next
// pivot (j+1, j+1) is the last entry of step j; its thread walks its entries
// in reverse, so it updates the pivot first and takes its reciprocal square
// root while the other threads work.
__global__ void __launch_bounds__(CHOL_THREADS) cholesky_small_kernel(const double *__restrict__ A,
                                                                     int M1,
                                                                     double *__restrict__ work,
                                                                     int *flag)
{
    extern __shared__ double sh[];
    double *rinv = sh, *adiag = sh + M1, *u = sh + 2 * M1, *L = sh + 3 * M1;
    uint32_t *tab = (uint32_t *) (L + M1 * M1);
    __shared__ int bad, ndrop;
    const int tid = threadIdx.x;
    const int n2 = M1 * M1, npair0 = M1 * (M1 - 1) / 2;
    if (tid == 0) {
        bad = 0;
        ndrop = 0;
    }
#pragma unroll 4
    for (int e = tid; e < n2; e += CHOL_THREADS)
        L[e] = A[e];
    for (int j = tid; j < M1; j += CHOL_THREADS)
        adiag[j] = A[j * M1 + j];
    for (int t = tid; t < npair0; t += CHOL_THREADS) {
        int a = (int) ((sqrtf(8.0f * (float) t + 1.0f) - 1.0f) * 0.5f);
        while ((a + 1) * (a + 2) / 2 <= t)
            a++;
        while (a * (a + 1) / 2 > t)
            a--;
        const int b = t - a * (a + 1) / 2;
        tab[t] = ((uint32_t) (M1 - 1 - b) << 16) | (uint32_t) (M1 - 1 - a);
    }
    __syncthreads();
    if (tid == 0)
        chol_pivot(L, adiag, M1, 0, rinv, &bad, &ndrop);
    for (int j = 0; j < M1; j++) {
        __syncthreads();  // r_j published, step j-1's updates done
        const double rj = rinv[j];
        for (int i = j + 1 + tid; i < M1; i += CHOL_THREADS) {
            const double ui = L[i * M1 + j] * rj;
            u[i] = ui;
            L[j * M1 + i] = ui;
        }
        __syncthreads();
        const int nj = M1 - 1 - j, npair = nj * (nj + 1) / 2;
        if (tid < npair) {
            for (int t = tid + (npair - 1 - tid) / CHOL_THREADS * CHOL_THREADS; t >= tid;
                 t -= CHOL_THREADS) {
                const uint32_t ik = tab[t];
                const int i = (int) (ik >> 16), k = (int) (ik & 0xFFFFu);
                L[i * M1 + k] = fma(-u[i], u[k], L[i * M1 + k]);
                if (t == npair - 1)
                    chol_pivot(L, adiag, M1, j + 1, rinv, &bad, &ndrop);
            }
        }
    }
    __syncthreads();
    for (int e = tid; e < n2; e += CHOL_THREADS) {
        const int i = e / M1, k = e - i * M1;
        if (k < i)
            work[e] = L[k * M1 + i];
        else if (k == i)
            work[e] = L[e];
    }
    for (int j = tid; j < M1; j += CHOL_THREADS)
        work[n2 + j] = rinv[j];
    if (tid == 0) {
        flag[0] = bad ? DGTM_ENONFINITE : 0;
        flag[1] = ndrop;
    }
}

// Forward (L y = b) and back (L^T w = y) substitution, right-looking: one warp
// per right-hand side (column of B), lane l holding entries l, l + 32, ...
// in NR = ceil(M1 / 32) registers; step i broadcasts the finished entry i and
// every lane updates the registers that can still hold later (forward) or
// earlier (back) entries with one FMA each.  Many blocks, so the D columns
// run on many SMs.
constexpr int TRI_WARPS = 4;

template <int NR>
__global__ void __launch_bounds__(TRI_WARPS * 32) tri_solve_kernel(const double *__restrict__ Lg,
                                                                  const double *__restrict__ B,
                                                                  int M1, int D, int l_in_smem,
                                                                  const int *__restrict__ flag,
                                                                  double *__restrict__ W)
{
    extern __shared__ double sh[];
    if (flag[0] != 0)
        return;  // non-finite factorisation: reported by the host
    const double *L = Lg;
    const double *inv = Lg + (size_t) M1 * M1;
    if (l_in_smem) {
        const size_t n = (size_t) M1 * M1 + M1;
#pragma unroll 8
        for (size_t i = threadIdx.x; i < n; i += blockDim.x)
            sh[i] = Lg[i];
        __syncthreads();
        L = sh;
        inv = sh + (size_t) M1 * M1;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = blockIdx.x * TRI_WARPS + warp;
    if (c >= D)
        return;
    double x[NR];
#pragma unroll
    for (int r = 0; r < NR; r++) {
        const int p = lane + 32 * r;
        x[r] = (p < M1) ? B[(size_t) p * D + c] : 0.0;
    }
    // forward: y_i = x_i / L_ii, then x_p -= L_pi y_i for p > i; entry i sits
    // in register rb = i / 32 of lane i % 32, and only registers rb.. hold p > i
#pragma unroll
    for (int rb = 0; rb < NR; rb++) {
        const int iend = min(32, M1 - 32 * rb);
        for (int il = 0; il < iend; il++) {
            const int i = 32 * rb + il;
            const double yi = __shfl_sync(0xffffffffu, x[rb], il) * inv[i];
#pragma unroll
            for (int r = rb; r < NR; r++) {
                const int p = lane + 32 * r;
                if (p == i)
                    x[r] = yi;
                else if (p > i && p < M1)
                    x[r] = fma(-L[(size_t) p * M1 + i], yi, x[r]);
            }
        }
    }
    // back: w_i = y_i / L_ii, then y_p -= L_ip w_i for p < i (registers ..rb)
#pragma unroll
    for (int rb = NR - 1; rb >= 0; rb--) {
        const int iend = min(32, M1 - 32 * rb);
        for (int il = iend - 1; il >= 0; il--) {
            const int i = 32 * rb + il;
            const double wi = __shfl_sync(0xffffffffu, x[rb], il) * inv[i];
#pragma unroll
            for (int r = 0; r <= rb; r++) {
                const int p = lane + 32 * r;
                if (p == i)
                    x[r] = wi;
                else if (p < i)
                    x[r] = fma(-L[(size_t) i * M1 + p], wi, x[r]);
            }
        }
    }
#pragma unroll
    for (int r = 0; r < NR; r++) {
        const int p = lane + 32 * r;
        if (p < M1)
            W[(size_t) p * D + c] = x[r];
    }
}

using TriKernel = void (*)(const double *, const double *, int, int, int, const int *, double *);

// exact register counts up to 8, then buckets (the registers past M1 hold 0
// and take no steps)
TriKernel tri_solve_for(int nr)
{
    switch (nr) {
    case 1: return tri_solve_kernel<1>;
    case 2: return tri_solve_kernel<2>;
    case 3: return tri_solve_kernel<3>;
    case 4: return tri_solve_kernel<4>;
    case 5: return tri_solve_kernel<5>;
    case 6: return tri_solve_kernel<6>;
    case 7: return tri_solve_kernel<7>;
    case 8: return tri_solve_kernel<8>;
    default:
        return nr <= 12 ? tri_solve_kernel<12>
                        : nr <= 16 ? tri_solve_kernel<16>
                                   : nr <= 24 ? tri_solve_kernel<24> : tri_solve_kernel<32>;
    }
}

// Parallel cyclic Jacobi (round-robin pairing) on the symmetric A, then
// W = V diag(1/lambda, 0 where lambda == 0) V^T B.
__global__ void __launch_bounds__(SOLVE_THREADS) jacobi_solve_kernel(const double *__restrict__ A,
                                                                    const double *__restrict__ B,
                                                                    int M1, int D,
                                                                    double *__restrict__ W,
                                                                    double *__restrict__ work,
                                                                    int *flag)
{
    double *S = work;                        // M1 x M1 (becomes diagonal)
    double *V = work + (size_t) M1 * M1;     // M1 x M1 eigenvectors (columns)
    double *tmp = V + (size_t) M1 * M1;      // M1 x D
    __shared__ double cs[SOLVE_THREADS], sn[SOLVE_THREADS];
    __shared__ int pp[SOLVE_THREADS], qq[SOLVE_THREADS];
    __shared__ double red[32];
    __shared__ int done;
    const int n = M1 + (M1 & 1);  // even number of slots; slot M1 (if any) is a dummy
    for (int i = threadIdx.x; i < M1 * M1; i += blockDim.x) {
        S[i] = A[i];
        V[i] = ((i / M1) == (i % M1)) ? 1.0 : 0.0;
    }
    __syncthreads();
    for (int sweep = 0; sweep < 60; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int i = threadIdx.x; i < M1 * M1; i += blockDim.x) {
            const double v = S[i] * S[i];
            tot += v;
            if ((i / M1) != (i % M1))
                off += v;
        }
        off = block_sum_fixed(off, red);
        tot = block_sum_fixed(tot, red);
        if (threadIdx.x == 0)
            done = (off <= 1e-32 * tot);
        __syncthreads();
        if (done)
            break;
        for (int r = 0; r < n - 1; r++) {
            // round-robin: slot 0 fixed, the others rotate
            for (int t = threadIdx.x; t < n / 2; t += blockDim.x) {
                int a = (t == 0) ? 0 : 1 + ((t - 1 + r) % (n - 1));
                int b = 1 + ((n - 2 - t + r) % (n - 1));
                int p = min(a, b), q = max(a, b);
                double c = 1.0, s = 0.0;
                if (q < M1) {
                    const double apq = S[(size_t) p * M1 + q];
                    if (apq != 0.0) {
                        const double app = S[(size_t) p * M1 + p], aqq = S[(size_t) q * M1 + q];
                        const double th = (aqq - app) / (2.0 * apq);
                        const double tt = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                        c = 1.0 / sqrt(tt * tt + 1.0);
                        s = tt * c;
                    }
                }
                pp[t] = p;
                qq[t] = q;
                cs[t] = c;
                sn[t] = s;
            }
            __syncthreads();
            // rows: S <- J^T S
            for (int idx = threadIdx.x; idx < (n / 2) * M1; idx += blockDim.x) {
                const int t = idx / M1, k = idx % M1;
                const int p = pp[t], q = qq[t];
                if (q >= M1 || sn[t] == 0.0)
                    continue;
                const double c = cs[t], s = sn[t];
                const double sp = S[(size_t) p * M1 + k], sq = S[(size_t) q * M1 + k];
                S[(size_t) p * M1 + k] = c * sp - s * sq;
                S[(size_t) q * M1 + k] = s * sp + c * sq;
            }
            __syncthreads();
            // columns: S <- S J, V <- V J
            for (int idx = threadIdx.x; idx < (n / 2) * M1; idx += blockDim.x) {
                const int t = idx / M1, k = idx % M1;
                const int p = pp[t], q = qq[t];
                if (q >= M1 || sn[t] == 0.0)
                    continue;
                const double c = cs[t], s = sn[t];
                const double sp = S[(size_t) k * M1 + p], sq = S[(size_t) k * M1 + q];
                S[(size_t) k * M1 + p] = c * sp - s * sq;
                S[(size_t) k * M1 + q] = s * sp + c * sq;
                const double vp = V[(size_t) k * M1 + p], vq = V[(size_t) k * M1 + q];
                V[(size_t) k * M1 + p] = c * vp - s * vq;
                V[(size_t) k * M1 + q] = s * vp + c * vq;
            }
            __syncthreads();
        }
    }
    // tmp = diag(1/lambda) V^T B
    for (int idx = threadIdx.x; idx < M1 * D; idx += blockDim.x) {
        const int i = idx / D, c = idx % D;
        double acc = 0.0;
        for (int r = 0; r < M1; r++)
            acc += V[(size_t) r * M1 + i] * B[(size_t) r * D + c];
        double lam = S[(size_t) i * M1 + i];
        if (lam != 0.0)
            lam = 1.0 / lam;
        tmp[idx] = lam * acc;
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < M1 * D; idx += blockDim.x) {
        const int r = idx / D, c = idx % D;
        double acc = 0.0;
        for (int i = 0; i < M1; i++)
            acc += V[(size_t) r * M1 + i] * tmp[(size_t) i * D + c];
        W[idx] = acc;
    }
    if (threadIdx.x == 0)
        flag[0] = 0;
}

int solve_launches(int M1, int solver)
{
    if (solver == DGTM_SOLVE_SVD)
        return 1;
    if (M1 <= SMEM_SOLVE_MAX)
        return 2;
    // np panels, np - 1 trailing updates (none after the last), the substitution
    const int np = ceil_div(M1, CHB);
    return np + (np - 1) + 1;
}

int launch_solve(const double *A, const double *B, int M1, int D, int solver, double *W,
                 double *work, int *flag, cudaStream_t s)
{
    DGTM_CUDA_TRY(cudaMemsetAsync(flag, 0, 2 * sizeof(int), s));
    if (solver != DGTM_SOLVE_SVD && M1 > 32 * TRI_MAXR) {
        set_error(DGTM_ENOTSUP, "the Cholesky solver supports M1 <= %d", 32 * TRI_MAXR);
        return DGTM_ENOTSUP;
    }
    if (solver == DGTM_SOLVE_SVD && M1 > 2 * SOLVE_THREADS - 2) {
        set_error(DGTM_ENOTSUP, "the eigen-SVD solver supports M1 <= %d", 2 * SOLVE_THREADS - 2);
        return DGTM_ENOTSUP;
    }
    if (solver == DGTM_SOLVE_SVD) {
        jacobi_solve_kernel<<<1, SOLVE_THREADS, 0, s>>>(A, B, M1, D, W, work, flag);
    } else {
        if (M1 <= SMEM_SOLVE_MAX) {
            const size_t smem = sizeof(double) * (3 * (size_t) M1 + (size_t) M1 * M1) +
                                sizeof(uint32_t) * ((size_t) M1 * (M1 - 1) / 2);
            DGTM_CUDA_TRY(cudaFuncSetAttribute(cholesky_small_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int) smem));
            cholesky_small_kernel<<<1, CHOL_THREADS, smem, s>>>(A, M1, work, flag);
        } else {
            DGTM_CUDA_TRY(cudaMemcpyAsync(work, A, sizeof(double) * (size_t) M1 * M1,
                                          cudaMemcpyDeviceToDevice, s));
            for (int p0 = 0; p0 < M1; p0 += CHB) {
                const int w = M1 - p0 < CHB ? M1 - p0 : CHB;
                chol_panel_kernel<<<1, CHB_THREADS, 0, s>>>(A, M1, p0, w, work, flag);
                const int nt = ceil_div(M1 - p0 - w, 32);
                if (nt > 0)
                    chol_update_kernel<<<nt * (nt + 1) / 2, 256, 0, s>>>(M1, p0, w, work);
            }
        }
        DGTM_CUDA_TRY(cudaGetLastError());
        const size_t lbytes = sizeof(double) * ((size_t) M1 * M1 + M1);
        const int l_in_smem = lbytes <= 96 * 1024;
        const size_t tsmem = l_in_smem ? lbytes : 16;
        const TriKernel tri = tri_solve_for(ceil_div(M1, 32));
        DGTM_CUDA_TRY(cudaFuncSetAttribute(tri, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int) tsmem));
        tri<<<ceil_div(D, TRI_WARPS), TRI_WARPS * 32, tsmem, s>>>(work, B, M1, D, l_in_smem, flag, W);
    }
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

// ---------------------------------------------------------------------------
// Y = FI W, the per-centre terms of beta and the E-step's copies of Y
// ---------------------------------------------------------------------------
// A warp computes two centres over all depths: lane l owns depths l + 32 c,
// c < NC (passes of 32 NC depths when D > 256).  Per basis function it loads
// the two FI values once (broadcast) and W[m][l + 32 c] from shared memory,
// where W is padded with zeros to whole passes so the loop has no guards.
// Each warp takes the next centre pair from a counter (*ticket, zero at
// launch), so the pairs spread evenly over the SM sub-partitions whatever the
// CTA placement.  The warp sums |y|^2, y.RT and, for the split form,
// |y_hi + y_lo|^2 of each centre by lane partials and shuffles in a fixed
// order (FP64).
//
// Two arithmetics.  DF = false (the FP64 form): 2 NC FP64 accumulators per
// lane; the FP64 pipe (about 2 FMA per clock per SM) bounds the kernel.
// DF = true (the FP32 and split-BF16 forms): FI and W as unevaluated sums of
// two FP32 (hi + lo, 48 bits) and each product accumulated by Dot2 of Ogita,
// Rump and Oishi ("Accurate sum and dot product", SIAM J. Sci. Comput. 26,
// 2005): the high parts' product split exactly by an FMA, the cross terms
// added to its error, the running sum kept exact by Knuth's TwoSum.  The
// result is as accurate as a product in twice FP32's precision (~1e-14
// relative), far inside those forms' 1e-4, on the FP32 pipe, which is 64
// times as wide as the FP64 one.
constexpr int UY_THREADS = 256;
constexpr int UY_NCMAX = 8;
constexpr size_t UY_WSMEM_MAX = 110 * 1024;  // two CTAs per SM

__device__ __forceinline__ double uy_warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// p + s += (a.x + a.y) (w.x + w.y); the _rn intrinsics keep each rounding
// where Dot2 needs it (no contraction into an FMA)
__device__ __forceinline__ void dot2_step(float &p, float &s, float2 a, float2 w)
{
    const float h = __fmul_rn(a.x, w.x);
    float r = fmaf(a.x, w.x, -h);
    r = fmaf(a.x, w.y, r);
    r = fmaf(a.y, w.x, r);
    const float t = __fadd_rn(p, h);
    const float z = __fsub_rn(t, p);
    const float q = __fadd_rn(__fsub_rn(p, __fsub_rn(t, z)), __fsub_rn(h, z));
    p = t;
    s = __fadd_rn(s, __fadd_rn(q, r));
}

__device__ __forceinline__ float2 f64_to_pair(double x)
{
    const float hi = (float) x;
    return make_float2(hi, (float) (x - (double) hi));
}

__global__ void to_pairs_kernel(const double *__restrict__ src, size_t n, float2 *__restrict__ dst)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        dst[i] = f64_to_pair(src[i]);
}

int launch_to_pairs(const double *src, size_t n, float2 *dst, cudaStream_t s)
{
    size_t blocks = (n + 255) / 256;
    if (blocks > 4096)
        blocks = 4096;
    to_pairs_kernel<<<(int) blocks, 256, 0, s>>>(src, n, dst);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

template <int NC, bool WS, bool DF>
__global__ void __launch_bounds__(UY_THREADS) update_y_kernel(
    const double *__restrict__ FI, const float2 *__restrict__ FIp, const double *__restrict__ Wg,
    const double *__restrict__ G, const double *__restrict__ RT, int K, int M1, int D, int Dw,
    double *__restrict__ Y, double *__restrict__ yy, double *__restrict__ bterm, YCopies cp,
    int *ticket, const float2 *__restrict__ Wq)
{
    // Wq (DF without WS, may be null): W as FP32 pairs in global memory, M1 x Dw
    // M1 x Dw, zero past D: FP64 values, or (hi, lo) pairs of the same size
    extern __shared__ double Ws[];
    float2 *const Wp = reinterpret_cast<float2 *>(Ws);
    if (WS) {
        const int n = M1 * Dw;
#pragma unroll 4
        for (int i = threadIdx.x; i < n; i += UY_THREADS) {
            const int m = i / Dw, d = i - m * Dw;
            const double w = (d < D) ? Wg[(size_t) m * D + d] : 0.0;
            if constexpr (DF)
                Wp[i] = f64_to_pair(w);
            else
                Ws[i] = w;
        }
        __syncthreads();
    }
    __nv_bfloat16 *const hi = reinterpret_cast<__nv_bfloat16 *>(cp.Yb);
    __nv_bfloat16 *const lo = hi ? hi + (size_t) cp.Kpad * cp.Dp : nullptr;
    const int lane = threadIdx.x & 31;
    for (;;) {
        int pair = 0;
        if (lane == 0)
            pair = atomicAdd(ticket, 1);
        const int k0 = 2 * __shfl_sync(0xffffffffu, pair, 0);
        if (k0 >= K)
            break;
        const int nr = (k0 + 1 < K) ? 2 : 1;
        const int k1 = k0 + nr - 1;
        double syy[2] = {0.0, 0.0}, srt[2] = {0.0, 0.0}, sq[2] = {0.0, 0.0};
        for (int db = 0; db < D; db += 32 * NC) {
            double y0[NC], y1[NC];
            if constexpr (DF) {
                float p0[NC], s0[NC], p1[NC], s1[NC];
#pragma unroll
                for (int c = 0; c < NC; c++)
                    p0[c] = s0[c] = p1[c] = s1[c] = 0.f;
                const float2 *f0 = FIp + (size_t) k0 * M1, *f1 = FIp + (size_t) k1 * M1;
                for (int m = 0; m < M1; m++) {
                    const float2 x0 = f0[m], x1 = f1[m];
#pragma unroll
                    for (int c = 0; c < NC; c++) {
                        const int d = db + lane + 32 * c;
                        const float2 w = WS ? Wp[m * Dw + d]
                                         : Wq ? Wq[(size_t) m * Dw + d]
                                              : ((d < D) ? f64_to_pair(Wg[(size_t) m * D + d])
                                                         : make_float2(0.f, 0.f));
                        dot2_step(p0[c], s0[c], x0, w);
                        dot2_step(p1[c], s1[c], x1, w);
                    }
                }
#pragma unroll
                for (int c = 0; c < NC; c++) {
                    y0[c] = (double) p0[c] + (double) s0[c];
                    y1[c] = (double) p1[c] + (double) s1[c];
                }
            } else {
#pragma unroll
                for (int c = 0; c < NC; c++)
                    y0[c] = y1[c] = 0.0;
                const double *f0 = FI + (size_t) k0 * M1, *f1 = FI + (size_t) k1 * M1;
                for (int m = 0; m < M1; m++) {
                    const double x0 = __ldg(f0 + m), x1 = __ldg(f1 + m);
#pragma unroll
                    for (int c = 0; c < NC; c++) {
                        const int d = db + lane + 32 * c;
                        const double w =
                            WS ? Ws[m * Dw + d] : ((d < D) ? __ldg(Wg + (size_t) m * D + d) : 0.0);
                        y0[c] = fma(x0, w, y0[c]);
                        y1[c] = fma(x1, w, y1[c]);
                    }
                }
            }
#pragma unroll
            for (int c = 0; c < NC; c++) {
                const int d = db + lane + 32 * c;
                if (d >= D)
                    continue;
#pragma unroll
                for (int r = 0; r < 2; r++) {
                    if (r >= nr)
                        break;
                    const int k = k0 + r;
                    const double y = r ? y1[c] : y0[c];
                    const size_t e = (size_t) k * D + d;
                    Y[e] = y;
                    syy[r] = fma(y, y, syy[r]);
                    if (RT)
                        srt[r] = fma(y, RT[e], srt[r]);
                    if (cp.Y32)
                        cp.Y32[e] = (float) y;
                    if (hi) {
                        // BF16 hi + lo of y, as the split form's set-up does
                        const __nv_bfloat16 h = __float2bfloat16_rn((float) y);
                        const double hd = (double) __bfloat162float(h);
                        const __nv_bfloat16 l = __float2bfloat16_rn((float) (y - hd));
                        const double yh = hd + (double) __bfloat162float(l);
                        hi[(size_t) k * cp.Dp + d] = h;
                        lo[(size_t) k * cp.Dp + d] = l;
                        sq[r] = fma(yh, yh, sq[r]);
                    }
                }
            }
        }
#pragma unroll
        for (int r = 0; r < 2; r++) {
            if (r >= nr)
                break;
            const int k = k0 + r;
            const double s_yy = uy_warp_sum(syy[r]);
            const double s_rt = RT ? uy_warp_sum(srt[r]) : 0.0;
            const double s_q = hi ? uy_warp_sum(sq[r]) : 0.0;
            if (lane == 0) {
                yy[k] = s_yy;
                if (bterm)
                    bterm[k] = G[k] * s_yy - 2.0 * s_rt;
            }
            if (hi && lane < 3) {
                // -q/2 in three BF16 pieces (24+ significant bits), columns D .. D+2
                const double v = -0.5 * s_q;
                const __nv_bfloat16 p1 = __float2bfloat16_rn((float) v);
                const double r1 = v - (double) __bfloat162float(p1);
                const __nv_bfloat16 p2 = __float2bfloat16_rn((float) r1);
                const double r2 = r1 - (double) __bfloat162float(p2);
                const __nv_bfloat16 p3 = __float2bfloat16_rn((float) r2);
                hi[(size_t) k * cp.Dp + D + lane] = (lane == 0) ? p1 : (lane == 1) ? p2 : p3;
            }
        }
    }
}

using UpdateYKernel = void (*)(const double *, const float2 *, const double *, const double *,
                               const double *, int, int, int, int, double *, double *, double *,
                               YCopies, int *, const float2 *);

// W (M1 x D) as FP32 pairs, M1 x Dw with zero columns past D
__global__ void w_pairs_kernel(const double *__restrict__ W, int M1, int D, int Dw,
                               float2 *__restrict__ Wq)
{
    const size_t n = (size_t) M1 * Dw;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x) {
        const int m = (int) (i / Dw), d = (int) (i % Dw);
        Wq[i] = d < D ? f64_to_pair(W[(size_t) m * D + d]) : make_float2(0.f, 0.f);
    }
}

template <bool WS, bool DF>
UpdateYKernel update_y_for(int nc)
{
    switch (nc) {
    case 1: return update_y_kernel<1, WS, DF>;
    case 2: return update_y_kernel<2, WS, DF>;
    case 3: return update_y_kernel<3, WS, DF>;
    case 4: return update_y_kernel<4, WS, DF>;
    case 5: return update_y_kernel<5, WS, DF>;
    case 6: return update_y_kernel<6, WS, DF>;
    case 7: return update_y_kernel<7, WS, DF>;
    default: return update_y_kernel<8, WS, DF>;
    }
}

int launch_update_y(const double *FI, const float2 *FIp, const double *W, const double *G,
                    const double *RT, int K, int M1, int D, double *Y, double *yy, double *bterm,
                    const YCopies &cp, int *ticket, double *scratch, size_t scratch_doubles,
                    int *nlaunch, cudaStream_t s)
{
    DGTM_CUDA_TRY(cudaMemsetAsync(ticket, 0, sizeof(int), s));
    int dev = 0, sms = 0;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int nc = ceil_div(D, 32);
    if (nc > UY_NCMAX)
        nc = UY_NCMAX;
    const int Dw = ceil_div(D, 32 * nc) * 32 * nc;
    const size_t wbytes = sizeof(double) * (size_t) M1 * Dw;  // = pairs of FP32
    const bool ws = wbytes <= UY_WSMEM_MAX;
    const bool df = FIp != nullptr;
    int blocks = ceil_div(K, 2 * (UY_THREADS / 32));
    const int cap = sms * (ws ? 2 : 4);
    if (blocks > cap)
        blocks = cap;
    const UpdateYKernel k = ws ? (df ? update_y_for<true, true>(nc) : update_y_for<true, false>(nc))
                               : (df ? update_y_for<false, true>(nc) : update_y_for<false, false>(nc));
    if (ws)
        DGTM_CUDA_TRY(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int) wbytes));
    // W beyond shared memory: converted to pairs once here, not per centre
    float2 *Wq = nullptr;
    int nl = 1;
    if (!ws && df && scratch && (size_t) M1 * Dw <= scratch_doubles) {
        Wq = reinterpret_cast<float2 *>(scratch);
        w_pairs_kernel<<<ceil_div(M1 * Dw, 256), 256, 0, s>>>(W, M1, D, Dw, Wq);
        DGTM_CUDA_TRY(cudaGetLastError());
        nl++;
    }
    k<<<blocks, UY_THREADS, ws ? wbytes : 0, s>>>(FI, FIp, W, G, RT, K, M1, D, Dw, Y, yy, bterm, cp,
                                                 ticket, Wq);
    DGTM_CUDA_TRY(cudaGetLastError());
    if (nlaunch)
        *nlaunch = nl;
    return DGTM_OK;
}

__global__ void norms_kernel(const double *__restrict__ X, int rows, int D,
                             double *__restrict__ out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    for (int r = blockIdx.x * wpb + warp; r < rows; r += gridDim.x * wpb) {
        double s = 0.0;
        for (int d = lane; d < D; d += 32) {
            const double v = X[(size_t) r * D + d];
            s += v * v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0)
            out[r] = s;
    }
}

int launch_norms(const double *X, int rows, int D, double *out, cudaStream_t s)
{
    int blocks = ceil_div(rows, 8);
    if (blocks > 4864)
        blocks = 4864;
    norms_kernel<<<blocks, 256, 0, s>>>(X, rows, D, out);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

__global__ void __launch_bounds__(1024) sum_ratio_kernel(const double *__restrict__ v, int n,
                                                        double add, double num, double *out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)  // coalesced, fixed order
        s += v[i];
    s = block_sum_fixed(s, red);
    if (threadIdx.x == 0) {
        const double den = s + add;
        out[0] = den;
        out[1] = num / den;
    }
}

int launch_sum_ratio(const double *v, int n, double add, double num, double *out, cudaStream_t s)
{
    sum_ratio_kernel<<<1, 1024, 0, s>>>(v, n, add, num, out);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

__global__ void __launch_bounds__(1024) sum_dev_kernel(const double *__restrict__ v, int n,
                                                      const double *__restrict__ add, double *out)
{
    __shared__ double red[32];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)  // coalesced, fixed order
        s += v[i];
    s = block_sum_fixed(s, red);
    if (threadIdx.x == 0)
        out[0] = s + add[0];
}

int launch_sum_ratio_dev(const double *v, int n, const double *add_dev, double *out,
                         cudaStream_t s)
{
    sum_dev_kernel<<<1, 1024, 0, s>>>(v, n, add_dev, out);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

__global__ void __launch_bounds__(1024) sum_pairs_kernel(const double *__restrict__ part,
                                                        int nb, double *out)
{
    __shared__ double red[32];
    double s0 = 0.0, s1 = 0.0;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) {  // coalesced, fixed order
        s0 += part[2 * i];
        s1 += part[2 * i + 1];
    }
    s0 = block_sum_fixed(s0, red);
    s1 = block_sum_fixed(s1, red);
    if (threadIdx.x == 0) {
        out[0] = s0;
        out[1] = s1;
    }
}

int launch_sum_pairs(const double *part, int nblocks, double *out, cudaStream_t s)
{
    sum_pairs_kernel<<<1, 1024, 0, s>>>(part, nblocks, out);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

__global__ void to_f32_kernel(const double *__restrict__ src, size_t n, float *__restrict__ dst)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        dst[i] = (float) src[i];
}

int launch_to_f32(const double *src, size_t n, float *dst, cudaStream_t s)
{
    size_t blocks = (n + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    if (blocks == 0)
        return DGTM_OK;
    to_f32_kernel<<<(unsigned) blocks, 256, 0, s>>>(src, n, dst);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

}  // namespace dgtm
