// mstep.cu -- the small FP64 kernels of the M-step, shared by every form.
//
//   reduce_slices : G_k = sum_s Gpart[s][k], RT = sum_s RTpart[s] (fixed order)
//   form_ab       : A = FI^T diag(G) FI, B = FI^T RT     (dagtm/dagtm.cxx:1715-1761),
//                   K-sliced 4 x 4 register tiles, slice partials summed in order
//   solve         : A W = B, FP64 Cholesky (numerically dependent pivots dropped;
//                   one-block factorisation, one warp per right-hand side)
//                   or symmetric-eigen pseudo-inverse
//                   with exactly-zero eigenvalues dropped (the semantics of
//                   gsl_linalg_SV_solve used by dagtm_solve2, comm/comm.c:1299-1348)
//   update_y      : Y = FI W (dagtm/dagtm.cxx:1769), |y_k|^2 and the beta terms
//   sum_ratio     : beta = N D / (sum_k G_k|y_k|^2 - 2 y_k.RT_k + sum_n |t_n|^2)
//                   = N D / sum_kn R_kn |y_k - t_n|^2 (comm/mpicomm.c:276-302
//                   evaluates the same sum over an explicit K x N distance matrix;
//                   every column of R sums to one, which gives the closed form)
//
// Every reduction runs in a fixed order, so repeated runs are bit-identical.
#include "common.cuh"
#include "kernels.cuh"

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

// C = FI^T [RT | diag(G) FI] (M1 x (D + M1)): B = C[:, :D], A = C[:, D:].
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
    const bool active = tile < (M1p / 4) * nct;
    const int m0 = active ? (tile / nct) * 4 : 0, c0 = active ? (tile % nct) * 4 : 0;
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
// solvers (one block)
// ---------------------------------------------------------------------------
constexpr int SOLVE_THREADS = 512;
constexpr int SMEM_SOLVE_MAX = 110;  // M1 up to which L lives in shared memory
constexpr int TRI_MAXR = 8;  // registers per lane in the substitution: M1 <= 256

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

// Right-looking Cholesky in one block, one barrier per column.  Thread t
// owns rows i = t/4, t/4 + 64, ... and in each the columns k = t (mod 4).
// Column j stays unscaled while it is in use: after the barrier of step j
// every thread reads the pivot's reciprocal square root r_j, updates its
// trailing elements as L[i][k] -= (a_ij r_j^2) a_kj (a: the unscaled column
// j), and the scaled a_ij r_j goes to the unused upper triangle at [j][i].
// The next pivot is the first element its owner updates in a step; the
// owner takes its reciprocal square root and publishes it before its other
// rows.  A last pass moves the scaled columns to the lower triangle.  A pivot
// that keeps less than CHOL_DROP of its diagonal (the column adds no new
// direction at FP64 precision) is dropped: its diagonal and column are stored
// as 0 and that unknown is fixed at 0, which keeps the solve defined when
// A = FI^T diag(G) FI is numerically singular (wide basis functions).
// L (lower triangle) goes to work[0 .. M1*M1), the reciprocal diagonal to
// work[M1*M1 .. M1*M1 + M1) (0 for a dropped pivot); flag[1] counts the drops.
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

__global__ void __launch_bounds__(CHOL_THREADS) cholesky_kernel(const double *__restrict__ A,
                                                               int M1, double *__restrict__ work,
                                                               int *flag)
{
    extern __shared__ double sh[];
    double *L = (M1 <= SMEM_SOLVE_MAX) ? sh : work;
    __shared__ double rinv[32 * TRI_MAXR], adiag[32 * TRI_MAXR];  // pivots: 1/sqrt, A's diagonal
    __shared__ int bad, ndrop;
    const int tid = threadIdx.x, q = tid & 3, r0 = tid >> 2;
    const size_t n2 = (size_t) M1 * M1;
    if (tid == 0) {
        bad = 0;
        ndrop = 0;
    }
#pragma unroll 4
    for (size_t e = tid; e < n2; e += CHOL_THREADS)
        L[e] = A[e];
    for (int j = tid; j < M1; j += CHOL_THREADS)
        adiag[j] = A[(size_t) j * M1 + j];
    __syncthreads();
    if (tid == 0)
        chol_pivot(L, adiag, M1, 0, rinv, &bad, &ndrop);
    for (int j = 0; j < M1; j++) {
        __syncthreads();
        const double rj = rinv[j], r2 = rj * rj;
        for (int i = r0; i < M1; i += 64) {
            if (i <= j)
                continue;
            const double aij = L[(size_t) i * M1 + j];
            if (q == 0)
                L[(size_t) j * M1 + i] = aij * rj;
            const double ti = aij * r2;
            for (int k = j + 1 + ((q - j - 1) & 3); k <= i; k += 4)
                L[(size_t) i * M1 + k] = fma(-ti, L[(size_t) k * M1 + j], L[(size_t) i * M1 + k]);
            if (i == j + 1 && q == ((j + 1) & 3))
                chol_pivot(L, adiag, M1, j + 1, rinv, &bad, &ndrop);
        }
    }
    __syncthreads();
    for (size_t e = tid; e < n2; e += CHOL_THREADS) {
        const int i = (int) (e / M1), k = (int) (e % M1);
        if (k < i)
            work[e] = L[(size_t) k * M1 + i];
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
    default: return tri_solve_kernel<8>;
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
        const size_t smem = (M1 <= SMEM_SOLVE_MAX) ? sizeof(double) * (size_t) M1 * M1 : 0;
        DGTM_CUDA_TRY(cudaFuncSetAttribute(cholesky_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int) (smem > 0 ? smem : 1)));
        cholesky_kernel<<<1, CHOL_THREADS, smem, s>>>(A, M1, work, flag);
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
// Y = FI W and the per-centre terms of beta
// ---------------------------------------------------------------------------
constexpr int WSMEM_MAX = 96 * 1024;

__global__ void __launch_bounds__(256) update_y_kernel(const double *__restrict__ FI,
                                                      const double *__restrict__ Wg,
                                                      const double *__restrict__ G,
                                                      const double *__restrict__ RT, int K,
                                                      int M1, int D, int w_in_smem,
                                                      double *__restrict__ Y,
                                                      double *__restrict__ yy,
                                                      double *__restrict__ bterm)
{
    extern __shared__ double Ws[];
    const double *W = Wg;
    if (w_in_smem) {
        for (int i = threadIdx.x; i < M1 * D; i += blockDim.x)
            Ws[i] = Wg[i];
        __syncthreads();
        W = Ws;
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = blockIdx.x * 8 + warp; k < K; k += gridDim.x * 8) {
        double syy = 0.0, syrt = 0.0;
        const double *fi = FI + (size_t) k * M1;
        for (int d = lane; d < D; d += 32) {
            double y = 0.0;
            for (int m = 0; m < M1; m++)
                y += fi[m] * W[(size_t) m * D + d];
            Y[(size_t) k * D + d] = y;
            syy += y * y;
            if (RT)
                syrt += y * RT[(size_t) k * D + d];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            syy += __shfl_xor_sync(0xffffffffu, syy, o);
            syrt += __shfl_xor_sync(0xffffffffu, syrt, o);
        }
        if (lane == 0) {
            yy[k] = syy;
            if (bterm)
                bterm[k] = G[k] * syy - 2.0 * syrt;
        }
    }
}

int launch_update_y(const double *FI, const double *W, const double *G, const double *RT, int K,
                    int M1, int D, double *Y, double *yy, double *bterm, cudaStream_t s)
{
    const size_t wbytes = sizeof(double) * (size_t) M1 * D;
    const int in_smem = wbytes <= WSMEM_MAX;
    const size_t smem = in_smem ? wbytes : 0;
    DGTM_CUDA_TRY(cudaFuncSetAttribute(update_y_kernel,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) (smem > 0 ? smem : 1)));
    int blocks = ceil_div(K, 8);
    if (blocks > 1216)
        blocks = 1216;
    update_y_kernel<<<blocks, 256, smem, s>>>(FI, W, G, RT, K, M1, D, in_smem, Y, yy, bterm);
    DGTM_CUDA_TRY(cudaGetLastError());
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
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    double s = 0.0;
    for (int i = b; i < e; i++)
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
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    double s = 0.0;
    for (int i = b; i < e; i++)
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
    const int per = (nb + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(nb, b + per);
    double s0 = 0.0, s1 = 0.0;
    for (int i = b; i < e; i++) {
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
