// ctemp.cu -- the next critical temperature of the AUTO cooling schedule
// (comm/mpicomm.c:562-674, dagtm_mpi_next_ctemp and its helper; the limit
// filter of dagtm_vector_max, comm/comm.c:2149-2161), FP64.
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
//   scatter_kernel : one CTA per (centre, 32 x 32 tile of the upper triangle);
//                    recomputes R_kn as the R-block kernel does and sums S1, S2
//                    over all points in a fixed order
//   eig_kernel     : one CTA per (centre, block); parallel cyclic Jacobi
//                    (round-robin pairing) on the D x D block, then the filter
#include "common.cuh"
#include "kernels.cuh"

#include <float.h>
#include <math.h>

namespace dgtm {

namespace {

constexpr int SC_THREADS = 256;
constexpr int SC_TILE = 32;   // output tile (rows x cols of S)
constexpr int SC_PTS = 32;    // points per staged chunk
constexpr int EIG_THREADS = 256;
constexpr double GG_MIN = 1e-250;  // comm/mpicomm.c:601-612

__global__ void __launch_bounds__(SC_THREADS) scatter_kernel(
    const double *__restrict__ T, const double *__restrict__ Y, const double *__restrict__ tt,
    const double *__restrict__ yy, const double2 *__restrict__ colstat, int N, int D, int K,
    double c, int k0, double *__restrict__ S, double *__restrict__ gsum)
{
    __shared__ double xr[SC_PTS][SC_TILE], xc[SC_PTS][SC_TILE], w[SC_PTS];
    const int kl = blockIdx.x, k = k0 + kl;
    // upper-triangle tile (ti <= tj) from the linear tile index
    int ti = 0, rem = blockIdx.y;
    const int nb = (D + SC_TILE - 1) / SC_TILE;
    while (rem >= nb - ti) {
        rem -= nb - ti;
        ti++;
    }
    const int tj = ti + rem;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int r = threadIdx.x >> 3, c0 = (threadIdx.x & 7) * 4;  // this thread's 1 x 4 entries
    const double *yk = Y + (size_t) k * D;
    double s1[4] = {0.0, 0.0, 0.0, 0.0}, s2[4] = {0.0, 0.0, 0.0, 0.0}, g = 0.0;
    for (int nb0 = 0; nb0 < N; nb0 += SC_PTS) {
        __syncthreads();
        // responsibilities of the chunk's points for centre k (warp per point)
        for (int p = warp; p < SC_PTS; p += SC_THREADS / 32) {
            const int n = nb0 + p;
            double rv = 0.0;
            if (n < N) {
                const double2 cs = colstat[n];
                if (isnan(cs.y)) {
                    rv = 1.0 / (double) K;
                } else {
                    double dot = 0.0;
                    for (int d = lane; d < D; d += 32)
                        dot += yk[d] * T[(size_t) n * D + d];
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1)
                        dot += __shfl_down_sync(0xffffffffu, dot, o);
                    dot = __shfl_sync(0xffffffffu, dot, 0);
                    const double dd = ((-2.0 * dot) + yy[k]) + tt[n];
                    rv = exp(-c * (dd - cs.x) - cs.y);
                }
            }
            if (lane == 0)
                w[p] = rv;
        }
        // x = t - y over the tile's row and column ranges
        for (int e = threadIdx.x; e < SC_PTS * SC_TILE; e += SC_THREADS) {
            const int p = e / SC_TILE, j = e % SC_TILE, n = nb0 + p;
            const int di = ti * SC_TILE + j, dj = tj * SC_TILE + j;
            xr[p][j] = (n < N && di < D) ? T[(size_t) n * D + di] - yk[di] : 0.0;
            xc[p][j] = (n < N && dj < D) ? T[(size_t) n * D + dj] - yk[dj] : 0.0;
        }
        __syncthreads();
        for (int p = 0; p < SC_PTS; p++) {
            const double wp = w[p], w2 = wp * wp, a = xr[p][r];
            if (threadIdx.x == 0)
                g += wp;
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const double v = a * xc[p][c0 + e];
                s1[e] = fma(wp, v, s1[e]);
                s2[e] = fma(w2, v, s2[e]);
            }
        }
    }
    // both triangles of S1 (block 0) and S2 (block 1) of this centre
    double *S1 = S + (size_t) kl * 2 * D * D, *S2 = S1 + (size_t) D * D;
    const int i = ti * SC_TILE + r;
#pragma unroll
    for (int e = 0; e < 4; e++) {
        const int j = tj * SC_TILE + c0 + e;
        if (i < D && j < D) {
            S1[(size_t) i * D + j] = s1[e];
            S2[(size_t) i * D + j] = s2[e];
            S1[(size_t) j * D + i] = s1[e];
            S2[(size_t) j * D + i] = s2[e];
        }
    }
    if (blockIdx.y == 0 && threadIdx.x == 0)
        gsum[kl] = g;
}

// fixed-order block sum (every thread gets the result)
__device__ double block_sum(double v, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0)
        red[warp] = v;
    __syncthreads();
    double t = 0.0;
    for (int i = 0; i < EIG_THREADS / 32; i++)
        t += red[i];
    return t;
}

// blockIdx.x = centre in the batch, blockIdx.y = 0: 2 S1, 1: 2 (S1 - S2)
__global__ void __launch_bounds__(EIG_THREADS) eig_kernel(const double *__restrict__ S, int D,
                                                          int in_smem, double *__restrict__ Mg,
                                                          const double *__restrict__ gg,
                                                          double lim_scale, double *__restrict__ out)
{
    extern __shared__ double sh[];
    const int kl = blockIdx.x, which = blockIdx.y;
    const int npair = (D + 1) / 2, nslot = 2 * npair;  // slot D (odd D) is a dummy
    double *M = in_smem ? sh : Mg + ((size_t) kl * 2 + which) * D * D;
    double *cs = in_smem ? sh + (size_t) D * D : sh;
    double *sn = cs + npair;
    int *pp = (int *) (sn + npair), *qq = pp + npair;
    __shared__ double red[EIG_THREADS / 32];
    __shared__ int done;
    const double *S1 = S + (size_t) kl * 2 * D * D, *S2 = S1 + (size_t) D * D;
    const double gk = gg[kl];
    if (gk == 0.0) {
        // the reference returns HUGE_VAL before any eigen work (comm/mpicomm.c:582-585)
        if (threadIdx.x == 0)
            out[(size_t) kl * 2 + which] = 0.0;
        return;
    }
    // gg < GG_MIN: the reference scales H by 1 / GG_MIN before gsl_eigen_symm
    const double sc = (gk < GG_MIN) ? 1.0 / GG_MIN : 1.0;
    for (int e = threadIdx.x; e < D * D; e += EIG_THREADS)
        M[e] = (which == 0 ? 2.0 * S1[e] : 2.0 * (S1[e] - S2[e])) * sc;
    __syncthreads();
    for (int sweep = 0; sweep < 100; sweep++) {
        double off = 0.0, tot = 0.0;
        for (int e = threadIdx.x; e < D * D; e += EIG_THREADS) {
            const double v = M[e] * M[e];
            tot += v;
            if (e / D != e % D)
                off += v;
        }
        off = block_sum(off, red);
        tot = block_sum(tot, red);
        if (threadIdx.x == 0)
            done = (off <= DBL_EPSILON * DBL_EPSILON * tot);
        __syncthreads();
        if (done)
            break;
        for (int step = 0; step < nslot - 1; step++) {
            for (int t = threadIdx.x; t < npair; t += EIG_THREADS) {
                // round-robin pairing: slot 0 fixed, the others rotate
                const int a = (t == 0) ? 0 : 1 + ((t - 1 + step) % (nslot - 1));
                const int b = 1 + ((nslot - 2 - t + step) % (nslot - 1));
                const int p = min(a, b), q = max(a, b);
                double cc = 1.0, ss = 0.0;
                if (q < D) {
                    const double apq = M[(size_t) p * D + q];
                    if (apq != 0.0) {
                        const double app = M[(size_t) p * D + p], aqq = M[(size_t) q * D + q];
                        const double th = (aqq - app) / (2.0 * apq);
                        const double tn = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
                        cc = 1.0 / sqrt(tn * tn + 1.0);
                        ss = tn * cc;
                    }
                }
                pp[t] = p;
                qq[t] = q;
                cs[t] = cc;
                sn[t] = ss;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < npair * D; idx += EIG_THREADS) {
                const int t = idx / D, j = idx % D;
                if (qq[t] >= D || sn[t] == 0.0)
                    continue;
                const int p = pp[t], q = qq[t];
                const double mp = M[(size_t) p * D + j], mq = M[(size_t) q * D + j];
                M[(size_t) p * D + j] = cs[t] * mp - sn[t] * mq;
                M[(size_t) q * D + j] = sn[t] * mp + cs[t] * mq;
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < npair * D; idx += EIG_THREADS) {
                const int t = idx / D, j = idx % D;
                if (qq[t] >= D || sn[t] == 0.0)
                    continue;
                const int p = pp[t], q = qq[t];
                const double mp = M[(size_t) j * D + p], mq = M[(size_t) j * D + q];
                M[(size_t) j * D + p] = cs[t] * mp - sn[t] * mq;
                M[(size_t) j * D + q] = sn[t] * mp + cs[t] * mq;
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        // eigenvalues at or above the limit count as 0, then the largest
        const double limit = lim_scale * gk;
        double mx = -INFINITY;
        for (int i = 0; i < D; i++) {
            double l = M[(size_t) i * D + i];
            if (gk < GG_MIN)
                l *= GG_MIN;
            if (l >= limit)
                l = 0.0;
            mx = fmax(mx, l);
        }
        out[(size_t) kl * 2 + which] = mx;
    }
}

}  // namespace

size_t ctemp_scratch_doubles(int D, int kb, bool *eig_in_smem)
{
    const size_t dd = (size_t) D * D;
    const size_t smem = sizeof(double) * (dd + (size_t) 2 * ((D + 1) / 2)) +
                        sizeof(int) * (size_t) 2 * ((D + 1) / 2);
    *eig_in_smem = smem <= (size_t) 200 * 1024;
    return (size_t) kb * 2 * dd * (*eig_in_smem ? 1 : 2) + (size_t) 4 * kb;
}

int launch_ctemp_batch(const double *T, const double *Y, const double *tt, const double *yy,
                       const double2 *colstat, int N, int D, int K, double c, int k0, int kb,
                       const double *gg_dev, double lim_scale, double *scratch, double *gsum_dev,
                       double *out_dev, cudaStream_t s)
{
    bool in_smem = false;
    ctemp_scratch_doubles(D, kb, &in_smem);
    double *S = scratch;
    double *Mg = scratch + (size_t) kb * 2 * D * D;
    const int nb = (D + SC_TILE - 1) / SC_TILE;
    scatter_kernel<<<dim3(kb, nb * (nb + 1) / 2), SC_THREADS, 0, s>>>(T, Y, tt, yy, colstat, N, D,
                                                                      K, c, k0, S, gsum_dev);
    DGTM_CUDA_TRY(cudaGetLastError());
    const int npair = (D + 1) / 2;
    const size_t small = sizeof(double) * 2 * npair + sizeof(int) * 2 * npair;
    const size_t smem = (in_smem ? sizeof(double) * (size_t) D * D : 0) + small;
    DGTM_CUDA_TRY(cudaFuncSetAttribute(eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int) smem));
    eig_kernel<<<dim3(kb, 2), EIG_THREADS, smem, s>>>(S, D, in_smem ? 1 : 0, Mg,
                                                      gg_dev ? gg_dev : gsum_dev, lim_scale,
                                                      out_dev);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

}  // namespace dgtm
