// estep_simt.cu -- FP64 / FP32 CUDA-core kernels of the E-step and of the
// responsibility pass of the M-step (the "plain" precision forms).
//
// Pass 1 (n-owner): one block per 64 data points; the block streams all K
// centres in chunks of 64 and keeps, per point, the running minimum distance
// and the two shifted sums
//     s1_n = sum_k exp(-c1 (d_kn - dmin_n)),  c1 = beta/2
//     s2_n = sum_k exp(-c2 (d_kn - dmin_n)),  c2 = beta/(2 temp)
// so that log vgc_n = -c1 dmin_n + log s1_n and log vgc2_n = -c2 dmin_n +
// log s2_n (comm/mpicomm.c:324-357 computes vgc/vgc2 unshifted).  Nothing of
// size K x N is stored.
//
// Pass 2 (k-owner): one block per 64 centres and one slice of the points.  It
// recomputes d_kn, forms R_kn = exp(-c (d_kn - dmin_n) - log s_n) and
// accumulates G_k = sum_n R_kn and RT_kd = sum_n R_kn t_nd for its slice;
// the slices are summed in a fixed order afterwards (mstep.cu).
//
// Distances follow comm/comm.c:560-629: d = (-2 y.t + |y|^2) + |t|^2 with the
// norms in FP64.
#include "common.cuh"
#include "kernels.cuh"

#include <math.h>

namespace dgtm {

namespace {

constexpr int BN = 64;   // points per tile
constexpr int BKT = 64;  // centres per tile
constexpr int DC = 16;   // depth of one streamed slice
constexpr int NT = 256;  // threads per block

template <typename F>
__device__ __forceinline__ F fexp(F x);
template <>
__device__ __forceinline__ double fexp<double>(double x) { return exp(x); }
template <>
__device__ __forceinline__ float fexp<float>(float x) { return expf(x); }

// Load Ys[d][k] (d in [d0, d0+DC), k in [k0, k0+BKT)) from Y (K x D, row-major).
template <typename F>
__device__ __forceinline__ void load_y_slice(F (*Ys)[BKT + 1], const F *__restrict__ Y,
                                             int K, int D, int k0, int d0)
{
    for (int idx = threadIdx.x; idx < BKT * DC; idx += NT) {
        const int k = idx / DC, d = idx % DC;
        const int gk = k0 + k, gd = d0 + d;
        Ys[d][k] = (gk < K && gd < D) ? Y[(size_t) gk * D + gd] : F(0);
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// Pass 1
// ---------------------------------------------------------------------------
template <typename F>
__global__ void __launch_bounds__(NT) pass1_simt_kernel(Pass1Args<F> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldt = a.D | 1;  // odd row stride: conflict-free column reads
    F *Tt = reinterpret_cast<F *>(smem_raw);              // [BN][ldt]
    F(*Ys)[BKT + 1] = reinterpret_cast<F(*)[BKT + 1]>(Tt + BN * ldt);  // [DC][BKT+1]
    __shared__ double red[32];

    const int tx = threadIdx.x & 15;  // centre lane
    const int ty = threadIdx.x >> 4;  // point lane
    const int n0 = blockIdx.x * BN;

    for (int idx = threadIdx.x; idx < BN * a.D; idx += NT) {
        const int n = idx / a.D, d = idx % a.D;
        const int gn = n0 + n;
        Tt[n * ldt + d] = (gn < a.N) ? a.T[(size_t) gn * a.D + d] : F(0);
    }

    double ttn[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gn = n0 + ty + 16 * i;
        ttn[i] = (gn < a.N) ? a.tt[gn] : 0.0;
    }
    double dmin[4], s1[4], s2[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        dmin[i] = INFINITY;
        s1[i] = 0.0;
        s2[i] = 0.0;
    }

    for (int k0 = 0; k0 < a.K; k0 += BKT) {
        F acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                acc[i][j] = F(0);
        for (int d0 = 0; d0 < a.D; d0 += DC) {
            __syncthreads();
            load_y_slice<F>(Ys, a.Y, a.K, a.D, k0, d0);
            __syncthreads();
            const int dl = min(DC, a.D - d0);
            for (int dd = 0; dd < dl; dd++) {
                F tv[4], yv[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    tv[i] = Tt[(ty + 16 * i) * ldt + d0 + dd];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    yv[j] = Ys[dd][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        acc[i][j] += tv[i] * yv[j];
            }
        }
        // distances of this chunk and the online update of (dmin, s1, s2)
        double yyk[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gk = k0 + tx + 16 * j;
            yyk[j] = (gk < a.K) ? a.yy[gk] : 0.0;
        }
#pragma unroll
        for (int i = 0; i < 4; i++) {
            double dv[4];
            double lm = INFINITY;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int gk = k0 + tx + 16 * j;
                double dd;
                if constexpr (sizeof(F) == 8)
                    dd = ((double) (F(-2) * acc[i][j]) + yyk[j]) + ttn[i];
                else
                    dd = (double) ((F(-2) * acc[i][j] + (F) yyk[j]) + (F) ttn[i]);
                dv[j] = (gk < a.K) ? dd : INFINITY;
                lm = fmin(lm, dv[j]);
            }
#pragma unroll
            for (int o = 8; o > 0; o >>= 1)
                lm = fmin(lm, __shfl_xor_sync(0xffffffffu, lm, o));
            const double nm = fmin(dmin[i], lm);
            double e1 = 0.0, e2 = 0.0;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const double x = dv[j] - nm;
                e1 += (double) fexp<F>((F) (-a.c1 * x));
                if (a.isDA)
                    e2 += (double) fexp<F>((F) (-a.c2 * x));
            }
#pragma unroll
            for (int o = 8; o > 0; o >>= 1) {
                e1 += __shfl_xor_sync(0xffffffffu, e1, o);
                e2 += __shfl_xor_sync(0xffffffffu, e2, o);
            }
            if (nm < dmin[i]) {
                const double x = dmin[i] - nm;  // >= 0 (inf on the first chunk)
                s1[i] = (s1[i] == 0.0) ? 0.0 : s1[i] * exp(-a.c1 * x);
                if (a.isDA)
                    s2[i] = (s2[i] == 0.0) ? 0.0 : s2[i] * exp(-a.c2 * x);
                dmin[i] = nm;
            }
            s1[i] += e1;
            s2[i] += e2;
        }
    }

    // per-point results: column statistics and the two log-sum-exp terms
    double l1 = 0.0, l2 = 0.0;
    if (tx == 0) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int gn = n0 + ty + 16 * i;
            if (gn >= a.N)
                continue;
            const double lse1 = -a.c1 * dmin[i] + log(s1[i]);
            const double ss = a.isDA ? s2[i] : s1[i];
            double lsn = log(ss);
            double t1 = lse1, t2 = a.isDA ? (-a.c2 * dmin[i] + log(s2[i])) : 0.0;
            // comm/mpicomm.c:382-389: a column whose every exp(-beta d/2)
            // underflows is replaced by R = 1/K with v = K
            if (exp(-a.c1 * dmin[i]) == 0.0) {
                lsn = NAN;
                if (a.isDA) {
                    t1 = -INFINITY;          // log(vgc) = log 0
                    t2 = log((double) a.K);  // log(vgc2) = log K
                } else {
                    t1 = log((double) a.K);
                }
            }
            a.colstat[gn] = make_double2(dmin[i], lsn);
            l1 += t1;
            l2 += t2;
        }
    }
    l1 = block_sum_fixed(l1, red);
    l2 = block_sum_fixed(l2, red);
    if (threadIdx.x == 0) {
        a.part[2 * blockIdx.x + 0] = l1;
        a.part[2 * blockIdx.x + 1] = l2;
    }
}

// ---------------------------------------------------------------------------
// Pass 2: G and RT slices
// ---------------------------------------------------------------------------
// OWN = false: owners are centres, streamed rows are points, the statistics
// belong to the points (the M-step).  OWN = true: the same contraction with the
// roles exchanged -- owners are points carrying their own statistics, streamed
// rows are centres -- which gives sum_k R_kn y_k per point (the gradient of the
// free energy with respect to the data).
template <typename F, int NDJ, bool OWN>
__global__ void __launch_bounds__(NT) pass2_simt_kernel(Pass2Args<F> a)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldt = a.D | 1;
    F *Tf = reinterpret_cast<F *>(smem_raw);                                 // [BN][ldt]
    F(*Ys)[BKT + 1] = reinterpret_cast<F(*)[BKT + 1]>(Tf + BN * ldt);         // [DC][BKT+1]
    F(*Rs)[BKT + 1] = reinterpret_cast<F(*)[BKT + 1]>(&Ys[DC][0]);            // [BN][BKT+1]
    double *cst_dmin = reinterpret_cast<double *>(&Rs[BN][0]);               // [BN]
    double *cst_lsn = cst_dmin + BN;                                          // [BN]

    const int tx = threadIdx.x & 15;  // point lane (distance phase) / depth lane (RT phase)
    const int ty = threadIdx.x >> 4;  // centre lane
    const int k0 = blockIdx.x * BKT;
    const int split = blockIdx.y;
    const int nb = split * a.n_per_split;
    const int ne = min(a.N, nb + a.n_per_split);

    double yyk[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gk = k0 + ty + 16 * i;
        yyk[i] = (gk < a.K) ? a.yy[gk] : 0.0;
    }
    const double invK = 1.0 / (double) (OWN ? a.N : a.K);
    double own_dmin[4] = {0.0, 0.0, 0.0, 0.0}, own_lsn[4] = {0.0, 0.0, 0.0, 0.0};
    if constexpr (OWN) {
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int gk = k0 + ty + 16 * i;
            if (gk < a.K) {
                const double2 cs = a.colstat[gk];
                own_dmin[i] = cs.x;
                own_lsn[i] = cs.y;
            }
        }
    }

    double g[4] = {0.0, 0.0, 0.0, 0.0};
    double rt[4][NDJ];
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < NDJ; j++)
            rt[i][j] = 0.0;

    for (int n0 = nb; n0 < ne; n0 += BN) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < BN * a.D; idx += NT) {
            const int n = idx / a.D, d = idx % a.D;
            const int gn = n0 + n;
            Tf[n * ldt + d] = (gn < ne) ? a.T[(size_t) gn * a.D + d] : F(0);
        }
        if (!OWN && threadIdx.x < BN) {
            const int gn = n0 + threadIdx.x;
            const double2 cs = (gn < ne) ? a.colstat[gn] : make_double2(0.0, 0.0);
            cst_dmin[threadIdx.x] = cs.x;
            cst_lsn[threadIdx.x] = cs.y;
        }
        // distances d[i][j]: centre k0 + ty + 16 i, point n0 + tx + 16 j
        F acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                acc[i][j] = F(0);
        for (int d0 = 0; d0 < a.D; d0 += DC) {
            __syncthreads();
            load_y_slice<F>(Ys, a.Y, a.K, a.D, k0, d0);
            __syncthreads();
            const int dl = min(DC, a.D - d0);
            for (int dd = 0; dd < dl; dd++) {
                F tv[4], yv[4];
#pragma unroll
                for (int j = 0; j < 4; j++)
                    tv[j] = Tf[(tx + 16 * j) * ldt + d0 + dd];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    yv[i] = Ys[dd][ty + 16 * i];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++)
                        acc[i][j] += yv[i] * tv[j];
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int nl = tx + 16 * j;
            const int gn = n0 + nl;
            const double dmn_c = OWN ? 0.0 : cst_dmin[nl], lsn_c = OWN ? 0.0 : cst_lsn[nl];
            const double ttn = (gn < ne) ? a.tt[gn] : 0.0;
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int gk = k0 + ty + 16 * i;
                const double dmn = OWN ? own_dmin[i] : dmn_c;
                const double lsn = OWN ? own_lsn[i] : lsn_c;
                F r = F(0);
                if (gn < ne && gk < a.K) {
                    if (isnan(lsn)) {
                        r = (F) invK;
                    } else {
                        double dd;
                        if constexpr (sizeof(F) == 8)
                            dd = ((double) (F(-2) * acc[i][j]) + yyk[i]) + ttn;
                        else
                            dd = (double) ((F(-2) * acc[i][j] + (F) yyk[i]) + (F) ttn);
                        r = (dd > a.dcut) ? F(0) : fexp<F>((F) (-a.c * (dd - dmn) - lsn));
                    }
                }
                g[i] += (double) r;
                Rs[nl][ty + 16 * i] = r;
            }
        }
        __syncthreads();
        // RT[k][d] += sum_n R[k][n] T[n][d]; centre k0 + ty + 16 i, depth tx + 16 j
        if constexpr (sizeof(F) == 8) {
            for (int n = 0; n < BN; n++) {
                F rv[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    rv[i] = Rs[n][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < NDJ; j++) {
                    const int d = tx + 16 * j;
                    const F tv = (d < a.D) ? Tf[n * ldt + d] : F(0);
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        rt[i][j] += (double) (rv[i] * tv);
                }
            }
        } else {
            F loc[4][NDJ];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < NDJ; j++)
                    loc[i][j] = F(0);
            for (int n = 0; n < BN; n++) {
                F rv[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    rv[i] = Rs[n][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < NDJ; j++) {
                    const int d = tx + 16 * j;
                    const F tv = (d < a.D) ? Tf[n * ldt + d] : F(0);
#pragma unroll
                    for (int i = 0; i < 4; i++)
                        loc[i][j] += rv[i] * tv;
                }
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < NDJ; j++)
                    rt[i][j] += (double) loc[i][j];
        }
    }

    // G: reduce the 16 point lanes holding the same centres
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int o = 8; o > 0; o >>= 1)
            g[i] += __shfl_xor_sync(0xffffffffu, g[i], o);
    double *Gp = a.Gpart + (size_t) split * a.K;
    double *RTp = a.RTpart + (size_t) split * a.K * a.D;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gk = k0 + ty + 16 * i;
        if (gk >= a.K)
            continue;
        if (tx == 0)
            Gp[gk] = g[i];
#pragma unroll
        for (int j = 0; j < NDJ; j++) {
            const int d = tx + 16 * j;
            if (d < a.D)
                RTp[(size_t) gk * a.D + d] = rt[i][j];
        }
    }
}

// ---------------------------------------------------------------------------
// MAP projection M = R^T X and explicit blocks of R (FP64, from the column
// statistics of the last E-step)
// ---------------------------------------------------------------------------
// RD: the weights are R_kn d'_kn with d' the squared distance to a second set
// of centres Y2 (|y2|^2 in yy2): the reference's R o D after its beta update.
template <bool RD>
__global__ void __launch_bounds__(NT) map_kernel(const double *__restrict__ T,
                                                 const double *__restrict__ Y,
                                                 const double *__restrict__ tt,
                                                 const double *__restrict__ yy,
                                                 const double2 *__restrict__ colstat, int N,
                                                 int D, int K, double c,
                                                 const double *__restrict__ X, int L,
                                                 const double *__restrict__ Y2,
                                                 const double *__restrict__ yy2,
                                                 double *__restrict__ Mout)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ldt = D | 1;
    double *Tt = reinterpret_cast<double *>(smem_raw);
    double(*Ys)[BKT + 1] = reinterpret_cast<double(*)[BKT + 1]>(Tt + BN * ldt);
    double(*Ys2)[BKT + 1] = Ys + DC;  // RD only
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int n0 = blockIdx.x * BN;
    for (int idx = threadIdx.x; idx < BN * D; idx += NT) {
        const int n = idx / D, d = idx % D;
        Tt[n * ldt + d] = (n0 + n < N) ? T[(size_t) (n0 + n) * D + d] : 0.0;
    }
    double ttn[4], dmn[4], lsn[4];
    double m[4][8];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int gn = n0 + ty + 16 * i;
        const double2 cs = (gn < N) ? colstat[gn] : make_double2(0.0, 0.0);
        ttn[i] = (gn < N) ? tt[gn] : 0.0;
        dmn[i] = cs.x;
        lsn[i] = cs.y;
#pragma unroll
        for (int l = 0; l < 8; l++)
            m[i][l] = 0.0;
    }
    const double invK = 1.0 / (double) K;
    for (int k0 = 0; k0 < K; k0 += BKT) {
        double acc[4][4], acc2[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++)
                acc[i][j] = acc2[i][j] = 0.0;
        for (int d0 = 0; d0 < D; d0 += DC) {
            __syncthreads();
            load_y_slice<double>(Ys, Y, K, D, k0, d0);
            if (RD)
                load_y_slice<double>(Ys2, Y2, K, D, k0, d0);
            __syncthreads();
            const int dl = min(DC, D - d0);
            for (int dd = 0; dd < dl; dd++) {
                double tv[4], yv[4], yv2[4];
#pragma unroll
                for (int i = 0; i < 4; i++)
                    tv[i] = Tt[(ty + 16 * i) * ldt + d0 + dd];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    yv[j] = Ys[dd][tx + 16 * j];
                    yv2[j] = RD ? Ys2[dd][tx + 16 * j] : 0.0;
                }
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        acc[i][j] += tv[i] * yv[j];
                        if (RD)
                            acc2[i][j] += tv[i] * yv2[j];
                    }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int gk = k0 + tx + 16 * j;
            if (gk >= K)
                continue;
            const double yyk = yy[gk];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                double r;
                if (isnan(lsn[i])) {
                    r = invK;
                } else {
                    const double dd = ((-2.0 * acc[i][j]) + yyk) + ttn[i];
                    r = exp(-c * (dd - dmn[i]) - lsn[i]);
                }
                if (RD)  // the reference's operation order: -2 y.t, + |y|^2, + |t|^2
                    r *= ((-2.0 * acc2[i][j]) + yy2[gk]) + ttn[i];
#pragma unroll
                for (int l = 0; l < 8; l++)
                    if (l < L)
                        m[i][l] += r * X[(size_t) gk * L + l];
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
#pragma unroll
        for (int l = 0; l < 8; l++)
#pragma unroll
            for (int o = 8; o > 0; o >>= 1)
                m[i][l] += __shfl_xor_sync(0xffffffffu, m[i][l], o);
        const int gn = n0 + ty + 16 * i;
        if (tx == 0 && gn < N)
            for (int l = 0; l < L; l++)
                Mout[(size_t) gn * L + l] = m[i][l];
    }
}

__global__ void r_block_kernel(const double *__restrict__ T, const double *__restrict__ Y,
                               const double *__restrict__ tt, const double *__restrict__ yy,
                               const double2 *__restrict__ colstat, int D, int K, double c,
                               int k0, int nk, int n0, int nn, const double *__restrict__ Y2,
                               const double *__restrict__ yy2, double dcut, double *__restrict__ R)
{
    const size_t total = (size_t) nk * nn;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int k = k0 + (int) (i / nn), n = n0 + (int) (i % nn);
        const double2 cs = colstat[n];
        double r;
        if (isnan(cs.y)) {
            r = 1.0 / (double) K;
        } else {
            double dot = 0.0;
            for (int d = 0; d < D; d++)
                dot += Y[(size_t) k * D + d] * T[(size_t) n * D + d];
            const double dd = ((-2.0 * dot) + yy[k]) + tt[n];
            r = (dd > dcut) ? 0.0 : exp(-c * (dd - cs.x) - cs.y);
        }
        if (Y2) {
            double dot = 0.0;
            for (int d = 0; d < D; d++)
                dot += Y2[(size_t) k * D + d] * T[(size_t) n * D + d];
            r *= ((-2.0 * dot) + yy2[k]) + tt[n];
        }
        R[i] = r;
    }
}

int launch_map(const double *T, const double *Y, const double *tt, const double *yy,
               const double2 *colstat, int N, int D, int K, double c, const double *X, int L,
               double *M, cudaStream_t s, const double *Y2, const double *yy2)
{
    const size_t smem =
        sizeof(double) * ((size_t) BN * (D | 1) + (size_t) (Y2 ? 2 : 1) * DC * (BKT + 1));
    if (Y2) {
        DGTM_CUDA_TRY(cudaFuncSetAttribute(map_kernel<true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
        map_kernel<true><<<ceil_div(N, BN), NT, smem, s>>>(T, Y, tt, yy, colstat, N, D, K, c, X,
                                                            L, Y2, yy2, M);
    } else {
        DGTM_CUDA_TRY(cudaFuncSetAttribute(map_kernel<false>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
        map_kernel<false><<<ceil_div(N, BN), NT, smem, s>>>(T, Y, tt, yy, colstat, N, D, K, c, X,
                                                             L, nullptr, nullptr, M);
    }
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int launch_r_block(const double *T, const double *Y, const double *tt, const double *yy,
                   const double2 *colstat, int D, int K, double c, int k0, int nk, int n0, int nn,
                   double *R, cudaStream_t s, const double *Y2, const double *yy2, double dcut)
{
    size_t blocks = ((size_t) nk * nn + 255) / 256;
    if (blocks > 8192)
        blocks = 8192;
    r_block_kernel<<<(unsigned) blocks, 256, 0, s>>>(T, Y, tt, yy, colstat, D, K, c, k0, nk, n0,
                                                    nn, Y2, yy2, dcut, R);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
template <typename F>
size_t pass1_simt_smem(int D)
{
    return sizeof(F) * ((size_t) BN * (D | 1) + (size_t) DC * (BKT + 1));
}

template <typename F>
size_t pass2_simt_smem(int D)
{
    return sizeof(F) * ((size_t) BN * (D | 1) + (size_t) DC * (BKT + 1) + (size_t) BN * (BKT + 1)) +
           sizeof(double) * 2 * BN;
}

template <typename F>
int launch_pass1_simt(const Pass1Args<F> &a, cudaStream_t s)
{
    const size_t smem = pass1_simt_smem<F>(a.D);
    DGTM_CUDA_TRY(cudaFuncSetAttribute(pass1_simt_kernel<F>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
    pass1_simt_kernel<F><<<ceil_div(a.N, BN), NT, smem, s>>>(a);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int pass1_simt_blocks(int N) { return ceil_div(N, BN); }

template <typename F, int NDJ, bool OWN>
static int launch_pass2_ndj(const Pass2Args<F> &a, int nsplit, cudaStream_t s)
{
    const size_t smem = pass2_simt_smem<F>(a.D);
    DGTM_CUDA_TRY(cudaFuncSetAttribute(pass2_simt_kernel<F, NDJ, OWN>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
    dim3 grid(ceil_div(a.K, BKT), nsplit);
    pass2_simt_kernel<F, NDJ, OWN><<<grid, NT, smem, s>>>(a);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

template <typename F>
int launch_pass2_simt(const Pass2Args<F> &a, int nsplit, cudaStream_t s, bool own)
{
    const int ndj = ceil_div(a.D, 16);
    if (own && sizeof(F) != 4) {
        set_error(DGTM_ENOTSUP, "the exchanged-role pass exists in FP32 only");
        return DGTM_ENOTSUP;
    }
    switch (ndj) {
#define DGTM_CASE(n)                                                    \
    case n:                                                             \
        if constexpr (sizeof(F) == 4) {                                 \
            if (own)                                                    \
                return launch_pass2_ndj<F, n, true>(a, nsplit, s);      \
        }                                                               \
        return launch_pass2_ndj<F, n, false>(a, nsplit, s);
        DGTM_CASE(1) DGTM_CASE(2) DGTM_CASE(3) DGTM_CASE(4) DGTM_CASE(5) DGTM_CASE(6)
        DGTM_CASE(7) DGTM_CASE(8) DGTM_CASE(9) DGTM_CASE(10) DGTM_CASE(11) DGTM_CASE(12)
        DGTM_CASE(13) DGTM_CASE(14) DGTM_CASE(15) DGTM_CASE(16)
#undef DGTM_CASE
    default:
        set_error(DGTM_ENOTSUP, "D = %d exceeds the CUDA-core form's limit of 256", a.D);
        return DGTM_ENOTSUP;
    }
}

int pass2_simt_ktiles(int K) { return ceil_div(K, BKT); }

template int launch_pass1_simt<double>(const Pass1Args<double> &, cudaStream_t);
template int launch_pass1_simt<float>(const Pass1Args<float> &, cudaStream_t);
template int launch_pass2_simt<double>(const Pass2Args<double> &, int, cudaStream_t, bool);
template int launch_pass2_simt<float>(const Pass2Args<float> &, int, cudaStream_t, bool);

}  // namespace dgtm
