// ctemp_tc.cu -- the scatter of the AUTO schedule's critical temperature
// (comm/mpicomm.c:562-674, dagtm_mpi_next_ctemp_helper) as a tensor-core GEMM
// over pair features, for the split-BF16 form on 0/1 data.
//
// For centre k the reference needs S1_k = sum_n R_kn x x^T and
// S2_k = sum_n R_kn^2 x x^T with x = t_n - y_k.  Expanded about the origin,
//     S1_k = P_k - y_k a_k^T - a_k y_k^T + g_k y_k y_k^T,
//     P_k = sum_n R_kn t_n t_n^T,  a_k = sum_n R_kn t_n,  g_k = sum_n R_kn,
// and S2_k the same with R^2.  With u_n = (t_ni t_nj for i <= j, t_ni, 1) --
// D (D + 1) / 2 + D + 1 pair features, exact in BF16 for 0/1 data -- all of
// P_k, a_k, g_k are row k of the product R U, and those of S2 of R^2 U.  So
// the scatter is two GEMMs of K x N by N x (D(D+1)/2 + D + 1):
//   rplanes_kernel : per chunk of points, R and R^2 of every centre from the
//                    split-BF16 distance product (as the responsibility pass
//                    of the M-step forms R), each as BF16 hi + lo, to HBM;
//   upairs_kernel  : the chunk's pair features, transposed (feature rows);
//   pair_gemm      : Q += (R_hi + R_lo) U^T and Q2 += (R2_hi + R2_lo) U^T,
//                    tcgen05 with both operands from shared memory (TMA),
//                    FP32 accumulators in tensor memory, added into FP32
//                    running sums in HBM every 4096 points (the tensor
//                    pipe's FP32 accumulation drifts low over long runs of
//                    MMAs; the adds at L2 round to nearest);
//   assemble_kernel: S1, S2 of a batch of centres from Q, Q2 and Y (FP64),
//                    in the layout of the CUDA-core scatter, for the eigen
//                    filter of ctemp.cu.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"
#include "tc.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>

#include <vector>

namespace dgtm {

int make_tmap_bf16(CUtensorMap *map, const void *ptr, uint64_t rows, uint64_t cols, uint64_t ld,
                   uint32_t box_rows, uint32_t box_cols);
int launch_ctemp_eig(const CtempPlan &pl, int kb, int D, const double *S, void *Mg,
                     const double *gg, double lim_scale, double *out, cudaStream_t s);

using namespace sm100;

namespace {

constexpr int PANEL = 64;        // BF16 elements per 128-byte swizzle row
constexpr int SMEM_LIMIT = 227 * 1024;

__host__ __device__ constexpr int rup(int a, int b) { return (a + b - 1) / b * b; }

// ---------------------------------------------------------------------------
// R and R^2 planes of a chunk of points
// ---------------------------------------------------------------------------
constexpr int RP_THREADS = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 responsibilities
constexpr int RP_TILE = 64;      // points per tile (MMA N)
constexpr int RP_TILES = 32;     // tiles per CTA
constexpr int RP_BK = 128;       // centres per CTA (MMA M)

struct RPParams {
    int Kpad, Dp, n0, ntile, nc, nstage, N;  // chunk: points n0 .. n0 + nc, nc = 64 ntile
    const uint32_t *Yb;                      // 2 x Kpad x Dp BF16 (as pairs)
    const float4 *colq;
    const float *hcut;                       // N: (|t_n|^2 - dcut) / 2; R = 0 where acc below it
    float dcut;
    float *dmin;                             // Kpad: each centre's least distance (FP32)
    uint32_t *planes;                     // 4 x Kpad x nc BF16 (as pairs): R hi, R lo, R^2 hi, R^2 lo
    int *status;
};

template <int NP, int KL>
__global__ void __launch_bounds__(RP_THREADS, 1)
    rplanes_kernel(const __grid_constant__ CUtensorMap tmT, const RPParams p)
{
    constexpr int KS = 4 * (NP - 1) + KL;
    constexpr int DP = NP * PANEL;
    constexpr int YCOLS = (KS * 8 + 15) / 16 * 16;  // TMEM columns of one Y piece
    constexpr int Y_COL = 0;
    constexpr int S_COL = 2 * YCOLS;                // two 64-column S buffers
    static_assert(S_COL + 2 * RP_TILE <= 512, "tensor memory plan");
    constexpr int TPANEL = RP_TILE * 128;           // 8 KB
    constexpr int TSTAGE = NP * TPANEL;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int nstage = p.nstage;
    unsigned char *Tst = base;
    uint64_t *bars = (uint64_t *) (Tst + nstage * TSTAGE);
    uint64_t *t_full = bars;
    uint64_t *t_empty = bars + nstage;
    uint64_t *s_full = bars + 2 * nstage;  // 2
    uint64_t *s_free = s_full + 2;         // 2
    uint64_t *y_ready = s_free + 2;
    uint64_t *drain = y_ready + 1;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int kt = blockIdx.x;
    const int j0 = blockIdx.y * RP_TILES;
    const int j1 = min(p.ntile, j0 + RP_TILES);
    const int ntl = j1 - j0;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < nstage; s++) {
            mbar_init(&t_full[s], 1);
            mbar_init(&t_empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&s_full[b], 1);
            mbar_init(&s_free[b], 256);
        }
        mbar_init(y_ready, 256);
        mbar_init(drain, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_sh, 512);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = __shfl_sync(0xffffffffu, *tmem_sh, 0);

    if (warp == 0 && lane == 0) {
        // ---------------- producer: the chunk's point tiles ----------------
        prefetch_tmap(&tmT);
        for (int j = 0; j < ntl; j++) {
            const int s = j % nstage;
            if (j >= nstage && !mbar_wait(&t_empty[s], ((j / nstage) & 1) ^ 1u, p.status, 61)) {
                failed = 1;
                break;
            }
            mbar_expect_tx(&t_full[s], (uint32_t) TSTAGE);
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(Tst + s * TSTAGE + pn * TPANEL, &tmT, &t_full[s], PANEL * pn,
                            p.n0 + (j0 + j) * RP_TILE);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer: S = Y T^T (M = 128 centres, N = 64 points) ----------------
        const uint32_t id1 = idesc_bf16(RP_BK, RP_TILE, 0, 0);
        const uint64_t tdesc = sdesc_sw128(smem_u32(Tst), 16, 1024);
        bool ok = mbar_wait_w(y_ready, 0, p.status, 62);
        tc_fence_after();
        for (int j = 0; ok && j < ntl; j++) {
            const int s = j % nstage, b = j & 1;
            if (!mbar_wait_w(&t_full[s], (j / nstage) & 1, p.status, 63) ||
                (j >= 2 && !mbar_wait_w(&s_free[b], ((j - 2) >> 1) & 1, p.status, 64))) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t d = tmem + (uint32_t) (S_COL + b * RP_TILE);
            const uint64_t bd = tdesc + (uint64_t) (s * (TSTAGE >> 4));
#pragma unroll
            for (int piece = 0; piece < 2; piece++)
#pragma unroll
                for (int ks = 0; ks < KS; ks++)
                    mma_ts_w(d, tmem + (uint32_t) (Y_COL + piece * YCOLS + ks * 8),
                             bd + (uint64_t) ((ks / 4) * (TPANEL >> 4) + 2 * (ks % 4)), id1,
                             (piece | ks) ? 1u : 0u);
            mma_commit_w(&t_empty[s]);
            mma_commit_w(&s_full[b]);
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- the centres into tensor memory, then R and R^2 ----------------
        const int q = warp & 3;
        const int g = (warp - 2) >> 2;  // points 32 g .. 32 g + 31 of a tile; centre piece g
        const int row = q * 32 + lane;
        const int k = kt * RP_BK + row;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        {
            // group 0 loads Y hi, group 1 Y lo (column j: depths 2 j, 2 j + 1)
            const uint4 *src = (const uint4 *) (p.Yb + ((size_t) g * p.Kpad + k) * (DP / 2));
            uint4 x[YCOLS / 4];
#pragma unroll
            for (int i = 0; i < YCOLS / 4; i++)
                x[i] = src[i];
#pragma unroll
            for (int c0 = 0; c0 < YCOLS; c0 += 16) {
                uint32_t w[16];
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    w[4 * i] = x[c0 / 4 + i].x;
                    w[4 * i + 1] = x[c0 / 4 + i].y;
                    w[4 * i + 2] = x[c0 / 4 + i].z;
                    w[4 * i + 3] = x[c0 / 4 + i].w;
                }
                tmem_st16(lane_base + (uint32_t) (Y_COL + g * YCOLS + c0), w);
            }
            tmem_st_wait();
            tc_fence_before();
            mbar_arrive(y_ready);
        }
        const size_t plane = (size_t) p.Kpad * p.nc / 2;  // uint32 per plane
        uint32_t *out = p.planes + ((size_t) k * p.nc) / 2;
        float mx = -INFINITY;  // this row's largest acc - hcut over its points
        bool ok = true;
        for (int j = 0; j < ntl; j++) {
            const int b = j & 1;
            if (!mbar_wait(&s_full[b], (j >> 1) & 1, p.status, 65)) {
                ok = false;
                break;
            }
            tc_fence_after();
            uint32_t va[32];
            tmem_ld32(lane_base + (uint32_t) (S_COL + b * RP_TILE + g * 32), va);
            tmem_ld_wait();
            tc_fence_before();
            mbar_arrive(&s_free[b]);
            const int nl = (j0 + j) * RP_TILE + g * 32;  // point within the chunk
            const float4 *cq = p.colq + p.n0 + nl;
            // acc_kn below hcut_n: d_kn > dcut, where the reference's
            // exp(-beta d / 2) underflows (padding points: +inf, R = 0 anyway)
            float hc[32];
#pragma unroll
            for (int e = 0; e < 32; e++) {
                const int na = p.n0 + nl + e;
                hc[e] = (na < p.N) ? p.hcut[na] : INFINITY;
                mx = fmaxf(mx, __uint_as_float(va[e]) - hc[e]);
            }
#pragma unroll
            for (int pl = 0; pl < 4; pl++) {
                // plane pl: R hi, R lo, R^2 hi, R^2 lo; one plane at a time keeps
                // the registers down
                uint32_t w[16];
#pragma unroll
                for (int e = 0; e < 16; e++) {
                    const float4 c0 = cq[2 * e], c1 = cq[2 * e + 1];
                    float r0 = ex2(fmaf(__uint_as_float(va[2 * e]) - c0.x, c0.y, -c0.z));
                    float r1 = ex2(fmaf(__uint_as_float(va[2 * e + 1]) - c1.x, c1.y, -c1.z));
                    if (__uint_as_float(va[2 * e]) < hc[2 * e])
                        r0 = 0.f;
                    if (__uint_as_float(va[2 * e + 1]) < hc[2 * e + 1])
                        r1 = 0.f;
                    if (pl >= 2) {
                        r0 *= r0;
                        r1 *= r1;
                    }
                    const uint32_t h = pack_bf16(r0, r1);
                    w[e] = (pl & 1) ? pack_bf16(r0 - bf16lo_to_f32(h), r1 - bf16hi_to_f32(h)) : h;
                }
                uint4 *dst = (uint4 *) (out + pl * plane + nl / 2);
#pragma unroll
                for (int i = 0; i < 4; i++)
                    dst[i] = make_uint4(w[4 * i], w[4 * i + 1], w[4 * i + 2], w[4 * i + 3]);
            }
        }
        // d_min = dcut - 2 max(acc - hcut); non-negative floats order like
        // their bit patterns
        if (mx > -INFINITY)
            atomicMin((int *) &p.dmin[k], __float_as_int(fmaxf(p.dcut - 2.0f * mx, 0.f)));
        if (!ok)
            failed = 1;
    }
    __syncthreads();
    if (failed && warp == 1) {
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 66, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

using RPKernel = void (*)(const CUtensorMap, const RPParams);

RPKernel rplanes_for(int np, int kl)
{
#define DGTM_RP(NP_, KL_) \
    if (np == NP_ && kl == KL_) return rplanes_kernel<NP_, KL_>;
    DGTM_RP(1, 1) DGTM_RP(1, 2) DGTM_RP(1, 3) DGTM_RP(1, 4)
    DGTM_RP(2, 1) DGTM_RP(2, 2) DGTM_RP(2, 3) DGTM_RP(2, 4)
    DGTM_RP(3, 1) DGTM_RP(3, 2) DGTM_RP(3, 3) DGTM_RP(3, 4)
#undef DGTM_RP
    return nullptr;
}

// (|t_n|^2 - dcut) / 2 in FP32: acc_kn below it means d_kn > dcut
__global__ void hcut_kernel(const double *__restrict__ tt, int N, double dcut, float *__restrict__ h)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n < N)
        h[n] = (float) (0.5 * (tt[n] - dcut));
}

// ---------------------------------------------------------------------------
// pair features of a chunk, transposed: U[f][n] for the chunk's points
// ---------------------------------------------------------------------------
constexpr int UP_PTS = 64;    // points per block
constexpr int UP_FEAT = 256;  // features per block (one per thread)

// f < npair: t_i t_j (i <= j, from `pairs`); then t_i; then 1; then 0 (padding)
__global__ void __launch_bounds__(UP_FEAT) upairs_kernel(const __nv_bfloat16 *__restrict__ Tb,
                                                         int Dp, int D, int n0, int nc, int npair,
                                                         const ushort2 *__restrict__ pairs,
                                                         int DUpad, __nv_bfloat16 *__restrict__ U)
{
    extern __shared__ __align__(16) __nv_bfloat16 tsh[];  // UP_PTS x Dp
    const int p0 = blockIdx.x * UP_PTS;
    for (int e = threadIdx.x; e < UP_PTS * Dp / 8; e += blockDim.x) {
        const int pt = e / (Dp / 8), c8 = e % (Dp / 8);
        reinterpret_cast<uint4 *>(tsh)[e] =
            reinterpret_cast<const uint4 *>(Tb + (size_t) (n0 + p0 + pt) * Dp)[c8];
    }
    __syncthreads();
    const int f = blockIdx.y * UP_FEAT + threadIdx.x;
    if (f >= DUpad)
        return;
    int i = -1, j = -1;
    float c = 0.f;
    if (f < npair) {
        const ushort2 ij = pairs[f];
        i = ij.x;
        j = ij.y;
    } else if (f < npair + D) {
        i = f - npair;
    } else if (f == npair + D) {
        c = 1.f;
    }
    uint4 *dst = reinterpret_cast<uint4 *>(U + (size_t) f * nc + p0);
#pragma unroll
    for (int b = 0; b < UP_PTS / 8; b++) {
        uint32_t w[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            float v[2];
#pragma unroll
            for (int z = 0; z < 2; z++) {
                const int pt = 8 * b + 2 * h + z;
                const __nv_bfloat16 *tr = tsh + (size_t) pt * Dp;
                if (i < 0)
                    v[z] = c;
                else if (j < 0)
                    v[z] = __bfloat162float(tr[i]);
                else
                    v[z] = __bfloat162float(tr[i]) * __bfloat162float(tr[j]);
            }
            w[h] = pack_bf16(v[0], v[1]);
        }
        dst[b] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// ---------------------------------------------------------------------------
// the pair GEMM: Q += R U^T, Q2 += R^2 U^T over a chunk
// ---------------------------------------------------------------------------
constexpr int PG_THREADS = 192;  // warp 0 TMA, warp 1 MMA, warps 2-5 move the accumulators
constexpr int PG_M = 128;        // centres per tile
constexpr int PG_N = 256;        // pair features per tile
constexpr int PG_KB = 64;        // points per stage
constexpr int PG_SEG = 64;       // stages per accumulation segment (4096 points)
constexpr int PG_ABYTES = PG_M * 128;             // one plane's 128 x 64 tile
constexpr int PG_BBYTES = PG_N * 128;             // the features' 256 x 64 tile
constexpr int PG_STAGE = 4 * PG_ABYTES + PG_BBYTES;
constexpr int PG_NSTAGE = 2;

struct PGParams {
    int Kpad, DUpad, nkb, ftiles, nunits;
    float *Q;  // 2 x Kpad x DUpad: sums with R, then with R^2
    int *status;
};

__global__ void __launch_bounds__(PG_THREADS, 1)
    pair_gemm_kernel(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                     const PGParams p)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    uint64_t *bars = (uint64_t *) (base + PG_NSTAGE * PG_STAGE);
    uint64_t *full = bars;
    uint64_t *empty = bars + PG_NSTAGE;
    uint64_t *acc_full = bars + 2 * PG_NSTAGE;
    uint64_t *acc_free = acc_full + 1;
    uint64_t *drain = acc_free + 1;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    __shared__ int failed;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nseg = (p.nkb + PG_SEG - 1) / PG_SEG;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < PG_NSTAGE; s++) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(acc_full, 1);
        mbar_init(acc_free, 128);
        mbar_init(drain, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_sh, 512);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = __shfl_sync(0xffffffffu, *tmem_sh, 0);

    if (warp == 0 && lane == 0) {
        // ---------------- producer ----------------
        prefetch_tmap(&tmA);
        prefetch_tmap(&tmB);
        int it = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            const int kt = v / p.ftiles, ft = v % p.ftiles;
            for (int kb = 0; kb < p.nkb; kb++, it++) {
                const int s = it % PG_NSTAGE;
                if (it >= PG_NSTAGE &&
                    !mbar_wait(&empty[s], ((it / PG_NSTAGE) & 1) ^ 1u, p.status, 71)) {
                    ok = false;
                    break;
                }
                unsigned char *st = base + s * PG_STAGE;
                mbar_expect_tx(&full[s], (uint32_t) PG_STAGE);
#pragma unroll
                for (int q = 0; q < 4; q++)
                    tma_load_2d(st + q * PG_ABYTES, &tmA, &full[s], kb * PG_KB,
                                q * p.Kpad + kt * PG_M);
                tma_load_2d(st + 4 * PG_ABYTES, &tmB, &full[s], kb * PG_KB, ft * PG_N);
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        const uint32_t idesc = idesc_bf16(PG_M, PG_N, 0, 0);
        const uint64_t d0 = sdesc_sw128(smem_u32(base), 16, 1024);
        int it = 0, seg = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            for (int kb = 0; kb < p.nkb; kb++, it++) {
                const int s = it % PG_NSTAGE;
                const bool seg_start = (kb % PG_SEG) == 0;
                if (!mbar_wait_w(&full[s], (it / PG_NSTAGE) & 1, p.status, 72) ||
                    (seg_start && seg > 0 && !mbar_wait_w(acc_free, (seg - 1) & 1, p.status, 73))) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint64_t sd = d0 + (uint64_t) (s * (PG_STAGE >> 4));
#pragma unroll
                for (int q = 0; q < 4; q++)
#pragma unroll
                    for (int kk = 0; kk < PG_KB / 16; kk++)
                        // q = 0, 1: R hi, lo into Q (columns 0..255); q = 2, 3: R^2 into Q2
                        mma_ss_w(tmem + (uint32_t) ((q >> 1) * PG_N),
                                 sd + (uint64_t) (q * (PG_ABYTES >> 4) + 2 * kk),
                                 sd + (uint64_t) (4 * (PG_ABYTES >> 4) + 2 * kk), idesc,
                                 (!seg_start || (q & 1) || kk) ? 1u : 0u);
                mma_commit_w(&empty[s]);
                if ((kb % PG_SEG) == PG_SEG - 1 || kb == p.nkb - 1) {
                    mma_commit_w(acc_full);
                    seg++;
                }
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- accumulators to the running sums (one centre row per thread) ----------------
        const int q = warp & 3;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        int seg = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            const int kt = v / p.ftiles, ft = v % p.ftiles;
            for (int sg = 0; sg < nseg; sg++, seg++) {
                if (!mbar_wait(acc_full, seg & 1, p.status, 74)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
#pragma unroll 1
                for (int c0 = 0; c0 < 2 * PG_N; c0 += 32) {
                    uint32_t x[32];
                    tmem_ld32(lane_base + (uint32_t) c0, x);
                    tmem_ld_wait();
                    float *dst = p.Q +
                                 ((size_t) (c0 / PG_N) * p.Kpad + (size_t) kt * PG_M + row) * p.DUpad +
                                 (size_t) ft * PG_N + (c0 % PG_N);
#pragma unroll
                    for (int e = 0; e < 32; e += 4)
                        red_add_f32x4(dst + e, __uint_as_float(x[e]), __uint_as_float(x[e + 1]),
                                      __uint_as_float(x[e + 2]), __uint_as_float(x[e + 3]));
                }
                tc_fence_before();
                mbar_arrive(acc_free);
            }
        }
        if (!ok)
            failed = 1;
    }
    __syncthreads();
    if (failed && warp == 1) {
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 75, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// S1 and S2 of a batch of centres from the sums (FP64), upper triangles in
// the layout of the CUDA-core scatter: per centre S1 (D x D) then S2.
// ---------------------------------------------------------------------------
__global__ void assemble_kernel(const float *__restrict__ Q, int Kpad, int DUpad, int D, int npair,
                                const ushort2 *__restrict__ pairs, const double *__restrict__ Y,
                                int k0, double *__restrict__ S, double *__restrict__ gsum)
{
    const int kl = blockIdx.x, k = k0 + kl;
    const float *q1 = Q + (size_t) k * DUpad, *q2 = Q + ((size_t) Kpad + k) * DUpad;
    const double *y = Y + (size_t) k * D;
    const double g1 = (double) q1[npair + D], g2 = (double) q2[npair + D];
    if (threadIdx.x == 0)
        gsum[kl] = g1;
    double *S1 = S + (size_t) kl * 2 * D * D, *S2 = S1 + (size_t) D * D;
    for (int f = threadIdx.x; f < npair; f += blockDim.x) {
        const ushort2 ij = pairs[f];
        const int i = ij.x, j = ij.y;
        const double yi = y[i], yj = y[j];
        const double a1i = q1[npair + i], a1j = q1[npair + j];
        const double a2i = q2[npair + i], a2j = q2[npair + j];
        S1[(size_t) i * D + j] = (double) q1[f] - yi * a1j - a1i * yj + g1 * yi * yj;
        S2[(size_t) i * D + j] = (double) q2[f] - yi * a2j - a2i * yj + g2 * yi * yj;
    }
}

}  // namespace

int tc_ctemp_pairs(const TcView &v, const double *Y64, const double *gg_dev, double lim_scale,
                   size_t budget, double dcut, double *gsum_dev, double *out_dev, float *dmin_dev,
                   cudaStream_t s)
{
    const int N = v.N, D = v.D, K = v.K;
    if (!v.binary || v.nT != 1 || v.npanel > 3) {
        set_error(DGTM_ENOTSUP, "the pair-feature scatter needs 0/1 data and D <= 189");
        return DGTM_ENOTSUP;
    }
    const int npair = D * (D + 1) / 2;
    const int DU = npair + D + 1;
    const int DUpad = rup(DU, PG_N);
    const int Kpad = v.Kpad;  // a multiple of 128
    const int ktiles = Kpad / PG_M, ftiles = DUpad / PG_N;
    // points per chunk: a multiple of 4096 within the budget (R planes 8 B and
    // features 2 B per element), at most the padded point count
    const size_t qbytes = sizeof(float) * 2 * (size_t) Kpad * DUpad;
    const size_t per_point = 8 * (size_t) Kpad + 2 * (size_t) DUpad;
    long nc_max = budget > qbytes ? (long) ((budget - qbytes) / per_point) : 0;
    nc_max = nc_max / 4096 * 4096;
    if (nc_max < 4096)
        nc_max = 4096;
    const int nc_cap = (int) (nc_max < v.Npad ? nc_max : v.Npad);
    // the eigen batches: centres whose S1, S2 fit 1/4 of the budget
    const CtempPlan pl = ctemp_plan(N, D, K, true, true, budget / 4, 1);
    const size_t sbytes = sizeof(double) * 2 * (size_t) D * D;
    const int kb = pl.kb;
    // the batch's S1, S2 (FP64), then the FP32 matrices of the eigenvalue step
    // when they do not fit shared memory
    const size_t s_at = (sbytes * kb + 255) / 256 * 256;
    const size_t mg_bytes = pl.eig_in_smem ? 0 : sizeof(float) * 2 * (size_t) D * D * kb;

    float *Q = nullptr;
    uint32_t *planes = nullptr;
    __nv_bfloat16 *U = nullptr;
    ushort2 *pairs = nullptr;
    float *hcut = nullptr;
    void *sbuf = nullptr;
    int rc = DGTM_OK;
    cudaError_t e = cudaMalloc((void **) &Q, qbytes);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &planes, 8 * (size_t) Kpad * nc_cap);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &U, 2 * (size_t) DUpad * nc_cap);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &pairs, sizeof(ushort2) * (size_t) npair);
    if (e == cudaSuccess)
        e = cudaMalloc(&sbuf, s_at + mg_bytes + 256);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &hcut, sizeof(float) * (size_t) N);
    auto cleanup = [&]() {
        cudaFree(Q);
        cudaFree(planes);
        cudaFree(U);
        cudaFree(pairs);
        cudaFree(sbuf);
        cudaFree(hcut);
    };
    if (e != cudaSuccess) {
        cleanup();
        set_error(DGTM_ENOMEM, "tc_ctemp_pairs: %s", cudaGetErrorString(e));
        return DGTM_ENOMEM;
    }
    {
        std::vector<ushort2> h((size_t) npair);
        size_t f = 0;
        for (int i = 0; i < D; i++)
            for (int j = i; j < D; j++)
                h[f++] = make_ushort2((unsigned short) i, (unsigned short) j);
        e = cudaMemcpyAsync(pairs, h.data(), sizeof(ushort2) * npair, cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = cudaMemsetAsync(Q, 0, qbytes, s);
        if (e == cudaSuccess)  // 0x7F7F7F7F: 3.4e38, above every distance
            e = cudaMemsetAsync(dmin_dev, 0x7F, sizeof(float) * (size_t) Kpad, s);
        if (e == cudaSuccess) {
            hcut_kernel<<<(N + 255) / 256, 256, 0, s>>>(v.tt, N, dcut, hcut);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaStreamSynchronize(s);  // the host table is freed here
    }
    // kernels and their shared-memory plans
    const int klast = v.ksteps - 4 * (v.npanel - 1);
    RPKernel rpk = rplanes_for(v.npanel, klast);
    const size_t tstage = (size_t) v.npanel * RP_TILE * 128;
    int rp_stages = (int) ((SMEM_LIMIT - 1024 - 256) / tstage);
    if (rp_stages > 8)
        rp_stages = 8;
    const size_t rp_smem = 1024 + (size_t) rp_stages * tstage + 256;
    const size_t pg_smem = 1024 + (size_t) PG_NSTAGE * PG_STAGE + 256;
    const size_t up_smem = sizeof(__nv_bfloat16) * (size_t) UP_PTS * v.Dp;
    if (e == cudaSuccess && !rpk)
        e = cudaErrorInvalidValue;
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(rpk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) rp_smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(pair_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) pg_smem);
    if (e != cudaSuccess) {
        cleanup();
        set_error(DGTM_ECUDA, "tc_ctemp_pairs: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    int dev = 0, sms = 148;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    CUtensorMap tmT, tmA, tmB;
    if ((rc = make_tmap_bf16(&tmT, v.Tb, (uint64_t) v.Npad, v.Dp, v.Dp, RP_TILE, PANEL)) != DGTM_OK) {
        cleanup();
        return rc;
    }
    for (int n0 = 0; n0 < v.Npad && rc == DGTM_OK; n0 += nc_cap) {
        const int nc = (v.Npad - n0 < nc_cap) ? v.Npad - n0 : nc_cap;  // a multiple of 256
        if ((rc = make_tmap_bf16(&tmA, planes, 4 * (uint64_t) Kpad, nc, nc, PG_M, PG_KB)) != DGTM_OK ||
            (rc = make_tmap_bf16(&tmB, U, (uint64_t) DUpad, nc, nc, PG_N, PG_KB)) != DGTM_OK)
            break;
        RPParams rp;
        rp.Kpad = Kpad;
        rp.Dp = v.Dp;
        rp.n0 = n0;
        rp.ntile = nc / RP_TILE;
        rp.nc = nc;
        rp.nstage = rp_stages;
        rp.Yb = (const uint32_t *) v.Yb;
        rp.colq = v.colq;
        rp.N = v.N;
        rp.hcut = hcut;
        rp.dcut = (float) dcut;
        rp.dmin = dmin_dev;
        rp.planes = planes;
        rp.status = v.status;
        rpk<<<dim3(ktiles, (rp.ntile + RP_TILES - 1) / RP_TILES), RP_THREADS, rp_smem, s>>>(tmT, rp);
        upairs_kernel<<<dim3(nc / UP_PTS, DUpad / UP_FEAT), UP_FEAT, up_smem, s>>>(
            (const __nv_bfloat16 *) v.Tb, v.Dp, D, n0, nc, npair, pairs, DUpad, U);
        PGParams pg;
        pg.Kpad = Kpad;
        pg.DUpad = DUpad;
        pg.nkb = nc / PG_KB;
        pg.ftiles = ftiles;
        pg.nunits = ktiles * ftiles;
        pg.Q = Q;
        pg.status = v.status;
        pair_gemm_kernel<<<pg.nunits < sms ? pg.nunits : sms, PG_THREADS, pg_smem, s>>>(tmA, tmB, pg);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(DGTM_ECUDA, "tc_ctemp_pairs: %s", cudaGetErrorString(e));
            rc = DGTM_ECUDA;
        }
    }
    for (int k0 = 0; rc == DGTM_OK && k0 < K; k0 += kb) {
        const int nb = (K - k0 < kb) ? K - k0 : kb;
        assemble_kernel<<<nb, 256, 0, s>>>(Q, Kpad, DUpad, D, npair, pairs, Y64, k0,
                                           (double *) sbuf, gsum_dev + k0);
        e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(DGTM_ECUDA, "tc_ctemp_pairs: %s", cudaGetErrorString(e));
            rc = DGTM_ECUDA;
            break;
        }
        rc = launch_ctemp_eig(pl, nb, D, (const double *) sbuf,
                              pl.eig_in_smem ? nullptr : (char *) sbuf + s_at,
                              gg_dev ? gg_dev + k0 : gsum_dev + k0, lim_scale,
                              out_dev + (size_t) 2 * k0, s);
    }
    if (rc == DGTM_OK)
        e = cudaStreamSynchronize(s);
    cleanup();
    if (rc == DGTM_OK && e != cudaSuccess) {
        set_error(DGTM_ECUDA, "tc_ctemp_pairs: %s", cudaGetErrorString(e));
        rc = DGTM_ECUDA;
    }
    return rc;
}

}  // namespace dgtm
