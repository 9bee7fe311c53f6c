// estep_tc.cu -- split-BF16 tensor-core form of the E-step and of the
// responsibility pass of the M-step (tcgen05 + TMA + TMEM, sm_103a).
//
// Operands.  The distance d_kn = |y_k|^2 + |t_n|^2 - 2 y_k.t_n is never formed
// directly: the contraction computes
//     acc_kn = y_k.t_n - |y_k|^2 / 2 = (|t_n|^2 - d_kn) / 2
// by appending three columns to both operands (T: 1, 1, 1; Y: the BF16
// pieces of -|y_k|^2/2), so -beta d_kn / 2 = beta acc_kn - beta |t_n|^2 / 2
// and the per-point term cancels inside every normalisation.  Y is split
// into y = hi + lo (two BF16 pieces, ~16 significant bits); T is split the
// same way unless every value is exactly representable in BF16 (0/1 data),
// in which case the third product Y_hi T_lo vanishes and is skipped.
// Products accumulate in FP32 in tensor memory; column statistics and every
// cross-block reduction are FP64.  |y|^2 is taken from the split centres so
// that acc is exact for the rounded Y, and the minimum distance of each point
// (the term that dominates its log-sum-exp) is recomputed in FP32 from the
// unsplit centre.
//
// Pass 1 (one CTA per two 128-point tiles, or one tile when the data are
// split): the data tiles are copied once into tensor memory as the MMA A
// operand; warp 0 streams 128-centre x 64-depth BF16 panels of Y through a
// TMA ring, warp 1 issues tcgen05.mma (M = 128 points, N = 128 centres,
// K = 16, A from tensor memory) into one 128-column accumulator per tile,
// warps 2-9 (one 4-warp group per tile, one thread per point = one TMEM lane)
// copy each finished chunk to registers, release the accumulator and run the
// online log-sum-exp over k at temperature 1 and at `temp`.
//
// Pass 2 (persistent, units of (128 centres) x 16384 points): the CTA
// keeps its 128 centres resident, streams 64-point T tiles, recomputes
// acc (M = 128 centres, N = 64 points), turns it into R_kn with the pass-1
// statistics, writes R as BF16 hi/lo back into tensor memory and multiplies
// R by the same T tile read MN-major (M = 128, N = D padded, K = 16 points),
// accumulating R T (and, through the column of ones, G = rowsum R) in TMEM.
// Every unit's FP32 R T is written to its own slot; a fixed-order FP64 sum
// over the slots gives RT and G.
#include "common.cuh"
#include "sm100.cuh"
#include "tc.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>

namespace dgtm {

int make_tmap_bf16(CUtensorMap *map, const void *ptr, uint64_t rows, uint64_t cols, uint64_t ld,
                   uint32_t box_rows, uint32_t box_cols);

using namespace sm100;

namespace {

constexpr int P1_THREADS = 320;       // warp 0 TMA, warp 1 MMA, warps 2-9 statistics
constexpr int P2_THREADS = 320;       // warp 0 TMA, warp 1 MMA, warps 2-9 responsibilities
constexpr int P1_TILE = 128;          // points per tile (MMA M); a CTA holds 1 or 2 tiles
constexpr int P1_BK = 128;            // centres per chunk (MMA N)
constexpr int PANEL_ELEMS = 64;       // BF16 elements per 128-byte swizzle row
constexpr int P2_BK = 128;            // centres per CTA (MMA M)
constexpr int P2_UNIT_POINTS = 16384; // points per output slot
constexpr int NPAD_ALIGN = 256;       // point padding (two pass-1 tiles)
constexpr float LOG2E = 1.4426950408889634f;
constexpr int SMEM_LIMIT = 227 * 1024;

__host__ __device__ constexpr int round_up(int a, int b) { return (a + b - 1) / b * b; }

struct P1Params {
    int N, D, Dp, npanel, nT, Npad, Kpad, K, nchunk, nstage, ntile;
    int ksteps;           // 16-deep MMA steps covering the D + 3 used columns
    float c1l, c2l;       // beta log2(e), beta/temp log2(e)
    double c1, c2;        // beta/2, beta/(2 temp)
    int isDA, two_temps;  // two_temps: isDA and temp != 1
    const float *Y32;     // K x D
    const double *T64;    // N x D (exact data, read when T is split in two pieces)
    const uint32_t *Tb;   // nT x Npad x Dp BF16 (as BF16 pairs)
    double2 *colstat;     // N
    float4 *colq;         // Npad
    double *part;         // 2 per CTA
    int *status;
};

// TMEM map of pass 1: the point tiles (MMA operand A, BF16 pairs) from column
// 0, the two 128-column accumulators at columns 256 and 384.
constexpr int P1_ACC_COL = 256;

// ---------------------------------------------------------------------------
// pass 1: one CTA per NTILE x 128 points.  The data tiles live in tensor
// memory as the A operand; shared memory holds only the Y ring.  NTILE = 2
// (data exact in BF16): each tile owns one accumulator and the two tiles
// ping-pong, so the tensor pipe works on one tile while the statistics warps
// read the other.  NTILE = 1 (data split in two BF16 pieces): one tile
// double-buffers the two accumulators.
//
// The kernel is a template on the operand shape -- NP 64-deep panels, KL
// 16-deep steps used in the last one, NT data pieces -- so that the MMA
// sequence of a chunk is straight-line code with constant operand offsets.
// One warp issues; a loop that recomputes descriptors per MMA cannot keep
// the tensor pipe busy at N = 128.  The Y ring is in slots of one piece
// (hi or lo) of a 128-centre chunk, NP panels of 16 KB each.
// ---------------------------------------------------------------------------
template <int NP, int KL, int NT>
__global__ void __launch_bounds__(P1_THREADS, 1)
    tc_pass1_kernel(const __grid_constant__ CUtensorMap tmY, const P1Params p)
{
    constexpr int NTILE = (NT == 1) ? 2 : 1;
    constexpr int ACOL = NP * 32;                      // TMEM columns of one data piece
    constexpr int PANEL_BYTES = P1_BK * 128;           // 16 KB
    constexpr int SLOT_BYTES = NP * PANEL_BYTES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int nslot = p.nstage;
    unsigned char *Yslot = base;
    uint64_t *bars = (uint64_t *) (Yslot + nslot * SLOT_BYTES);
    uint64_t *y_full = bars;
    uint64_t *y_empty = bars + nslot;
    uint64_t *a_ready = bars + 2 * nslot;
    uint64_t *acc_full = a_ready + 1;   // [region]
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *drain = acc_empty + 2;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    double *red = (double *) (tmem_sh + 2);            // 2 x 256
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * NTILE * P1_TILE;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < nslot; s++) {
            mbar_init(&y_full[s], 1);
            mbar_init(&y_empty[s], 1);
        }
        mbar_init(a_ready, 128 * NTILE);
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            mbar_init(&acc_empty[b], 128);
        }
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
    // accumulator region and its use count for (tile g, chunk c)
    auto region = [&](int g, int c) { return NTILE == 2 ? g : (c & 1); };
    auto ruse = [&](int c) { return NTILE == 2 ? c : (c >> 1); };

    if (warp == 0 && lane == 0) {
        // ---------------- producer: the Y ring, one piece of a chunk per slot ----------------
        prefetch_tmap(&tmY);
        int q = 0;
        uint32_t ph = 0;
        for (int it = 0; it < 2 * p.nchunk; it++) {
            if (it >= nslot && !mbar_wait(&y_empty[q], ph ^ 1u, p.status, 11)) {
                failed = 1;
                break;
            }
            const int c = it >> 1, piece = it & 1;
            mbar_expect_tx(&y_full[q], (uint32_t) SLOT_BYTES);
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(Yslot + q * SLOT_BYTES + pn * PANEL_BYTES, &tmY, &y_full[q],
                            PANEL_ELEMS * pn, piece * p.Kpad + c * P1_BK);
            if (++q == nslot) {
                q = 0;
                ph ^= 1u;
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (whole warp; one elected lane issues) ----------------
        const uint32_t idesc = idesc_bf16(P1_TILE, P1_BK, 0, 0);
        const uint64_t ydesc0 = sdesc_sw128(smem_u32(Yslot), 16, 1024);
        bool ok = mbar_wait_w(a_ready, 0, p.status, 12);
        int q0 = 0;
        uint32_t ph0 = 0;
        for (int c = 0; ok && c < p.nchunk; c++) {
            int q = q0;
            uint32_t ph = ph0;
#pragma unroll
            for (int g = 0; g < NTILE; g++) {
                const int rg = region(g, c), use = ruse(c);
                if (use > 0 && !mbar_wait_w(&acc_empty[rg], (use - 1) & 1, p.status, 13)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t d_tmem = tmem + (uint32_t) (P1_ACC_COL + rg * P1_BK);
                const uint32_t a_tile = tmem + (uint32_t) (g * NT * ACOL);
                q = q0;
                ph = ph0;
#pragma unroll
                for (int piece = 0; piece < 2; piece++) {
                    if (g == 0) {
                        if (!mbar_wait_w(&y_full[q], ph, p.status, 14)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint64_t bd = ydesc0 + (uint64_t) (q * (SLOT_BYTES >> 4));
                    // Y_hi pairs with T_hi (and T_lo when T is split); Y_lo with T_hi
#pragma unroll
                    for (int pn = 0; pn < NP; pn++) {
#pragma unroll
                        for (int tp = 0; tp < (piece == 0 ? NT : 1); tp++) {
#pragma unroll
                            for (int kk = 0; kk < (pn == NP - 1 ? KL : 4); kk++)
                                mma_ts_w(d_tmem, a_tile + (uint32_t) (tp * ACOL + pn * 32 + kk * 8),
                                         bd + (uint64_t) (pn * (PANEL_BYTES >> 4) + 2 * kk), idesc,
                                         (piece | pn | tp | kk) ? 1u : 0u);
                        }
                    }
                    if (g == NTILE - 1)
                        mma_commit_w(&y_empty[q]);
                    if (++q == nslot) {
                        q = 0;
                        ph ^= 1u;
                    }
                }
                if (!ok)
                    break;
                mma_commit_w(&acc_full[rg]);
            }
            q0 = q;
            ph0 = ph;
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- statistics: one 4-warp group per point tile ----------------
        const int q = warp & 3;
        const int g = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        const int prow = g * P1_TILE + row;
        const int n = n0 + prow;
        double t1 = 0.0, t2 = 0.0;
        bool ok = true;
        if (g < NTILE) {
            // this thread's data row into tensor memory (A operand): column j of
            // piece tp holds depths 2j (low half) and 2j + 1
            for (int tp = 0; tp < NT; tp++) {
                const uint4 *src = (const uint4 *) (p.Tb + ((size_t) tp * p.Npad + n) * ACOL);
                for (int c0 = 0; c0 < ACOL; c0 += 16) {
                    uint32_t v[16];
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const uint4 w = src[c0 / 4 + j];
                        v[4 * j] = w.x;
                        v[4 * j + 1] = w.y;
                        v[4 * j + 2] = w.z;
                        v[4 * j + 3] = w.w;
                    }
                    tmem_st16(lane_base + (uint32_t) ((g * NT + tp) * ACOL + c0), v);
                }
            }
            tmem_st_wait();
            tc_fence_before();
            mbar_arrive(a_ready);

            float m = -INFINITY;
            int kstar = 0;
            double s1 = 0.0, s2 = 0.0;
            for (int c = 0; c < p.nchunk; c++) {
                const int rg = region(g, c);
                if (!mbar_wait(&acc_full[rg], ruse(c) & 1, p.status, 15)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // copy the whole chunk out and hand the accumulator back at
                // once, so the next chunk's MMAs overlap this arithmetic
                uint32_t v[P1_BK];
                {
                    const uint32_t col = lane_base + (uint32_t) (P1_ACC_COL + rg * P1_BK);
                    tmem_ld32p(col, v);
                    tmem_ld32p(col + 32, v + 32);
                    tmem_ld32p(col + 64, v + 64);
                    tmem_ld32p(col + 96, v + 96);
                    tmem_ld_wait();
                }
                tc_fence_before();
                mbar_arrive(&acc_empty[rg]);
                float mxq[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
#pragma unroll
                for (int j = 0; j < P1_BK; j += 4) {
                    mxq[0] = fmaxf(mxq[0], __uint_as_float(v[j]));
                    mxq[1] = fmaxf(mxq[1], __uint_as_float(v[j + 1]));
                    mxq[2] = fmaxf(mxq[2], __uint_as_float(v[j + 2]));
                    mxq[3] = fmaxf(mxq[3], __uint_as_float(v[j + 3]));
                }
                const float mx = fmaxf(fmaxf(mxq[0], mxq[1]), fmaxf(mxq[2], mxq[3]));
                if (mx > m) {
                    if (m > -INFINITY) {
                        s1 *= (double) ex2((m - mx) * p.c1l);
                        s2 *= (double) ex2((m - mx) * p.c2l);
                    }
                    int j0 = P1_BK;
#pragma unroll
                    for (int j = P1_BK - 1; j >= 0; j--) {
                        if (__uint_as_float(v[j]) == mx)
                            j0 = j;
                    }
                    m = mx;
                    kstar = c * P1_BK + j0;
                }
                // four independent accumulation chains per sum
                float e1[4] = {0.f, 0.f, 0.f, 0.f}, e2[4] = {0.f, 0.f, 0.f, 0.f};
                if (p.two_temps) {
#pragma unroll
                    for (int j = 0; j < P1_BK; j += 4) {
#pragma unroll
                        for (int u = 0; u < 4; u++) {
                            const float x = __uint_as_float(v[j + u]) - m;
                            e1[u] += ex2(x * p.c1l);
                            e2[u] += ex2(x * p.c2l);
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < P1_BK; j += 4) {
#pragma unroll
                        for (int u = 0; u < 4; u++)
                            e1[u] += ex2((__uint_as_float(v[j + u]) - m) * p.c1l);
                    }
                }
                s1 += (double) ((e1[0] + e1[1]) + (e1[2] + e1[3]));
                s2 += (double) ((e2[0] + e2[1]) + (e2[2] + e2[3]));
            }
            if (!p.two_temps)
                s2 = s1;
            // exact (FP32) distance to the best centre, from the unsplit centre
            // and the data, then the per-point terms
            if (ok && n < p.N) {
                const int k = min(kstar, p.K - 1);
                const float *yk = p.Y32 + (size_t) k * p.D;
                float dsum = 0.f;
                if (NT == 1) {
                    // the data are exact in BF16
                    const uint32_t *tr = p.Tb + (size_t) n * ACOL;
                    for (int d = 0; d < p.D; d += 2) {
                        const uint32_t w = tr[d / 2];
                        const float df0 = yk[d] - __uint_as_float(w << 16);
                        dsum = fmaf(df0, df0, dsum);
                        if (d + 1 < p.D) {
                            const float df1 = yk[d + 1] - __uint_as_float(w & 0xFFFF0000u);
                            dsum = fmaf(df1, df1, dsum);
                        }
                    }
                } else {
                    const double *tn = p.T64 + (size_t) n * p.D;
                    for (int d = 0; d < p.D; d++) {
                        const float df = yk[d] - (float) tn[d];
                        dsum = fmaf(df, df, dsum);
                    }
                }
                const double dstar = (double) dsum;
                const double ls1 = log(s1), ls2 = log(s2);
                const double ls_sel = p.isDA ? ls2 : ls1;
                const double c_sel = p.isDA ? p.c2 : p.c1;
                t1 = -p.c1 * dstar + ls1;
                t2 = p.isDA ? (-p.c2 * dstar + ls2) : 0.0;
                double lsn = ls_sel;
                float4 cq = make_float4(m, (float) (2.0 * c_sel) * LOG2E,
                                        (float) (ls_sel * 1.4426950408889634), 0.f);
                // comm/mpicomm.c:382-389 zero-column fallback
                if (exp(-p.c1 * dstar) == 0.0) {
                    lsn = NAN;
                    if (p.isDA) {
                        t1 = -INFINITY;
                        t2 = log((double) p.K);
                    } else {
                        t1 = log((double) p.K);
                    }
                    cq = make_float4(0.f, 0.f, (float) log2((double) p.K), 0.f);
                }
                p.colstat[n] = make_double2(dstar, lsn);
                p.colq[n] = cq;
            } else if (n < p.Npad) {
                p.colq[n] = make_float4(0.f, 0.f, INFINITY, 0.f);  // padding: R = 0
            }
            if (!ok)
                failed = 1;
        }
        red[g * P1_TILE + row] = t1;
        red[256 + g * P1_TILE + row] = t2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b2 = 0.0;
        for (int i = 0; i < NTILE * P1_TILE; i++) {
            a += red[i];
            b2 += red[256 + i];
        }
        p.part[2 * blockIdx.x] = a;
        p.part[2 * blockIdx.x + 1] = b2;
    }
    if (failed && warp == 1) {
        // let every issued MMA finish before the accumulators are released
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 16, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// pass 2
// ---------------------------------------------------------------------------
struct P2Params {
    int D, Dp, npanel, nT, Npad, Kpad, bn, ntiles, units_per_k, ktiles, nunits, nstage;
    int ksteps;           // 16-deep steps of the distance product (D + 3 used columns)
    const float4 *colq;   // Npad
    float *RTpart;        // nunits x 128 x Dp
    int *status;
};

// The CTAs take units v = blockIdx.x, blockIdx.x + gridDim.x, ... in point-
// major order, so at any time all CTAs stream the same few point tiles (which
// stay in L2) against different centre tiles.  Each unit writes the slot
// u = kt * units_per_k + nu (centre-major, the order of the final reduction).
__device__ __forceinline__ void unit_of(const P2Params &p, int v, int &u, int &kt, int &t0, int &t1)
{
    const int nu = v / p.ktiles;
    kt = v % p.ktiles;
    u = kt * p.units_per_k + nu;
    const int per_unit = P2_UNIT_POINTS / p.bn;
    t0 = nu * per_unit;
    t1 = min(p.ntiles, t0 + per_unit);
}

__global__ void __launch_bounds__(P2_THREADS, 1)
    tc_pass2_kernel(const __grid_constant__ CUtensorMap tmT, const __grid_constant__ CUtensorMap tmY,
                    const P2Params p)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int bn = p.bn;                                   // points per tile: 64 or 128
    const int ng = bn / 64;                                // active responsibility groups
    const int ypanel_bytes = P2_BK * 128;                  // 16 KB
    const int tpanel_bytes = bn * 128;
    const int tstage_bytes = p.nT * p.npanel * tpanel_bytes;
    unsigned char *Ys = base;                               // 2 x npanel panels
    unsigned char *Tst = base + 2 * p.npanel * ypanel_bytes;
    float4 *cq = (float4 *) (Tst + p.nstage * tstage_bytes); // nstage x bn
    uint64_t *bars = (uint64_t *) (cq + p.nstage * bn);
    uint64_t *t_full = bars;
    uint64_t *t_empty = bars + p.nstage;
    uint64_t *y_full = bars + 2 * p.nstage;
    uint64_t *y_empty = y_full + 1;
    uint64_t *s_full = y_empty + 1;   // 2
    uint64_t *p_full = s_full + 2;    // 2
    uint64_t *rt_full = p_full + 2;
    uint64_t *rt_empty = rt_full + 1;
    uint64_t *drain = rt_empty + 1;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < p.nstage; s++) {
            mbar_init(&t_full[s], 1);
            mbar_init(&t_empty[s], 1);
        }
        mbar_init(y_full, 1);
        mbar_init(y_empty, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&s_full[b], 1);
            mbar_init(&p_full[b], 128 * ng);
        }
        mbar_init(rt_full, 1);
        mbar_init(rt_empty, 128 * ng);
        mbar_init(drain, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(tmem_sh, 512);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_sh;
    const uint32_t rt_tmem = tmem + 256;

    if (warp == 0 && lane == 0) {
        // ---------------- producer ----------------
        prefetch_tmap(&tmT);
        prefetch_tmap(&tmY);
        int jt = 0, cur_kt = -1, yuse = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            int u, kt, t0, t1;
            unit_of(p, v, u, kt, t0, t1);
            if (kt != cur_kt) {
                if (yuse > 0 && !mbar_wait(y_empty, (yuse - 1) & 1, p.status, 21)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(y_full, (uint32_t) (2 * p.npanel * ypanel_bytes));
                for (int piece = 0; piece < 2; piece++)
                    for (int pn = 0; pn < p.npanel; pn++)
                        tma_load_2d(Ys + (piece * p.npanel + pn) * ypanel_bytes, &tmY, y_full,
                                    PANEL_ELEMS * pn, piece * p.Kpad + kt * P2_BK);
                yuse++;
                cur_kt = kt;
            }
            for (int t = t0; t < t1; t++, jt++) {
                const int s = jt % p.nstage, use = jt / p.nstage;
                if (use > 0 && !mbar_wait(&t_empty[s], (use - 1) & 1, p.status, 22)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(&t_full[s], (uint32_t) (tstage_bytes + bn * 16));
                for (int tp = 0; tp < p.nT; tp++)
                    for (int pn = 0; pn < p.npanel; pn++)
                        tma_load_2d(Tst + s * tstage_bytes + (tp * p.npanel + pn) * tpanel_bytes,
                                    &tmT, &t_full[s], PANEL_ELEMS * pn, tp * p.Npad + t * bn);
                bulk_load(cq + s * bn, p.colq + (size_t) t * bn, (uint32_t) (bn * 16), &t_full[s]);
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        const uint32_t id1 = idesc_bf16(P2_BK, bn, 0, 0);
        const uint32_t id2 = idesc_bf16(P2_BK, p.Dp, 0, 1);
        int jt = 0, cur_kt = -1, yuse = 0, nunit = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            int u, kt, t0, t1;
            unit_of(p, v, u, kt, t0, t1);
            if (kt != cur_kt) {
                if (yuse > 0)
                    mma_commit_w(y_empty);
                if (!mbar_wait_w(y_full, yuse & 1, p.status, 23)) {
                    ok = false;
                    break;
                }
                yuse++;
                cur_kt = kt;
            }
            uint32_t rt_acc = 0;
            const int first_j = jt;
            for (int t = t0; t <= t1 && ok; t++) {
                if (t < t1) {
                    // distances of tile jt: M = 128 centres, N = bn points
                    const int s = jt % p.nstage, b = jt & 1;
                    if (!mbar_wait_w(&t_full[s], (jt / p.nstage) & 1, p.status, 24)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t) (b * bn);
                    const uint32_t tst = smem_u32(Tst + s * tstage_bytes);
                    uint32_t acc = 0;
                    for (int piece = 0; piece < 2; piece++) {
                        const int ntp = (piece == 0) ? p.nT : 1;
                        for (int pn = 0; pn < p.npanel; pn++) {
                            const uint64_t ad0 = sdesc_sw128(
                                smem_u32(Ys + (piece * p.npanel + pn) * ypanel_bytes), 16, 1024);
                            const int kmax = min(4, p.ksteps - 4 * pn);  // skip all-zero steps
                            for (int tp = 0; tp < ntp; tp++) {
                                const uint64_t bd0 = sdesc_sw128(
                                    tst + (tp * p.npanel + pn) * tpanel_bytes, 16, 1024);
#pragma unroll
                                for (int kk = 0; kk < 4; kk++) {
                                    if (kk < kmax) {
                                        mma_ss_w(d, ad0 + 2 * kk, bd0 + 2 * kk, id1, acc);
                                        acc = 1;
                                    }
                                }
                            }
                        }
                    }
                    mma_commit_w(&s_full[b]);
                }
                if (t > t0) {
                    // R T of the previous tile: A = R (TMEM), B = the same T tile, MN-major
                    const int j = jt - 1;
                    const int s = j % p.nstage, b = j & 1;
                    if (j == first_j && nunit > 0 &&
                        !mbar_wait_w(rt_empty, (nunit - 1) & 1, p.status, 25)) {
                        ok = false;
                        break;
                    }
                    if (!mbar_wait_w(&p_full[b], (j >> 1) & 1, p.status, 26)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t tst = smem_u32(Tst + s * tstage_bytes);
                    for (int rp = 0; rp < 2; rp++) {
                        const int ntp = (rp == 0) ? p.nT : 1;
                        for (int tp = 0; tp < ntp; tp++) {
                            const uint64_t bd0 =
                                sdesc_sw128(tst + tp * p.npanel * tpanel_bytes, tpanel_bytes, 1024);
                            for (int kk = 0; kk < bn / 16; kk++) {
                                const uint32_t a = tmem + (uint32_t) (b * bn + (kk >> 2) * 64 +
                                                                      rp * 32 + (kk & 3) * 8);
                                mma_ts_w(rt_tmem, a, bd0 + (uint64_t) (kk * (2048 >> 4)), id2, rt_acc);
                                rt_acc = 1;
                            }
                        }
                    }
                    mma_commit_w(&t_empty[s]);
                }
                if (t < t1)
                    jt++;
            }
            if (!ok)
                break;
            mma_commit_w(rt_full);
            nunit++;
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- responsibilities and the R T drain ----------------
        // group g (warps 2-5 / 6-9) handles points 64 g .. 64 g + 63 of each tile
        const int q = warp & 3;
        const int g = (warp - 2) >> 2;
        const int row = q * 32 + lane;  // centre within the tile
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        if (g < ng) {
            int jt = 0, nunit = 0;
            bool ok = true;
            for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
                int u, kt, t0, t1;
                unit_of(p, v, u, kt, t0, t1);
                for (int t = t0; t < t1; t++, jt++) {
                    const int s = jt % p.nstage, b = jt & 1;
                    if (!mbar_wait(&t_full[s], (jt / p.nstage) & 1, p.status, 27) ||
                        !mbar_wait(&s_full[b], (jt >> 1) & 1, p.status, 28)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t col0 = (uint32_t) (b * bn + g * 64);
                    uint32_t va[32], vb[32];
                    tmem_ld32(lane_base + col0, va);
                    tmem_ld32(lane_base + col0 + 32, vb);
                    tmem_ld_wait();
                    const float4 *cqs = cq + s * bn + g * 64;
                    uint32_t hi[32], lo[32];
#pragma unroll
                    for (int j = 0; j < 16; j++) {
                        float r[4];
#pragma unroll
                        for (int e = 0; e < 4; e++) {
                            const int n = 4 * j + e;  // point within the sub-block
                            const float a = (n < 32) ? __uint_as_float(va[n]) : __uint_as_float(vb[n - 32]);
                            const float4 c = cqs[n];
                            r[e] = ex2(fmaf(a - c.x, c.y, -c.z));
                        }
#pragma unroll
                        for (int e = 0; e < 4; e += 2) {
                            const uint32_t h = pack_bf16(r[e], r[e + 1]);
                            const float rl0 = r[e] - bf16lo_to_f32(h);
                            const float rl1 = r[e + 1] - bf16hi_to_f32(h);
                            hi[2 * j + e / 2] = h;
                            lo[2 * j + e / 2] = pack_bf16(rl0, rl1);
                        }
                    }
                    // R_hi over the first half of the sub-block, R_lo over the second
                    uint32_t h16[16], l16[16];
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        h16[i] = hi[i];
                        l16[i] = lo[i];
                    }
                    tmem_st16(lane_base + col0, h16);
                    tmem_st16(lane_base + col0 + 32, l16);
#pragma unroll
                    for (int i = 0; i < 16; i++) {
                        h16[i] = hi[16 + i];
                        l16[i] = lo[16 + i];
                    }
                    tmem_st16(lane_base + col0 + 16, h16);
                    tmem_st16(lane_base + col0 + 48, l16);
                    tmem_st_wait();
                    tc_fence_before();
                    mbar_arrive(&p_full[b]);
                }
                if (!ok)
                    break;
                // drain this unit's R T (FP32) to its slot; the groups split the columns
                if (!mbar_wait(rt_full, nunit & 1, p.status, 29)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                float *dst = p.RTpart + ((size_t) u * P2_BK + row) * p.Dp;
                const int cw = p.Dp / ng;
                for (int c0 = g * cw; c0 < (g + 1) * cw; c0 += 32) {
                    uint32_t vv[32];
                    tmem_ld32(lane_base + 256 + (uint32_t) c0, vv);
                    tmem_ld_wait();
#pragma unroll
                    for (int j = 0; j < 32; j += 4)
                        *(float4 *) (dst + c0 + j) =
                            make_float4(__uint_as_float(vv[j]), __uint_as_float(vv[j + 1]),
                                        __uint_as_float(vv[j + 2]), __uint_as_float(vv[j + 3]));
                }
                tc_fence_before();
                mbar_arrive(rt_empty);
                nunit++;
            }
            if (!ok)
                failed = 1;
        }
    }
    __syncthreads();
    if (failed && warp == 1) {
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 30, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// operand preparation and the slot reduction
// ---------------------------------------------------------------------------
__global__ void t_exact_kernel(const double *__restrict__ T64, size_t n, int *inexact)
{
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x) {
        const double t = T64[i];
        const double h = (double) __bfloat162float(__float2bfloat16_rn((float) t));
        if (h != t)
            atomicExch(inexact, 1);
    }
}

// T pieces (nT x Npad x Dp): value pieces, three columns of ones, zero padding.
__global__ void t_split_kernel(const double *__restrict__ T64, int N, int D, int Dp, int Npad,
                               int nT, __nv_bfloat16 *__restrict__ Tb)
{
    const size_t total = (size_t) Npad * Dp;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int n = (int) (i / Dp), d = (int) (i % Dp);
        float hi = 0.f, lo = 0.f;
        if (n < N) {
            if (d < D) {
                const double t = T64[(size_t) n * D + d];
                const __nv_bfloat16 h = __float2bfloat16_rn((float) t);
                hi = __bfloat162float(h);
                lo = (float) (t - (double) hi);
            } else if (d < D + 3) {
                hi = 1.f;
            }
        }
        Tb[i] = __float2bfloat16_rn(hi);
        if (nT == 2)
            Tb[total + i] = __float2bfloat16_rn(lo);
    }
}

// Y pieces (2 x Kpad x Dp) with the folded -|y_hat|^2/2 column, and Y in FP32.
// One warp per centre row.
__global__ void y_split_kernel(const double *__restrict__ Y64, int K, int D, int Dp, int Kpad,
                               __nv_bfloat16 *__restrict__ Yb, float *__restrict__ Y32)
{
    const int lane = threadIdx.x & 31;
    const int wpb = blockDim.x >> 5;
    const size_t plane = (size_t) Kpad * Dp;
    for (int k = blockIdx.x * wpb + (threadIdx.x >> 5); k < Kpad; k += gridDim.x * wpb) {
        __nv_bfloat16 *hi = Yb + (size_t) k * Dp;
        __nv_bfloat16 *lo = hi + plane;
        if (k >= K) {
            for (int d = lane; d < Dp; d += 32) {
                hi[d] = __float2bfloat16_rn(d == D ? -1.0e30f : 0.f);
                lo[d] = __float2bfloat16_rn(0.f);
            }
            continue;
        }
        double q = 0.0;
        for (int d = lane; d < D; d += 32) {
            const double y = Y64[(size_t) k * D + d];
            const __nv_bfloat16 h = __float2bfloat16_rn((float) y);
            const double hd = (double) __bfloat162float(h);
            const __nv_bfloat16 l = __float2bfloat16_rn((float) (y - hd));
            const double yh = hd + (double) __bfloat162float(l);
            hi[d] = h;
            lo[d] = l;
            Y32[(size_t) k * D + d] = (float) y;
            q += yh * yh;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            q += __shfl_xor_sync(0xffffffffu, q, o);
        // -q/2 in three BF16 pieces (24+ significant bits)
        const double v = -0.5 * q;
        const __nv_bfloat16 p1 = __float2bfloat16_rn((float) v);
        const double r1 = v - (double) __bfloat162float(p1);
        const __nv_bfloat16 p2 = __float2bfloat16_rn((float) r1);
        const double r2 = r1 - (double) __bfloat162float(p2);
        const __nv_bfloat16 p3 = __float2bfloat16_rn((float) r2);
        for (int d = D + lane; d < Dp; d += 32) {
            const int a = d - D;
            hi[d] = (a == 0) ? p1 : (a == 1) ? p2 : (a == 2) ? p3 : __float2bfloat16_rn(0.f);
            lo[d] = __float2bfloat16_rn(0.f);
        }
    }
}

// RT[k][d] = sum_u RTpart[kt][u][k % 128][d]; G[k] from the column of ones.
__global__ void slot_reduce_kernel(const float *__restrict__ RTpart, int K, int D, int Dp, int U,
                                   double *__restrict__ G, double *__restrict__ RT)
{
    const size_t total = (size_t) K * (D + 1);
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int k = (int) (i / (D + 1)), d = (int) (i % (D + 1));
        const int kt = k / P2_BK, kl = k % P2_BK;
        const float *src = RTpart + ((size_t) kt * U * P2_BK + kl) * Dp + d;
        double s = 0.0;
        for (int u = 0; u < U; u++)
            s += (double) src[(size_t) u * P2_BK * Dp];
        if (d < D)
            RT[(size_t) k * D + d] = s;
        else
            G[k] = s;
    }
}

using P1Kernel = void (*)(const CUtensorMap, const P1Params);

// the pass-1 instantiation for a shape (NP panels, KL steps in the last, NT pieces)
P1Kernel pass1_for(int np, int kl, int nt)
{
#define DGTM_P1(NP_, KL_, NT_) \
    if (np == NP_ && kl == KL_ && nt == NT_) return tc_pass1_kernel<NP_, KL_, NT_>;
#define DGTM_P1_KL(NP_, NT_) DGTM_P1(NP_, 1, NT_) DGTM_P1(NP_, 2, NT_) DGTM_P1(NP_, 3, NT_) DGTM_P1(NP_, 4, NT_)
    DGTM_P1_KL(1, 1) DGTM_P1_KL(1, 2) DGTM_P1_KL(2, 1) DGTM_P1_KL(2, 2)
    DGTM_P1_KL(3, 1) DGTM_P1_KL(3, 2) DGTM_P1_KL(4, 1) DGTM_P1_KL(4, 2)
#undef DGTM_P1_KL
#undef DGTM_P1
    return nullptr;
}

}  // namespace

struct TcState {
    int N, D, K, sms;
    int Dp, npanel, Npad, Kpad, nT, ksteps;
    int nchunk, nstage1, nstage2, ntile1, bn2;
    int ntiles2, units_per_k, nunits, grid2;
    size_t smem1, smem2;
    P1Kernel pass1;
    __nv_bfloat16 *Tb, *Yb;
    float *Y32;
    float4 *colq;
    float *RTpart;
    int *status, *hstatus;
    const double *tt, *T64;
    CUtensorMap tmT1, tmT2, tmY1, tmY2;
};

static int grid_for(size_t n, int per = 256, int cap = 8192)
{
    size_t b = (n + per - 1) / per;
    if (b > (size_t) cap)
        b = cap;
    return b == 0 ? 1 : (int) b;
}

int tc_create(TcState **out, int N, int D, int K, int sms, const double *T64, const double *tt,
              cudaStream_t s)
{
    *out = nullptr;
    int dev = 0, major = 0, minor = 0;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form needs a Blackwell (sm_10x) GPU, found sm_%d%d",
                  major, minor);
        return DGTM_ENOTSUP;
    }
    if (D + 3 > 256) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form supports D <= 253 (D = %d)", D);
        return DGTM_ENOTSUP;
    }
    TcState *st = new TcState();
    st->N = N;
    st->D = D;
    st->K = K;
    st->sms = sms;
    st->tt = tt;
    st->T64 = T64;
    st->Dp = round_up(D + 3, PANEL_ELEMS);
    st->npanel = st->Dp / PANEL_ELEMS;
    st->ksteps = (D + 3 + 15) / 16;  // columns D + 3 .. Dp - 1 are zero in both operands
    st->Npad = round_up(N, NPAD_ALIGN);
    st->Kpad = round_up(K, P1_BK);
    st->nchunk = st->Kpad / P1_BK;
    int rc = DGTM_OK;
    auto fail = [&](int code) {
        tc_destroy(st);
        return code;
    };
    cudaError_t e = cudaMalloc((void **) &st->status, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &st->hstatus, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(st->status, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        t_exact_kernel<<<grid_for((size_t) N * D), 256, 0, s>>>(T64, (size_t) N * D, st->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st->hstatus, st->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "tc_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    st->nT = (*st->hstatus) ? 2 : 1;
    // exact 0/1 data: two 128-point tiles per pass-1 CTA and 128-point pass-2
    // tiles; split data (two T pieces) halve both to fit shared memory
    st->ntile1 = (st->nT == 1) ? 2 : 1;
    st->bn2 = (st->nT == 1) ? 128 : 64;

    const size_t tpl = (size_t) st->Npad * st->Dp, ypl = (size_t) st->Kpad * st->Dp;
    // pass 2 work units
    st->ntiles2 = st->Npad / st->bn2;
    st->units_per_k = (st->Npad + P2_UNIT_POINTS - 1) / P2_UNIT_POINTS;
    const int ktiles2 = (K + P2_BK - 1) / P2_BK;
    st->nunits = ktiles2 * st->units_per_k;
    st->grid2 = st->nunits < sms ? st->nunits : sms;

    e = cudaMalloc((void **) &st->Tb, sizeof(__nv_bfloat16) * tpl * st->nT);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->Yb, sizeof(__nv_bfloat16) * ypl * 2);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->Y32, sizeof(float) * (size_t) K * D);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->colq, sizeof(float4) * st->Npad);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->RTpart, sizeof(float) * (size_t) st->nunits * P2_BK * st->Dp);
    if (e != cudaSuccess) {
        set_error(DGTM_ENOMEM, "tc_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ENOMEM);
    }
    t_split_kernel<<<grid_for(tpl), 256, 0, s>>>(T64, N, D, st->Dp, st->Npad, st->nT, st->Tb);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "t_split: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    // tensor maps: T pieces stacked by rows, Y pieces stacked by rows
    if ((rc = make_tmap_bf16(&st->tmT1, st->Tb, (uint64_t) st->nT * st->Npad, st->Dp, st->Dp,
                             P1_TILE, PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmT2, st->Tb, (uint64_t) st->nT * st->Npad, st->Dp, st->Dp,
                             st->bn2, PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmY1, st->Yb, 2 * (uint64_t) st->Kpad, st->Dp, st->Dp, P1_BK,
                             PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmY2, st->Yb, 2 * (uint64_t) st->Kpad, st->Dp, st->Dp, P2_BK,
                             PANEL_ELEMS)) != DGTM_OK)
        return fail(rc);
    // shared memory plans
    const size_t bar_bytes = 64 * 8 + 16 + 2 * 256 * 8;
    // pass 1: Y slots of one chunk piece (npanel panels of 16 KB); the data
    // tiles live in tensor memory
    const size_t slot1 = (size_t) st->npanel * P1_BK * 128;
    int ns1 = (int) ((SMEM_LIMIT - 1024 - bar_bytes) / slot1);
    if (ns1 > 12)
        ns1 = 12;
    st->pass1 = pass1_for(st->npanel, st->ksteps - 4 * (st->npanel - 1), st->nT);
    const size_t y2 = (size_t) 2 * st->npanel * P2_BK * 128;
    const size_t ts2 = (size_t) st->nT * st->npanel * st->bn2 * 128 + st->bn2 * 16;
    int ns2 = (int) ((SMEM_LIMIT - 1024 - bar_bytes - y2) / ts2);
    if (ns2 > 4)
        ns2 = 4;
    if (ns1 < 2 || ns2 < 2 || !st->pass1) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form does not fit shared memory (D = %d)", D);
        return fail(DGTM_ENOTSUP);
    }
    st->nstage1 = ns1;
    st->nstage2 = ns2;
    st->smem1 = 1024 + (size_t) ns1 * slot1 + bar_bytes;
    st->smem2 = 1024 + y2 + (size_t) ns2 * ts2 + bar_bytes;
    e = cudaFuncSetAttribute(st->pass1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int) st->smem1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(tc_pass2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) st->smem2);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "tc_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    *out = st;
    return DGTM_OK;
}

void tc_destroy(TcState *st)
{
    if (!st)
        return;
    cudaFree(st->Tb);
    cudaFree(st->Yb);
    cudaFree(st->Y32);
    cudaFree(st->colq);
    cudaFree(st->RTpart);
    cudaFree(st->status);
    if (st->hstatus)
        cudaFreeHost(st->hstatus);
    delete st;
}

int tc_prepare_y(TcState *st, const double *Y64, cudaStream_t s)
{
    y_split_kernel<<<grid_for((size_t) st->Kpad * 32, 256, 4096), 256, 0, s>>>(
        Y64, st->K, st->D, st->Dp, st->Kpad, st->Yb, st->Y32);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int tc_pass1_blocks(const TcState *st) { return st->Npad / (st->ntile1 * P1_TILE); }

int tc_estep(TcState *st, const double *, double c1, double c2, int isDA, double2 *colstat,
             double *part, cudaStream_t s, int *nlaunch)
{
    P1Params p;
    p.N = st->N;
    p.D = st->D;
    p.Dp = st->Dp;
    p.npanel = st->npanel;
    p.nT = st->nT;
    p.Npad = st->Npad;
    p.Kpad = st->Kpad;
    p.K = st->K;
    p.nchunk = st->nchunk;
    p.nstage = st->nstage1;
    p.ntile = st->ntile1;
    p.ksteps = st->ksteps;
    p.c1 = c1;
    p.c2 = c2;
    p.c1l = (float) (2.0 * c1 * 1.4426950408889634);
    p.c2l = (float) (2.0 * c2 * 1.4426950408889634);
    p.isDA = isDA;
    p.two_temps = isDA && (c1 != c2);
    p.Y32 = st->Y32;
    p.T64 = st->T64;
    p.Tb = (const uint32_t *) st->Tb;
    p.colstat = colstat;
    p.colq = st->colq;
    p.part = part;
    p.status = st->status;
    DGTM_CUDA_TRY(cudaMemsetAsync(st->status, 0, sizeof(int), s));
    st->pass1<<<tc_pass1_blocks(st), P1_THREADS, st->smem1, s>>>(st->tmY1, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 1;
    return DGTM_OK;
}

int tc_mstep_pass(TcState *st, const double2 *, double, cudaStream_t s, int *nlaunch)
{
    P2Params p;
    p.D = st->D;
    p.Dp = st->Dp;
    p.npanel = st->npanel;
    p.nT = st->nT;
    p.Npad = st->Npad;
    p.Kpad = st->Kpad;
    p.bn = st->bn2;
    p.ntiles = st->ntiles2;
    p.units_per_k = st->units_per_k;
    p.ktiles = (st->K + P2_BK - 1) / P2_BK;
    p.nunits = st->nunits;
    p.nstage = st->nstage2;
    p.ksteps = st->ksteps;
    p.colq = st->colq;
    p.RTpart = st->RTpart;
    p.status = st->status;
    tc_pass2_kernel<<<st->grid2, P2_THREADS, st->smem2, s>>>(st->tmT2, st->tmY2, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 1;
    return DGTM_OK;
}

int tc_mstep_reduce(TcState *st, double *G, double *RT, cudaStream_t s, int *nlaunch)
{
    slot_reduce_kernel<<<grid_for((size_t) st->K * (st->D + 1)), 256, 0, s>>>(
        st->RTpart, st->K, st->D, st->Dp, st->units_per_k, G, RT);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 1;
    return DGTM_OK;
}

int tc_fetch_status(TcState *st, cudaStream_t s)
{
    DGTM_CUDA_TRY(cudaMemcpyAsync(st->hstatus, st->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    return DGTM_OK;
}

int tc_check_status(TcState *st)
{
    if (*st->hstatus != 0) {
        set_error(DGTM_ETIMEOUT, "a tensor-core kernel gave up waiting (site %d)", *st->hstatus);
        return DGTM_ETIMEOUT;
    }
    return DGTM_OK;
}

}  // namespace dgtm
