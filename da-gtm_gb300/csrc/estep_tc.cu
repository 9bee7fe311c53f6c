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
// Pass 2 (persistent, units of (128 centres) x 16K-40K points): the CTA
// keeps its 128 centres resident, streams 64-point T tiles, recomputes
// acc (M = 128 centres, N = 64 points), turns it into R_kn with the pass-1
// statistics, writes R as BF16 hi/lo back into tensor memory and multiplies
// R by the same T tile read MN-major (M = 128, N = D padded, K = 16 points),
// accumulating R T (and, through the column of ones, G = rowsum R) in TMEM
// over 4096-point segments, which are summed in shared memory.  Every unit's
// FP32 R T is written to its own slot; a fixed-order sum over the slots
// (TwoSum, exact to FP64) gives RT and G.
#include "common.cuh"
#include "kernels.cuh"
#include "sm100.cuh"
#include "tc.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <vector>

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
    const double *T64;    // N x D (exact data, read when T is split in two pieces) ...
    const float *T32;     // ... or, when not null, the data as given in FP32
    const uint32_t *Tb;   // nT x Npad x Dp BF16 (as BF16 pairs)
    double2 *colstat;     // N
    float4 *colq;         // Npad
    double *part;         // 2 per CTA
    int *status;
};

// lowest j in block B (columns 32 B .. 32 B + 31) with v[j] == mx; the block
// is known to hold mx.  Constant indices keep v in registers.
template <int B, int NV>
__device__ __forceinline__ int first_equal(const uint32_t (&v)[NV], float mx)
{
    int j0 = 32 * B + 31;
#pragma unroll
    for (int j = 31; j >= 0; j--)
        if (__uint_as_float(v[32 * B + j]) == mx)
            j0 = 32 * B + j;
    return j0;
}

// TMEM map of pass 1: the point tiles (MMA operand A, BF16 pairs) from column
// 0, the two 128-column accumulators at columns 256 and 384.
constexpr int P1_ACC_COL = 256;

// ---------------------------------------------------------------------------
// pass 1: one CTA per NTILE x 128 points.  The data tiles live in tensor
// memory as the A operand; shared memory holds only the Y ring.  NTILE = 2
// (data exact in BF16): each tile owns one accumulator and the two tiles
// ping-pong, so the tensor pipe works on one tile while the statistics warps
// read the other.  NTILE = 1 (data split in two BF16 pieces): one tile
// double-buffers the two accumulators, and both statistics warp groups read
// each chunk, half the centres apiece, merging a point's two partial maxima
// and sums at the end.
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
    tc_pass1_kernel(const __grid_constant__ CUtensorMap tmY, const __grid_constant__ CUtensorMap tmT,
                    const P1Params p)
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
    uint64_t *t_full = bars + 2 * nslot;  // the data tiles are in shared memory
    uint64_t *t_done = t_full + 1;        // ... and copied into tensor memory
    uint64_t *acc_full = t_done + 1;      // [region]
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
        mbar_init(t_full, 1);
        mbar_init(t_done, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&acc_full[b], 1);
            // the statistics threads of the accumulator's tile: one group of
            // 128, or both groups when a CTA holds a single tile
            mbar_init(&acc_empty[b], NTILE == 2 ? 128 : 256);
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
        // ---------------- producer ----------------
        prefetch_tmap(&tmY);
        prefetch_tmap(&tmT);
        // the CTA's two data pieces (tiles g = 0, 1, or pieces hi, lo of one
        // tile) into the last two slots, for the copy into tensor memory
        mbar_expect_tx(t_full, (uint32_t) (2 * SLOT_BYTES));
#pragma unroll
        for (int s2 = 0; s2 < 2; s2++) {
            const int g = (NTILE == 2) ? s2 : 0, tp = (NT == 2) ? s2 : 0;
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(Yslot + (nslot - 2 + s2) * SLOT_BYTES + pn * PANEL_BYTES, &tmT, t_full,
                            PANEL_ELEMS * pn, tp * p.Npad + n0 + g * P1_TILE);
        }
        // the Y ring, one piece of a chunk per slot
        int q = 0;
        uint32_t ph = 0;
        for (int it = 0; it < 2 * p.nchunk; it++) {
            if (it >= nslot && !mbar_wait(&y_empty[q], ph ^ 1u, p.status, 11)) {
                failed = 1;
                break;
            }
            if (it < nslot && q >= nslot - 2 && !mbar_wait(t_done, 0, p.status, 17)) {
                failed = 1;  // the slot still held a data piece
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
        // data pieces: shared memory -> tensor memory (the MMA A operand; piece
        // s2 goes to columns s2 * ACOL, column j holding depths 2 j and 2 j + 1)
        bool ok = mbar_wait_w(t_full, 0, p.status, 12);
        if (ok) {
            tc_fence_after();
            const uint64_t tdesc = ydesc0 + (uint64_t) ((nslot - 2) * (SLOT_BYTES >> 4));
#pragma unroll
            for (int s2 = 0; s2 < 2; s2++)
#pragma unroll
                for (int pn = 0; pn < NP; pn++)
#pragma unroll
                    for (int kk = 0; kk < (pn == NP - 1 ? KL : 4); kk++)
                        tmem_cp_w(tmem + (uint32_t) (s2 * ACOL + pn * 32 + kk * 8),
                                  tdesc + (uint64_t) (s2 * (SLOT_BYTES >> 4) + pn * (PANEL_BYTES >> 4) + 2 * kk));
            mma_commit_w(t_done);
            ok = mbar_wait_w(t_done, 0, p.status, 12);
            tc_fence_after();
        }
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
        // With a single tile per CTA (data in two pieces) both groups serve
        // it: group g takes columns 64 g .. 64 g + 63 of each chunk, and the
        // two partial maxima and sums of a point are merged at the end.
        constexpr int W = (NTILE == 2) ? P1_BK : P1_BK / 2;  // columns per thread and chunk
        const int q = warp & 3;
        const int g = (warp - 2) >> 2;
        const int tile = (NTILE == 2) ? g : 0;
        const int cofs = (NTILE == 2) ? 0 : W * g;
        const bool owner = (NTILE == 2) || g == 0;  // writes the point's results
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        const int prow = tile * P1_TILE + row;
        const int n = n0 + prow;
        double t1 = 0.0, t2 = 0.0;
        bool ok = true;
        {
            float m = -INFINITY;
            int kstar = 0;
            // shifted sums at temperature 1 and at `temp`, FP32 with Kahan
            // compensation (the FP64 pipe of this part is too narrow for the
            // per-chunk update); the result carries ~2 ulp of FP32
            float s1 = 0.f, s2 = 0.f, k1 = 0.f, k2 = 0.f;
            for (int c = 0; c < p.nchunk; c++) {
                const int rg = region(tile, c);
                if (!mbar_wait(&acc_full[rg], ruse(c) & 1, p.status, 15)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // copy this thread's columns out and hand the accumulator back
                // at once, so the next chunk's MMAs overlap this arithmetic
                uint32_t v[W];
                {
                    const uint32_t col = lane_base + (uint32_t) (P1_ACC_COL + rg * P1_BK + cofs);
#pragma unroll
                    for (int u = 0; u < W / 32; u++)
                        tmem_ld32p(col + 32 * u, v + 32 * u);
                    tmem_ld_wait();
                }
                tc_fence_before();
                mbar_arrive(&acc_empty[rg]);
                // maxima of the 32-column blocks (independent chains)
                float mxq[W / 32];
#pragma unroll
                for (int u = 0; u < W / 32; u++)
                    mxq[u] = -INFINITY;
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
#pragma unroll
                    for (int u = 0; u < W / 32; u++)
                        mxq[u] = fmax3(mxq[u], __uint_as_float(v[32 * u + j]), __uint_as_float(v[32 * u + j + 1]));
                }
                float mx = mxq[0];
#pragma unroll
                for (int u = 1; u < W / 32; u++)
                    mx = fmaxf(mx, mxq[u]);
                if (mx > m) {
                    if (m > -INFINITY) {
                        const float f1 = ex2((m - mx) * p.c1l), f2 = ex2((m - mx) * p.c2l);
                        s1 *= f1;
                        k1 *= f1;
                        s2 *= f2;
                        k2 *= f2;
                    }
                    // lowest index attaining the maximum: first block holding it,
                    // then a scan of that block only
                    int j0;
                    if (mxq[0] == mx)
                        j0 = first_equal<0>(v, mx);
                    else if (W == 64 || mxq[1] == mx)
                        j0 = first_equal<1>(v, mx);
                    else if (mxq[2 % (W / 32)] == mx)
                        j0 = first_equal<2 % (W / 32)>(v, mx);
                    else
                        j0 = first_equal<3 % (W / 32)>(v, mx);
                    m = mx;
                    kstar = c * P1_BK + cofs + j0;
                }
                // four independent accumulation chains per sum (element j goes
                // to chain j % 4), as two packed pairs: (0, 1) and (2, 3)
                float e1[4], e2[4];
                {
                    const f2 mm = f2_pack(m, m), k1 = f2_pack(p.c1l, p.c1l);
                    f2 a1 = f2_pack(0.f, 0.f), b1 = a1, a2 = a1, b2 = a1;
                    if (p.two_temps) {
                        const f2 k2 = f2_pack(p.c2l, p.c2l);
#pragma unroll
                        for (int j = 0; j < W; j += 4) {
                            const f2 xa = f2_sub(f2_pack(__uint_as_float(v[j]), __uint_as_float(v[j + 1])), mm);
                            const f2 xb = f2_sub(f2_pack(__uint_as_float(v[j + 2]), __uint_as_float(v[j + 3])), mm);
                            a1 = f2_add(a1, f2_ex2(f2_mul(xa, k1)));
                            b1 = f2_add(b1, f2_ex2(f2_mul(xb, k1)));
                            a2 = f2_add(a2, f2_ex2(f2_mul(xa, k2)));
                            b2 = f2_add(b2, f2_ex2(f2_mul(xb, k2)));
                        }
                    } else {
#pragma unroll
                        for (int j = 0; j < W; j += 4) {
                            const f2 xa = f2_sub(f2_pack(__uint_as_float(v[j]), __uint_as_float(v[j + 1])), mm);
                            const f2 xb = f2_sub(f2_pack(__uint_as_float(v[j + 2]), __uint_as_float(v[j + 3])), mm);
                            a1 = f2_add(a1, f2_ex2(f2_mul(xa, k1)));
                            b1 = f2_add(b1, f2_ex2(f2_mul(xb, k1)));
                        }
                    }
                    e1[0] = f2_lo(a1);
                    e1[1] = f2_hi(a1);
                    e1[2] = f2_lo(b1);
                    e1[3] = f2_hi(b1);
                    e2[0] = f2_lo(a2);
                    e2[1] = f2_hi(a2);
                    e2[2] = f2_lo(b2);
                    e2[3] = f2_hi(b2);
                }
                {
                    const float y1 = ((e1[0] + e1[1]) + (e1[2] + e1[3])) - k1;
                    const float u1 = s1 + y1;
                    k1 = (u1 - s1) - y1;
                    s1 = u1;
                    const float y2 = ((e2[0] + e2[1]) + (e2[2] + e2[3])) - k2;
                    const float u2 = s2 + y2;
                    k2 = (u2 - s2) - y2;
                    s2 = u2;
                }
            }
            if (NTILE == 1) {
                // group 1 hands its partial maximum, index and compensated sums
                // to group 0 through shared memory (the red array, written with
                // the per-point terms only after the second barrier)
                float *xm = (float *) red;  // [4][128]: m, s1 - k1, s2 - k2, kstar
                if (g == 1) {
                    xm[row] = m;
                    xm[128 + row] = s1 - k1;
                    xm[256 + row] = s2 - k2;
                    xm[384 + row] = __int_as_float(kstar);
                }
                asm volatile("bar.sync 1, 256;" ::: "memory");
                if (g == 0) {
                    const float mb = xm[row], sb1 = xm[128 + row], sb2 = xm[256 + row];
                    const int kb = __float_as_int(xm[384 + row]);
                    const float mn = fmaxf(m, mb);
                    if (mn > -INFINITY) {
                        const float fa1 = ex2((m - mn) * p.c1l), fb1 = ex2((mb - mn) * p.c1l);
                        const float fa2 = ex2((m - mn) * p.c2l), fb2 = ex2((mb - mn) * p.c2l);
                        s1 = fmaf(s1 - k1, fa1, sb1 * fb1);
                        s2 = fmaf(s2 - k2, fa2, sb2 * fb2);
                        k1 = 0.f;
                        k2 = 0.f;
                    }
                    // the lowest index among equal maxima
                    if (mb > m || (mb == m && kb < kstar))
                        kstar = kb;
                    m = mn;
                }
                asm volatile("bar.sync 1, 256;" ::: "memory");
            }
            if (!p.two_temps) {
                s2 = s1;
                k2 = k1;
            }
            // exact (FP32) distance to the best centre, from the unsplit centre
            // and the data, then the per-point terms.  With exact (0/1) data the
            // row is read back from tensor memory (the A operand, warp-
            // collective, so outside the per-point branch), 64 dimensions per
            // batch of centre loads.
            // only the owning group writes a point's results (group 1 of a
            // single-tile CTA holds unmerged partials)
            const bool active = owner && ok && n < p.N;
            const int kb = min(kstar, p.K - 1);
            const float *yk = p.Y32 + (size_t) kb * p.D;
            float dsum = 0.f;
            if (NT == 1) {
#pragma unroll 1
                for (int b = 0; b < NP; b++) {
                    uint32_t tw[32];
                    tmem_ld32p(lane_base + (uint32_t) (g * ACOL + 32 * b), tw);
                    float yv[64];
                    const int d0 = 64 * b;
                    if (active) {
                        if ((p.D & 1) == 0) {
                            // even D: every row starts on an 8-byte boundary
#pragma unroll
                            for (int e = 0; e < 32; e++) {
                                const float2 y2 = (d0 + 2 * e < p.D) ? *(const float2 *) (yk + d0 + 2 * e)
                                                                     : make_float2(0.f, 0.f);
                                yv[2 * e] = y2.x;
                                yv[2 * e + 1] = y2.y;
                            }
                        } else {
#pragma unroll
                            for (int e = 0; e < 64; e++)
                                yv[e] = (d0 + e < p.D) ? yk[d0 + e] : 0.f;
                        }
                    }
                    tmem_ld_wait();
                    if (active) {
#pragma unroll
                        for (int e = 0; e < 64; e++) {
                            if (d0 + e < p.D) {
                                const uint32_t w = tw[e >> 1];
                                const float t = __uint_as_float((e & 1) ? (w & 0xFFFF0000u) : (w << 16));
                                const float df = yv[e] - t;
                                dsum = fmaf(df, df, dsum);
                            }
                        }
                    }
                }
            } else if (active && p.T32) {
                const float *tn = p.T32 + (size_t) n * p.D;
#pragma unroll 8
                for (int d = 0; d < p.D; d++) {
                    const float df = yk[d] - tn[d];
                    dsum = fmaf(df, df, dsum);
                }
            } else if (active) {
                const double *tn = p.T64 + (size_t) n * p.D;
#pragma unroll 8
                for (int d = 0; d < p.D; d++) {
                    const float df = yk[d] - (float) tn[d];
                    dsum = fmaf(df, df, dsum);
                }
            }
            if (active) {
                const double dstar = (double) dsum;
                // FP32 logarithms of the FP32 sums (the FP64 pipe is narrow here)
                const double ls1 = (double) logf(s1 - k1), ls2 = (double) logf(s2 - k2);
                const double ls_sel = p.isDA ? ls2 : ls1;
                const double c_sel = p.isDA ? p.c2 : p.c1;
                t1 = -p.c1 * dstar + ls1;
                t2 = p.isDA ? (-p.c2 * dstar + ls2) : 0.0;
                double lsn = ls_sel;
                float4 cq = make_float4(m, (float) (2.0 * c_sel) * LOG2E,
                                        (float) (ls_sel * 1.4426950408889634), 0.f);
                // comm/mpicomm.c:382-389 zero-column fallback (exp(-700) is far
                // from underflow, so the FP64 exp runs only near the limit)
                if (p.c1 * dstar > 700.0 && exp(-p.c1 * dstar) == 0.0) {
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
            } else if (owner && n < p.Npad) {
                p.colq[n] = make_float4(0.f, 0.f, INFINITY, 0.f);  // padding: R = 0
            }
            if (!ok)
                failed = 1;
        }
        red[g * P1_TILE + row] = t1;
        red[256 + g * P1_TILE + row] = t2;
    }
    __syncthreads();
    if (warp < 2) {
        // fixed-order sum of the CTA's per-point terms: warp 0 the temperature-1
        // terms, warp 1 the `temp` terms; each lane a contiguous run, then a
        // butterfly over the lanes
        constexpr int PER = NTILE * P1_TILE / 32;
        const double *src = red + warp * 256 + lane * PER;
        double a = 0.0;
#pragma unroll
        for (int i = 0; i < PER; i++)
            a += src[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0)
            p.part[2 * blockIdx.x + warp] = a;
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
    int D, Dp, Npad, Kpad, ntiles, unit_tiles, units_per_k, ktiles, nunits, nstage;
    const uint32_t *Yb;   // 2 x Kpad x Dp BF16 (as BF16 pairs): the centre pieces
    const float4 *colq;   // Npad
    float *RTpart;        // nunits x 128 x Dp
    int *status;
};

constexpr int P2_TILE = 64;  // points per tile (MMA N of the distance product)
// R T is accumulated in tensor memory over at most this many tiles (4096
// points), a segment.  The tensor pipe's FP32 accumulation rounds each MMA's
// sum down a little, which over a whole 16384-point unit came to ~6e-5 of G
// and R T (4096 points: ~1e-5).  A power of two: the MMA warp finds segment
// starts with a mask.
constexpr int P2_SEG_TILES = 64;
static_assert((P2_SEG_TILES & (P2_SEG_TILES - 1)) == 0, "segment length");

// Where the segments of a unit are summed.  With shared memory to spare
// (128 x (Dp + 4) FP32 beside at least four ring stages) they are summed
// there in FP32 (round-to-nearest) and the unit's total is stored to its
// slot.  Otherwise (two data pieces and three panels: the ring would drop to
// two stages, which measured 1.5x slower) the first segment is stored to
// the slot and the later ones are added at L2 with red.global.add.
__host__ __device__ constexpr bool p2_segbuf(int np, int nt) { return nt * np <= 4; }

// The CTAs take units v = blockIdx.x, blockIdx.x + gridDim.x, ... in point-
// major order, so at any time all CTAs stream the same few point tiles (which
// stay in L2) against different centre tiles.  Each unit writes the slot
// u = kt * units_per_k + nu (centre-major, the order of the final reduction).
__device__ __forceinline__ void unit_of(const P2Params &p, int v, int &u, int &kt, int &t0, int &t1)
{
    const int nu = v / p.ktiles;
    kt = v % p.ktiles;
    u = kt * p.units_per_k + nu;
    t0 = nu * p.unit_tiles;
    t1 = min(p.ntiles, t0 + p.unit_tiles);
}

// Pass 2, a template on the operand shape like pass 1.  Tensor memory holds
// the unit's R T accumulator (columns 0 .. Dp-1), two 64-point buffers in
// which the distance accumulator S is turned into R (BF16 hi/lo), and the
// unit's 128 centres (Y hi, Y lo) as the A operand of the distance product,
// so shared memory is left to a deep ring of point tiles.  Per 64-point tile:
// MMA 1 (A = Y from tensor memory, B = T tile, N = 64) gives S; eight warps
// (two 32-point groups x four lane quarters) form R and write it over S; MMA 2
// (A = R from tensor memory, B = the same T tile read MN-major, N = Dp)
// accumulates R T.  At a unit boundary the same warps drain R T to the
// unit's slot and load the next unit's centres into tensor memory.
template <int NP, int KL, int NT>
__global__ void __launch_bounds__(P2_THREADS, 1)
    tc_pass2_kernel(const __grid_constant__ CUtensorMap tmT, const P2Params p)
{
    constexpr int KS = 4 * (NP - 1) + KL;               // 16-deep steps of the distance product
    constexpr int DP = NP * PANEL_ELEMS;
    constexpr int YCOLS = (KS * 8 + 15) / 16 * 16;      // TMEM columns of one Y piece
    constexpr int SP_COL = DP;                          // S / P buffers: 2 x 64 columns
    constexpr int Y_COL = DP + 2 * P2_TILE;             // Y hi, then Y lo
    static_assert(Y_COL + 2 * YCOLS <= 512, "pass 2 tensor memory plan");
    constexpr int TPANEL_BYTES = P2_TILE * 128;         // 8 KB
    constexpr int TSTAGE_BYTES = NT * NP * TPANEL_BYTES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int nstage = p.nstage;
    unsigned char *Tst = base;
    float4 *cq = (float4 *) (Tst + nstage * TSTAGE_BYTES);  // nstage x 64
    // the unit's segment sums: 128 rows of DP + 4 floats (the pad spreads a
    // quarter-warp's float4 accesses to one row each over all banks)
    constexpr bool SEGBUF = p2_segbuf(NP, NT);
    constexpr int RB = DP + 4;
    float *rtbuf = (float *) (cq + nstage * P2_TILE);
    uint64_t *bars = (uint64_t *) (rtbuf + (SEGBUF ? P2_BK * RB : 0));
    uint64_t *t_full = bars;
    uint64_t *t_empty = bars + nstage;
    uint64_t *s_full = bars + 2 * nstage;  // 2
    uint64_t *p_full = s_full + 2;         // 2
    uint64_t *rt_full = p_full + 2;
    uint64_t *y_ready = rt_full + 1;       // a unit's centres are in tensor memory
    uint64_t *drain = y_ready + 1;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < nstage; s++) {
            mbar_init(&t_full[s], 1);
            mbar_init(&t_empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&s_full[b], 1);
            mbar_init(&p_full[b], 256);
        }
        mbar_init(rt_full, 1);
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
        // ---------------- producer: point tiles and their column statistics ----------------
        prefetch_tmap(&tmT);
        int s = 0;
        uint32_t ph = 0;
        int jt = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            int u, kt, t0, t1;
            unit_of(p, v, u, kt, t0, t1);
            for (int t = t0; t < t1; t++, jt++) {
                if (jt >= nstage && !mbar_wait(&t_empty[s], ph ^ 1u, p.status, 22)) {
                    ok = false;
                    break;
                }
                mbar_expect_tx(&t_full[s], (uint32_t) (TSTAGE_BYTES + P2_TILE * 16));
#pragma unroll
                for (int tp = 0; tp < NT; tp++)
#pragma unroll
                    for (int pn = 0; pn < NP; pn++)
                        tma_load_2d(Tst + s * TSTAGE_BYTES + (tp * NP + pn) * TPANEL_BYTES, &tmT,
                                    &t_full[s], PANEL_ELEMS * pn, tp * p.Npad + t * P2_TILE);
                bulk_load(cq + s * P2_TILE, p.colq + (size_t) t * P2_TILE, (uint32_t) (P2_TILE * 16),
                          &t_full[s]);
                if (++s == nstage) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp == 1) {
        // ---------------- MMA issuer (whole warp; one elected lane issues) ----------------
        const uint32_t id1 = idesc_bf16(P2_BK, P2_TILE, 0, 0);
        const uint32_t id2 = idesc_bf16(P2_BK, DP, 0, 1);
        const uint64_t tdesc_k = sdesc_sw128(smem_u32(Tst), 16, 1024);            // K-major (MMA 1)
        const uint64_t tdesc_mn = sdesc_sw128(smem_u32(Tst), TPANEL_BYTES, 1024); // MN-major (MMA 2)
        const uint32_t rt_tmem = tmem;
        int jt = 0, s = 0, nunit = 0;
        uint32_t ph = 0;
        int sp = 0;  // stage of the tile awaiting MMA 2
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            int u, kt, t0, t1;
            unit_of(p, v, u, kt, t0, t1);
            // the unit's centres are in tensor memory; its first MMA 2 waits on
            // a p_full given after the previous unit's R T has left
            if (!mbar_wait_w(y_ready, nunit & 1, p.status, 23)) {
                ok = false;
                break;
            }
            tc_fence_after();
            for (int t = t0; t <= t1; t++) {
                if (t < t1) {
                    // S = Y T^T for tile jt: M = 128 centres, N = 64 points
                    const int b = jt & 1;
                    if (!mbar_wait_w(&t_full[s], ph, p.status, 24)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t) (SP_COL + b * P2_TILE);
                    const uint64_t bd = tdesc_k + (uint64_t) (s * (TSTAGE_BYTES >> 4));
#pragma unroll
                    for (int piece = 0; piece < 2; piece++) {
#pragma unroll
                        for (int tp = 0; tp < (piece == 0 ? NT : 1); tp++) {
#pragma unroll
                            for (int ks = 0; ks < KS; ks++)
                                mma_ts_w(d, tmem + (uint32_t) (Y_COL + piece * YCOLS + ks * 8),
                                         bd + (uint64_t) ((tp * NP + ks / 4) * (TPANEL_BYTES >> 4) +
                                                          2 * (ks % 4)),
                                         id1, (piece | tp | ks) ? 1u : 0u);
                        }
                    }
                    mma_commit_w(&s_full[b]);
                }
                if (t > t0) {
                    // R T += R (TMEM, hi/lo) x the same T tile, MN-major, N = Dp
                    const int j = jt - 1, b = j & 1;
                    if (!mbar_wait_w(&p_full[b], (uint32_t) ((j >> 1) & 1), p.status, 26)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t bd = tdesc_mn + (uint64_t) (sp * (TSTAGE_BYTES >> 4));
                    const uint32_t a0 = tmem + (uint32_t) (SP_COL + b * P2_TILE);
#pragma unroll
                    for (int rp = 0; rp < 2; rp++) {
#pragma unroll
                        for (int tp = 0; tp < (rp == 0 ? NT : 1); tp++) {
#pragma unroll
                            for (int kk = 0; kk < P2_TILE / 16; kk++)
                                // points 16 kk .. 16 kk + 15 belong to group kk / 2, whose
                                // 32 columns hold R hi (16) then R lo (16)
                                mma_ts_w(rt_tmem,
                                         a0 + (uint32_t) ((kk >> 1) * 32 + rp * 16 + (kk & 1) * 8),
                                         bd + (uint64_t) (tp * NP * (TPANEL_BYTES >> 4) + kk * (2048 >> 4)),
                                         id2, (((uint32_t) (t - 1 - t0) & (P2_SEG_TILES - 1)) != 0u ||
                                               rp | tp | kk) ? 1u : 0u);
                        }
                    }
                    // also tells the responsibility warps that a segment's
                    // R T is complete
                    mma_commit_w(&t_empty[sp]);
                }
                if (t < t1) {
                    sp = s;
                    if (++s == nstage) {
                        s = 0;
                        ph ^= 1u;
                    }
                    jt++;
                }
            }
            if (!ok)
                break;
            mma_commit_w(rt_full);
            nunit++;
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- responsibilities, the R T drain and the centre loads ----------------
        const int q = warp & 3;                 // TMEM lane quarter
        const int g = (warp - 2) >> 2;          // point group: points 32 g .. 32 g + 31 of a tile
        const int row = q * 32 + lane;          // centre within the tile
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        // This group's half of row `row` of the R T accumulator (FP32) out of
        // tensor memory, at the end of a segment (last: the unit's last one;
        // later: not the unit's first one).  With the shared-memory sums the
        // segment is stored or added there, and after the unit's last one the
        // thread's half row (384 B at D_p = 192) goes to the unit's slot as one
        // bulk copy by the TMA engine.  Without them every segment goes to the
        // slot, stored or added at L2.  Each element has this one owner
        // thread, in program order.
        float *const buf = rtbuf + row * RB;
        auto move_rt = [&](bool last, bool later, int uslot) {
            float *dst = p.RTpart + ((size_t) uslot * P2_BK + row) * DP;
            if constexpr (SEGBUF)
                bulk_wait_read();  // the previous unit's copy has left the half row
#pragma unroll 1
            for (int c0 = g * (DP / 2); c0 < (g + 1) * (DP / 2); c0 += 32) {
                uint32_t vv[32];
                tmem_ld32(lane_base + (uint32_t) c0, vv);
                tmem_ld_wait();
#pragma unroll
                for (int j = 0; j < 32; j += 4) {
                    float4 x = make_float4(__uint_as_float(vv[j]), __uint_as_float(vv[j + 1]),
                                           __uint_as_float(vv[j + 2]), __uint_as_float(vv[j + 3]));
                    if constexpr (SEGBUF) {
                        if (later) {
                            const float4 y = *(const float4 *) (buf + c0 + j);
                            x.x += y.x;
                            x.y += y.y;
                            x.z += y.z;
                            x.w += y.w;
                        }
                        *(float4 *) (buf + c0 + j) = x;
                    } else if (later) {
                        red_add_f32x4(dst + c0 + j, x.x, x.y, x.z, x.w);
                    } else {
                        *(float4 *) (dst + c0 + j) = x;
                    }
                }
            }
            if constexpr (SEGBUF) {
                if (last) {
                    fence_proxy_async_smem();
                    bulk_store(dst + g * (DP / 2), buf + g * (DP / 2), (uint32_t) (DP / 2 * 4));
                    bulk_commit();
                }
            }
        };
        // The centre row of centre tile ktc (group 0: Y hi, group 1: Y lo) into
        // tensor memory, column j holding depths 2 j and 2 j + 1, then y_ready.
        // Every load is issued before the first store: one L2 round trip.
        auto load_y = [&](int ktc) {
            const uint4 *src =
                (const uint4 *) (p.Yb + ((size_t) g * p.Kpad + (size_t) ktc * P2_BK + row) * (DP / 2));
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
        };
        int jt = 0, s = 0, nunit = 0;
        uint32_t ph = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x) {
            int u, kt, t0, t1;
            unit_of(p, v, u, kt, t0, t1);
            if (nunit == 0)
                load_y(kt);
            const bool multi = t1 - t0 > P2_SEG_TILES;
            int seg_r = t0 + P2_SEG_TILES;  // the first tile of the next segment
            for (int t = t0; t < t1; t++, jt++) {
                const int b = jt & 1;
                if (!mbar_wait(&t_full[s], ph, p.status, 27) ||
                    !mbar_wait(&s_full[b], (uint32_t) ((jt >> 1) & 1), p.status, 28)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t col0 = (uint32_t) (SP_COL + b * P2_TILE + g * 32);
                uint32_t va[32];
                tmem_ld32(lane_base + col0, va);
                tmem_ld_wait();
                const float4 *cqs = cq + s * P2_TILE + g * 32;
                uint32_t hi[16], lo[16];
#pragma unroll
                for (int j = 0; j < 16; j++) {
                    const float4 c0 = cqs[2 * j], c1 = cqs[2 * j + 1];
                    const float r0 = ex2(fmaf(__uint_as_float(va[2 * j]) - c0.x, c0.y, -c0.z));
                    const float r1 = ex2(fmaf(__uint_as_float(va[2 * j + 1]) - c1.x, c1.y, -c1.z));
                    const uint32_t h = pack_bf16(r0, r1);
                    hi[j] = h;
                    lo[j] = pack_bf16(r0 - bf16lo_to_f32(h), r1 - bf16hi_to_f32(h));
                }
                // over S: R hi in the group's first 16 columns, R lo in the next 16
                tmem_st16(lane_base + col0, hi);
                tmem_st16(lane_base + col0 + 16, lo);
                tmem_st_wait();
                if (t == seg_r) {
                    // A segment ended with tile t - 1.  Its MMA 2 completes the
                    // phase of its stage's t_empty that this wait names (the
                    // next phase needs a p_full not yet given), and this tile's
                    // p_full lets MMA 2 start the next segment over it.
                    const int sq = s == 0 ? nstage - 1 : s - 1;
                    if (!mbar_wait(&t_empty[sq], s == 0 ? ph ^ 1u : ph, p.status, 31)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    move_rt(false, t > t0 + P2_SEG_TILES, u);
                    seg_r += P2_SEG_TILES;
                }
                tc_fence_before();
                mbar_arrive(&p_full[b]);
                if (++s == nstage) {
                    s = 0;
                    ph ^= 1u;
                }
            }
            if (!ok)
                break;
            // Every MMA 1 of this unit has completed (the s_full of its last
            // tile), so the next unit's centres can replace these at once and
            // its distance products start while this unit's R T drains.  That
            // unit's first MMA 2 waits on a p_full given after the drain.
            const int vn = v + gridDim.x;
            if (vn < p.nunits) {
                int un, ktn, t0n, t1n;
                unit_of(p, vn, un, ktn, t0n, t1n);
                load_y(ktn);
            }
            if (!mbar_wait(rt_full, nunit & 1, p.status, 29)) {
                ok = false;
                break;
            }
            tc_fence_after();
            move_rt(true, multi, u);
            nunit++;
        }
        if constexpr (SEGBUF)
            bulk_wait();
        if (!ok)
            failed = 1;
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

using P2Kernel = void (*)(const CUtensorMap, const P2Params);

// the pass-2 instantiation for a shape (NP <= 3 panels, KL steps in the last, NT pieces)
P2Kernel pass2_for(int np, int kl, int nt)
{
#define DGTM_P2(NP_, KL_, NT_) \
    if (np == NP_ && kl == KL_ && nt == NT_) return tc_pass2_kernel<NP_, KL_, NT_>;
#define DGTM_P2_KL(NP_, NT_) DGTM_P2(NP_, 1, NT_) DGTM_P2(NP_, 2, NT_) DGTM_P2(NP_, 3, NT_) DGTM_P2(NP_, 4, NT_)
    DGTM_P2_KL(1, 1) DGTM_P2_KL(1, 2) DGTM_P2_KL(2, 1) DGTM_P2_KL(2, 2) DGTM_P2_KL(3, 1) DGTM_P2_KL(3, 2)
#undef DGTM_P2_KL
#undef DGTM_P2
    return nullptr;
}

// ---------------------------------------------------------------------------
// pass 3: C_n = sum_k R_kn y_k for every point (the free energy's gradient
// with respect to the data, and the projection of new points onto a map).
// The transpose of pass 2's problem: points own the rows and the centres are
// streamed.  One CTA per 128-point tile; the tile's data pieces live in
// tensor memory as the A operand of the distance product, like pass 1.  Per
// 64-centre chunk of Y (hi and lo pieces through a TMA ring):
//   MMA 1  S = T Y^T (M = 128 points, N = 64 centres, A from tensor memory);
//   eight warps (four lane quarters x two 32-centre halves) turn S into
//          R = exp2(scale (S - m) - log2 s) with the forward's per-point
//          statistics, split into BF16 hi / lo and written over S;
//   MMA 2  OUT += R Y (M = 128 points, N = D rounded up to 64, K = 16
//          centres, A = R from tensor memory, B = the same Y chunk read
//          MN-major): R_hi Y_hi + R_hi Y_lo + R_lo Y_hi.
// Two S buffers let MMA 1 of the next chunk run while the warps work.  OUT
// is moved to C (FP32, global) every P3_SEG chunks (a segment) so that no
// accumulator runs over more than 2048 centres: the tensor pipe's FP32
// accumulation drifts low over long runs of MMAs, as measured for pass 2.
// ---------------------------------------------------------------------------
constexpr int P3_THREADS = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 responsibilities
constexpr int P3_TILE = 128;     // points per CTA (MMA M)
constexpr int P3_BK = 64;        // centres per chunk
constexpr int P3_SEG = 32;       // chunks per segment of the output accumulator

struct P3Params {
    int N, D, Npad, Kpad, nchunk, nstage, nout;  // nout = D rounded up to 64
    const float4 *colq;  // Npad: (m, scale, log2 s) of each point at the temperature
    float *C;            // N x D
    int *status;
};

template <int NP, int KL, int NT>
__global__ void __launch_bounds__(P3_THREADS, 1)
    tc_rty_kernel(const __grid_constant__ CUtensorMap tmY, const __grid_constant__ CUtensorMap tmT,
                  const P3Params p)
{
    constexpr int ACOL = NP * 32;          // TMEM columns of one data piece
    constexpr int KS = 4 * (NP - 1) + KL;  // 16-deep steps of the distance product
    constexpr int YPANEL = P3_BK * 128;    // 8 KB: 64 centres x 64 depths
    constexpr int SLOT = NP * YPANEL;      // one piece (hi or lo) of a chunk
    constexpr int DPANEL = P3_TILE * 128;  // 16 KB: 128 points x 64 depths
    constexpr int NDATA = 2 * NT;          // ring slots that first hold the data pieces
    constexpr int S_COL = NT * ACOL;       // two 64-column S / R buffers
    constexpr int O_COL = S_COL + 2 * P3_BK;
    static_assert(O_COL + NP * 64 <= 512, "pass 3 tensor memory plan");
    static_assert(NDATA * SLOT == NT * NP * DPANEL, "data pieces fill whole ring slots");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int nslot = p.nstage;
    unsigned char *Yslot = base;
    uint64_t *bars = (uint64_t *) (Yslot + nslot * SLOT);
    uint64_t *y_full = bars;
    uint64_t *y_empty = bars + nslot;
    uint64_t *t_full = bars + 2 * nslot;
    uint64_t *t_done = t_full + 1;
    uint64_t *s_full = t_done + 1;   // [2]
    uint64_t *s_free = s_full + 2;   // [2]
    uint64_t *p_full = s_free + 2;   // [2]
    uint64_t *o_full = p_full + 2;
    uint64_t *o_empty = o_full + 1;
    uint64_t *drain = o_empty + 1;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * P3_TILE;
    const int nseg = (p.nchunk + P3_SEG - 1) / P3_SEG;

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < nslot; s++) {
            mbar_init(&y_full[s], 1);
            mbar_init(&y_empty[s], 1);
        }
        mbar_init(t_full, 1);
        mbar_init(t_done, 1);
        for (int b = 0; b < 2; b++) {
            mbar_init(&s_full[b], 1);
            mbar_init(&s_free[b], 1);
            mbar_init(&p_full[b], 256);
        }
        mbar_init(o_full, 1);
        mbar_init(o_empty, 256);
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
        prefetch_tmap(&tmY);
        prefetch_tmap(&tmT);
        unsigned char *dstage = Yslot + (nslot - NDATA) * SLOT;
        mbar_expect_tx(t_full, (uint32_t) (NT * NP * DPANEL));
#pragma unroll
        for (int tp = 0; tp < NT; tp++)
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(dstage + (tp * NP + pn) * DPANEL, &tmT, t_full, PANEL_ELEMS * pn,
                            tp * p.Npad + n0);
        for (int it = 0; it < 2 * p.nchunk; it++) {
            const int q = it % nslot;
            if (it >= nslot && !mbar_wait(&y_empty[q], ((it / nslot) & 1) ^ 1u, p.status, 41)) {
                failed = 1;
                break;
            }
            if (it < nslot && q >= nslot - NDATA && !mbar_wait(t_done, 0, p.status, 42)) {
                failed = 1;
                break;
            }
            const int c = it >> 1, piece = it & 1;
            mbar_expect_tx(&y_full[q], (uint32_t) SLOT);
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(Yslot + q * SLOT + pn * YPANEL, &tmY, &y_full[q], PANEL_ELEMS * pn,
                            piece * p.Kpad + c * P3_BK);
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer (whole warp; one elected lane issues) ----------------
        const uint32_t id1 = idesc_bf16(P3_TILE, P3_BK, 0, 0);
        const uint32_t id2 = idesc_bf16(P3_TILE, p.nout, 0, 1);
        const uint64_t yk = sdesc_sw128(smem_u32(Yslot), 16, 1024);      // K-major (MMA 1)
        const uint64_t ymn = sdesc_sw128(smem_u32(Yslot), YPANEL, 1024);  // MN-major (MMA 2)
        bool ok = mbar_wait_w(t_full, 0, p.status, 43);
        if (ok) {
            tc_fence_after();
            const uint64_t tdesc = yk + (uint64_t) ((nslot - NDATA) * (SLOT >> 4));
#pragma unroll
            for (int tp = 0; tp < NT; tp++)
#pragma unroll
                for (int pn = 0; pn < NP; pn++)
#pragma unroll
                    for (int kk = 0; kk < (pn == NP - 1 ? KL : 4); kk++)
                        tmem_cp_w(tmem + (uint32_t) (tp * ACOL + pn * 32 + kk * 8),
                                  tdesc + (uint64_t) ((tp * NP + pn) * (DPANEL >> 4) + 2 * kk));
            mma_commit_w(t_done);
            ok = mbar_wait_w(t_done, 0, p.status, 43);
            tc_fence_after();
        }
        for (int c = 0; ok && c <= p.nchunk; c++) {
            if (c < p.nchunk) {
                const int b = c & 1;
                if (c >= 2 && !mbar_wait_w(&s_free[b], ((c - 2) >> 1) & 1, p.status, 44)) {
                    ok = false;
                    break;
                }
                const uint32_t d = tmem + (uint32_t) (S_COL + b * P3_BK);
#pragma unroll
                for (int piece = 0; piece < 2; piece++) {
                    const int it = 2 * c + piece, q = it % nslot;
                    if (!mbar_wait_w(&y_full[q], (it / nslot) & 1, p.status, 45)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t bd = yk + (uint64_t) (q * (SLOT >> 4));
#pragma unroll
                    for (int tp = 0; tp < (piece == 0 ? NT : 1); tp++)
#pragma unroll
                        for (int ks = 0; ks < KS; ks++)
                            mma_ts_w(d, tmem + (uint32_t) (tp * ACOL + ks * 8),
                                     bd + (uint64_t) ((ks >> 2) * (YPANEL >> 4) + 2 * (ks & 3)), id1,
                                     (piece | tp | ks) ? 1u : 0u);
                }
                if (!ok)
                    break;
                mma_commit_w(&s_full[b]);
            }
            if (c > 0) {
                const int j = c - 1, b = j & 1;
                if (!mbar_wait_w(&p_full[b], (j >> 1) & 1, p.status, 46)) {
                    ok = false;
                    break;
                }
                const int seg = j / P3_SEG;
                const bool seg_first = (j % P3_SEG) == 0;
                if (seg_first && seg > 0 && !mbar_wait_w(o_empty, (seg - 1) & 1, p.status, 47)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t a0 = tmem + (uint32_t) (S_COL + b * P3_BK);
                const int qh = (2 * j) % nslot, ql = (2 * j + 1) % nslot;
#pragma unroll
                for (int pr = 0; pr < 3; pr++) {
                    // (R hi, Y hi), (R hi, Y lo), (R lo, Y hi)
                    const int rp = pr == 2 ? 1 : 0;
                    const uint64_t bd = ymn + (uint64_t) ((pr == 1 ? ql : qh) * (SLOT >> 4));
#pragma unroll
                    for (int kk = 0; kk < P3_BK / 16; kk++)
                        // centres 16 kk .. 16 kk + 15 belong to half kk / 2, whose 32
                        // columns hold R hi (16) then R lo (16)
                        mma_ts_w(tmem + (uint32_t) O_COL,
                                 a0 + (uint32_t) ((kk >> 1) * 32 + rp * 16 + (kk & 1) * 8),
                                 bd + (uint64_t) (kk * (2048 >> 4)), id2,
                                 (!seg_first || pr || kk) ? 1u : 0u);
                }
                mma_commit_w(&y_empty[qh]);
                mma_commit_w(&y_empty[ql]);
                mma_commit_w(&s_free[b]);
                if ((j % P3_SEG) == P3_SEG - 1 || j == p.nchunk - 1)
                    mma_commit_w(o_full);
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- responsibilities and the segment drains ----------------
        const int q = warp & 3;          // TMEM lane quarter: points 32 q .. 32 q + 31
        const int h = (warp - 2) >> 2;   // centres 32 h .. 32 h + 31 of a chunk
        const int row = q * 32 + lane;
        const int n = n0 + row;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        const float4 cq = p.colq[n];  // n < Npad: padding points carry R = 0
        bool ok = true;
        // OUT (this thread's row) to C: 32-column batches, batch i to half i % 2
        auto drain_out = [&](bool add) {
#pragma unroll 1
            for (int c0 = 32 * h; c0 < p.nout; c0 += 64) {
                uint32_t v[32];
                tmem_ld32(lane_base + (uint32_t) (O_COL + c0), v);
                tmem_ld_wait();
                if (n < p.N) {
                    float *dst = p.C + (size_t) n * p.D + c0;
#pragma unroll
                    for (int e = 0; e < 32; e++) {
                        if (c0 + e < p.D)
                            dst[e] = add ? dst[e] + __uint_as_float(v[e]) : __uint_as_float(v[e]);
                    }
                }
            }
        };
        for (int c = 0; c < p.nchunk; c++) {
            const int b = c & 1;
            if (!mbar_wait(&s_full[b], (c >> 1) & 1, p.status, 48)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t col0 = (uint32_t) (S_COL + b * P3_BK + h * 32);
            uint32_t va[32];
            tmem_ld32(lane_base + col0, va);
            tmem_ld_wait();
            uint32_t hi[16], lo[16];
#pragma unroll
            for (int e = 0; e < 16; e++) {
                const float r0 = ex2(fmaf(__uint_as_float(va[2 * e]) - cq.x, cq.y, -cq.z));
                const float r1 = ex2(fmaf(__uint_as_float(va[2 * e + 1]) - cq.x, cq.y, -cq.z));
                const uint32_t hh = pack_bf16(r0, r1);
                hi[e] = hh;
                lo[e] = pack_bf16(r0 - bf16lo_to_f32(hh), r1 - bf16hi_to_f32(hh));
            }
            tmem_st16(lane_base + col0, hi);
            tmem_st16(lane_base + col0 + 16, lo);
            tmem_st_wait();
            tc_fence_before();
            mbar_arrive(&p_full[b]);
            if ((c % P3_SEG) == P3_SEG - 1 || c == p.nchunk - 1) {
                const int seg = c / P3_SEG;
                if (!mbar_wait(o_full, seg & 1, p.status, 49)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                drain_out(seg > 0);
                if (seg + 1 < nseg) {
                    tc_fence_before();
                    mbar_arrive(o_empty);
                }
            }
        }
        if (!ok)
            failed = 1;
    }
    __syncthreads();
    if (failed && warp == 1) {
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 50, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

using P3Kernel = void (*)(const CUtensorMap, const CUtensorMap, const P3Params);

// the pass-3 instantiation for a shape (NP <= 3 panels, KL steps in the last, NT pieces)
P3Kernel pass3_for(int np, int kl, int nt)
{
#define DGTM_P3(NP_, KL_, NT_) \
    if (np == NP_ && kl == KL_ && nt == NT_) return tc_rty_kernel<NP_, KL_, NT_>;
#define DGTM_P3_KL(NP_, NT_) DGTM_P3(NP_, 1, NT_) DGTM_P3(NP_, 2, NT_) DGTM_P3(NP_, 3, NT_) DGTM_P3(NP_, 4, NT_)
    DGTM_P3_KL(1, 1) DGTM_P3_KL(1, 2) DGTM_P3_KL(2, 1) DGTM_P3_KL(2, 2) DGTM_P3_KL(3, 1) DGTM_P3_KL(3, 2)
#undef DGTM_P3_KL
#undef DGTM_P3
    return nullptr;
}

// ---------------------------------------------------------------------------
// operand preparation and the slot reduction
// ---------------------------------------------------------------------------
// flags |= 1 when a value is not exactly a BF16 number, |= 2 when a value is
// neither 0 nor 1
__global__ void t_class_kernel(const double *__restrict__ T64, size_t n, int *flags)
{
    int f = 0;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x) {
        const double t = T64[i];
        const double h = (double) __bfloat162float(__float2bfloat16_rn((float) t));
        if (h != t)
            f |= 1;
        if (t != 0.0 && t != 1.0)
            f |= 2;
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if (f && (threadIdx.x & 31) == 0)
        atomicOr(flags, f);
}

// T pieces (nT x Npad x Dp): value pieces, three columns of ones, zero
// padding.  F: the data as the caller holds it (FP64 for a context, FP32 for
// the free energy); the second piece is the remainder t - hi, rounded to BF16.
template <typename F>
__global__ void t_split_kernel(const F *__restrict__ T, int N, int D, int Dp, int Npad, int nT,
                               __nv_bfloat16 *__restrict__ Tb)
{
    const size_t total = (size_t) Npad * Dp;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int n = (int) (i / Dp), d = (int) (i % Dp);
        float hi = 0.f, lo = 0.f;
        if (n < N) {
            if (d < D) {
                const F t = T[(size_t) n * D + d];
                const __nv_bfloat16 h = __float2bfloat16_rn((float) t);
                hi = __bfloat162float(h);
                lo = (float) (t - (F) hi);
            } else if (d < D + 3) {
                hi = 1.f;
            }
        }
        Tb[i] = __float2bfloat16_rn(hi);
        if (nT == 2)
            Tb[total + i] = __float2bfloat16_rn(lo);
    }
}

// Y pieces (2 x Kpad x Dp) with the folded -|y_hat|^2/2 column, and Y in FP32
// (when Y32 is not null).  One warp per centre row.
template <typename F>
__global__ void y_split_kernel(const F *__restrict__ Y64, int K, int D, int Dp, int Kpad,
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
            const double y = (double) Y64[(size_t) k * D + d];
            const __nv_bfloat16 h = __float2bfloat16_rn((float) y);
            const double hd = (double) __bfloat162float(h);
            const __nv_bfloat16 l = __float2bfloat16_rn((float) (y - hd));
            const double yh = hd + (double) __bfloat162float(l);
            hi[d] = h;
            lo[d] = l;
            if (Y32)
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
// The FP32 slot values are summed with an error-free FP32 TwoSum (the rounding
// error of each addition is carried in a second FP32 word), in slot order,
// and hi + lo is formed in FP64: as exact as FP64 accumulation of the same
// FP32 inputs would be, without loading the narrow FP64 pipe.
__global__ void slot_reduce_kernel(const float *__restrict__ RTpart, int K, int D, int Dp, int U,
                                   double *__restrict__ G, double *__restrict__ RT)
{
    const size_t total = (size_t) K * (D + 1);
    const size_t ustride = (size_t) P2_BK * Dp;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int k = (int) (i / (D + 1)), d = (int) (i % (D + 1));
        const int kt = k / P2_BK, kl = k % P2_BK;
        const float *src = RTpart + ((size_t) kt * U * P2_BK + kl) * Dp + d;
        float hi = 0.f, lo = 0.f;
        int u = 0;
        for (; u + 8 <= U; u += 8) {
            float x[8];
#pragma unroll
            for (int j = 0; j < 8; j++)
                x[j] = src[(size_t) (u + j) * ustride];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float t = hi + x[j];
                const float bp = t - hi;
                lo += (hi - (t - bp)) + (x[j] - bp);
                hi = t;
            }
        }
        for (; u < U; u++) {
            const float xv = src[(size_t) u * ustride];
            const float t = hi + xv;
            const float bp = t - hi;
            lo += (hi - (t - bp)) + (xv - bp);
            hi = t;
        }
        const double sum = (double) hi + (double) lo;
        if (d < D)
            RT[(size_t) k * D + d] = sum;
        else
            G[k] = sum;
    }
}

using P1Kernel = void (*)(const CUtensorMap, const CUtensorMap, const P1Params);

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

// Pass-2 unit length in tiles.  CTA b takes units v = b, b + grid, ...; a
// unit boundary costs about four tiles' time (pipeline drain, centre reload,
// R T drain) and each unit adds a slot to the final sum (~0.02 tile-times).
// Among whole-segment lengths of 256..640 tiles (16K..40K points) take the
// one that minimises the busiest CTA's tiles + 4 x its units, + 0.02 x all
// units.  At N = 1M, K = 8000 on 152 SMs that is 384 tiles, which measured
// fastest of 256 / 384 / 512 / 640 (5.56 ms against 5.72 / 5.65 / 5.63).
static int p2_unit_tiles(int ntiles, int ktiles, int grid_max)
{
    int best = 256;
    double best_cost = 0.0;
    std::vector<long> work;
    for (int ut = 256; ut <= 640; ut += P2_SEG_TILES) {
        const long upk = (ntiles + ut - 1) / ut;
        const long nunits = upk * ktiles;
        const int grid = nunits < grid_max ? (int) nunits : grid_max;
        work.assign((size_t) grid, 0);
        for (long v = 0; v < nunits; v++) {
            const long t0 = (v / ktiles) * ut;
            work[(size_t) (v % grid)] += std::min<long>(ntiles - t0, ut) + 4;
        }
        const double cost = (double) *std::max_element(work.begin(), work.end()) + 0.02 * (double) nunits;
        if (ut == 256 || cost < best_cost) {
            best_cost = cost;
            best = ut;
        }
    }
    return best;
}

struct TcState {
    int N, D, K, sms;
    int Dp, npanel, Npad, Kpad, nT, ksteps;
    int binary;  // every data value is 0 or 1
    int nchunk, nstage1, nstage2, nstage3, ntile1, bn2;
    int ntiles2, unit_tiles, units_per_k, nunits, grid2;
    size_t smem1, smem2, smem3;
    P1Kernel pass1;
    P2Kernel pass2;
    P3Kernel pass3;
    __nv_bfloat16 *Tb, *Yb;
    float *Y32;
    float4 *colq;
    float *RTpart;
    int *status, *hstatus;
    const double *tt, *T64;
    const float *T32;  // the data in FP32 (free energy), or null
    CUtensorMap tmT1, tmT2, tmY1, tmY3;
};

static int grid_for(size_t n, int per = 256, int cap = 8192)
{
    size_t b = (n + per - 1) / per;
    if (b > (size_t) cap)
        b = cap;
    return b == 0 ? 1 : (int) b;
}

// The split form's shapes, kernel instantiations and shared-memory plans for
// N points, K centres, D dimensions and nT data pieces (no allocation).
static int tc_plan(TcState *st, int N, int D, int K, int sms, int nT)
{
    if (D + 3 > 3 * PANEL_ELEMS) {
        // pass 2 keeps the R T accumulator (D + 3 padded to 64-column panels),
        // two S/P buffers and the centres in the 512 tensor-memory columns
        set_error(DGTM_ENOTSUP, "the split-BF16 form supports D <= 189 (D = %d)", D);
        return DGTM_ENOTSUP;
    }
    st->N = N;
    st->D = D;
    st->K = K;
    st->sms = sms;
    st->nT = nT;
    st->Dp = round_up(D + 3, PANEL_ELEMS);
    st->npanel = st->Dp / PANEL_ELEMS;
    st->ksteps = (D + 3 + 15) / 16;  // columns D + 3 .. Dp - 1 are zero in both operands
    st->Npad = round_up(N, NPAD_ALIGN);
    st->Kpad = round_up(K, P1_BK);
    st->nchunk = st->Kpad / P1_BK;
    // exact 0/1 data: two 128-point tiles per pass-1 CTA; split data (two T
    // pieces) one, to fit tensor memory.  Pass-2 tiles are 64 points.
    st->ntile1 = (nT == 1) ? 2 : 1;
    st->bn2 = P2_TILE;
    st->ntiles2 = st->Npad / st->bn2;
    const int ktiles2 = (K + P2_BK - 1) / P2_BK;
    st->unit_tiles = p2_unit_tiles(st->ntiles2, ktiles2, sms);
    st->units_per_k = (st->ntiles2 + st->unit_tiles - 1) / st->unit_tiles;
    st->nunits = ktiles2 * st->units_per_k;
    st->grid2 = st->nunits < sms ? st->nunits : sms;
    const size_t bar_bytes = 64 * 8 + 16 + 2 * 256 * 8;
    const int klast = st->ksteps - 4 * (st->npanel - 1);
    // pass 1: Y slots of one chunk piece (npanel panels of 16 KB); the data
    // tiles live in tensor memory
    const size_t slot1 = (size_t) st->npanel * P1_BK * 128;
    int ns1 = (int) ((SMEM_LIMIT - 1024 - bar_bytes) / slot1);
    if (ns1 > 12)
        ns1 = 12;
    st->pass1 = pass1_for(st->npanel, klast, nT);
    // pass 2: the point-tile ring (T pieces + column statistics); the centres
    // live in tensor memory
    const size_t ts2 = (size_t) nT * st->npanel * P2_TILE * 128 + P2_TILE * 16;
    const size_t rtbuf2 =
        p2_segbuf(st->npanel, nT) ? (size_t) P2_BK * (st->npanel * PANEL_ELEMS + 4) * 4 : 0;
    int ns2 = (int) ((SMEM_LIMIT - 1024 - bar_bytes - rtbuf2) / ts2);
    if (ns2 > 8)
        ns2 = 8;
    st->pass2 = (st->npanel <= 3) ? pass2_for(st->npanel, klast, nT) : nullptr;
    // pass 3: Y slots of one 64-centre chunk piece; the first 2 nT slots
    // stage the data tile on its way to tensor memory
    const size_t slot3 = (size_t) st->npanel * P3_BK * 128;
    int ns3 = (int) ((SMEM_LIMIT - 1024 - bar_bytes) / slot3);
    if (ns3 > 12)
        ns3 = 12;
    st->pass3 = (st->npanel <= 3) ? pass3_for(st->npanel, klast, nT) : nullptr;
    if (!st->pass2 || !st->pass3) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form supports D <= 189 (D = %d)", D);
        return DGTM_ENOTSUP;
    }
    if (ns1 < 2 || ns2 < 2 || ns3 < 4 || ns3 < 2 * nT || !st->pass1) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form does not fit shared memory (D = %d)", D);
        return DGTM_ENOTSUP;
    }
    st->nstage1 = ns1;
    st->nstage2 = ns2;
    st->nstage3 = ns3;
    st->smem1 = 1024 + (size_t) ns1 * slot1 + bar_bytes;
    st->smem2 = 1024 + (size_t) ns2 * ts2 + rtbuf2 + bar_bytes;
    st->smem3 = 1024 + (size_t) ns3 * slot3 + bar_bytes;
    cudaError_t e = cudaFuncSetAttribute(st->pass1, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int) st->smem1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(st->pass2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) st->smem2);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(st->pass3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) st->smem3);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "tc_plan: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    return DGTM_OK;
}

// The TMA maps of the operand buffers the state points to.
static int tc_maps(TcState *st)
{
    int rc;
    // T pieces stacked by rows (pass-1 data tiles, pass-2 tiles), Y pieces
    // stacked by rows (pass-1 chunks, pass-3 chunks)
    if ((rc = make_tmap_bf16(&st->tmT1, st->Tb, (uint64_t) st->nT * st->Npad, st->Dp, st->Dp,
                             P1_TILE, PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmT2, st->Tb, (uint64_t) st->nT * st->Npad, st->Dp, st->Dp,
                             P2_TILE, PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmY1, st->Yb, 2 * (uint64_t) st->Kpad, st->Dp, st->Dp, P1_BK,
                             PANEL_ELEMS)) != DGTM_OK ||
        (rc = make_tmap_bf16(&st->tmY3, st->Yb, 2 * (uint64_t) st->Kpad, st->Dp, st->Dp, P3_BK,
                             PANEL_ELEMS)) != DGTM_OK)
        return rc;
    return DGTM_OK;
}

static int sm10x_or_fail()
{
    int dev = 0, major = 0, minor = 0;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev));
    if (major != 10) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form needs a Blackwell (sm_10x) GPU, found sm_%d%d",
                  major, minor);
        return DGTM_ENOTSUP;
    }
    return DGTM_OK;
}

int tc_create(TcState **out, int N, int D, int K, int sms, const double *T64, const double *tt,
              cudaStream_t s)
{
    *out = nullptr;
    int rc = sm10x_or_fail();
    if (rc != DGTM_OK)
        return rc;
    if (D + 3 > 3 * PANEL_ELEMS) {
        set_error(DGTM_ENOTSUP, "the split-BF16 form supports D <= 189 (D = %d)", D);
        return DGTM_ENOTSUP;
    }
    TcState *st = new TcState();
    st->tt = tt;
    st->T64 = T64;
    st->T32 = nullptr;
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
        t_class_kernel<<<grid_for((size_t) N * D), 256, 0, s>>>(T64, (size_t) N * D, st->status);
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
    st->binary = (*st->hstatus & 2) == 0;
    if ((rc = tc_plan(st, N, D, K, sms, (*st->hstatus & 1) ? 2 : 1)) != DGTM_OK)
        return fail(rc);
    const size_t tpl = (size_t) st->Npad * st->Dp, ypl = (size_t) st->Kpad * st->Dp;
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
    t_split_kernel<double><<<grid_for(tpl), 256, 0, s>>>(T64, N, D, st->Dp, st->Npad, st->nT,
                                                         st->Tb);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "t_split: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    if ((rc = tc_maps(st)) != DGTM_OK)
        return fail(rc);
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

void tc_y_copies(TcState *st, YCopies *cp)
{
    cp->Y32 = st->Y32;
    cp->Yb = reinterpret_cast<uint16_t *>(st->Yb);
    cp->Dp = st->Dp;
    cp->Kpad = st->Kpad;
}

int tc_prepare_y(TcState *st, const double *Y64, cudaStream_t s)
{
    y_split_kernel<double><<<grid_for((size_t) st->Kpad * 32, 256, 4096), 256, 0, s>>>(
        Y64, st->K, st->D, st->Dp, st->Kpad, st->Yb, st->Y32);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

int tc_pass1_blocks(const TcState *st) { return st->Npad / (st->ntile1 * P1_TILE); }

int tc_estep(TcState *st, const double *, double c1, double c2, int isDA, double2 *colstat,
             double *part, cudaStream_t s, int *nlaunch, bool need_llh)
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
    p.c2l = (float) (2.0 * c2 * 1.4426950408889634);
    // without the log-likelihood only the sums at `temp` are formed (the
    // temperature-1 terms are then not meaningful; c1 still drives the
    // zero-column test)
    p.c1l = need_llh ? (float) (2.0 * c1 * 1.4426950408889634) : p.c2l;
    p.isDA = isDA;
    p.two_temps = need_llh && isDA && (c1 != c2);
    p.Y32 = st->Y32;
    p.T64 = st->T64;
    p.T32 = st->T32;
    p.Tb = (const uint32_t *) st->Tb;
    p.colstat = colstat;
    p.colq = st->colq;
    p.part = part;
    p.status = st->status;
    DGTM_CUDA_TRY(cudaMemsetAsync(st->status, 0, sizeof(int), s));
    st->pass1<<<tc_pass1_blocks(st), P1_THREADS, st->smem1, s>>>(st->tmY1, st->tmT1, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 1;
    return DGTM_OK;
}

int tc_mstep_pass(TcState *st, const double2 *, double, cudaStream_t s, int *nlaunch)
{
    P2Params p;
    p.D = st->D;
    p.Dp = st->Dp;
    p.Npad = st->Npad;
    p.Kpad = st->Kpad;
    p.ntiles = st->ntiles2;
    p.unit_tiles = st->unit_tiles;
    p.units_per_k = st->units_per_k;
    p.ktiles = (st->K + P2_BK - 1) / P2_BK;
    p.nunits = st->nunits;
    p.nstage = st->nstage2;
    p.Yb = (const uint32_t *) st->Yb;
    p.colq = st->colq;
    p.RTpart = st->RTpart;
    p.status = st->status;
    st->pass2<<<st->grid2, P2_THREADS, st->smem2, s>>>(st->tmT2, p);
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

// ---------------------------------------------------------------------------
// the free energy's tensor-core passes over caller-owned FP32 arrays
// ---------------------------------------------------------------------------
static size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

// A plan over the workspace: T always in two BF16 pieces (the data of a
// gradient step are real-valued, and the piece count must be known without
// inspecting them); Y pieces with the folded -|y|^2/2 columns; the column
// statistics; the pass-2 slots; the status word of the bounded waits.
static int fe_state(int N, int K, int D, int sms, TcState *st, TcFeLayout *L)
{
    int rc = sm10x_or_fail();
    if (rc != DGTM_OK)
        return rc;
    if ((rc = tc_plan(st, N, D, K, sms, 2)) != DGTM_OK)
        return rc;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o += align256(bytes);
        return at;
    };
    L->Tb = take(sizeof(__nv_bfloat16) * 2 * (size_t) st->Npad * st->Dp);
    L->Yb = take(sizeof(__nv_bfloat16) * 2 * (size_t) st->Kpad * st->Dp);
    L->colq = take(sizeof(float4) * (size_t) st->Npad);
    L->RTpart = take(sizeof(float) * (size_t) st->nunits * P2_BK * st->Dp);
    L->status = take(sizeof(int));
    L->total = o;
    L->pass1_blocks = tc_pass1_blocks(st);
    return DGTM_OK;
}

static int fe_bind(const TcFeLayout &L, void *ws, TcState *st)
{
    char *b = static_cast<char *>(ws);
    st->Tb = reinterpret_cast<__nv_bfloat16 *>(b + L.Tb);
    st->Yb = reinterpret_cast<__nv_bfloat16 *>(b + L.Yb);
    st->colq = reinterpret_cast<float4 *>(b + L.colq);
    st->RTpart = reinterpret_cast<float *>(b + L.RTpart);
    st->status = reinterpret_cast<int *>(b + L.status);
    st->hstatus = nullptr;
    st->T64 = nullptr;
    st->tt = nullptr;
    return tc_maps(st);
}

int tc_fe_layout(int N, int K, int D, int sms, TcFeLayout *L)
{
    TcState st{};
    return fe_state(N, K, D, sms, &st, L);
}

int tc_fe_estep(const TcFeLayout &L, void *ws, const float *Y, const float *T, int N, int K, int D,
                int sms, double c1, double c2, double2 *colstat, double *part, cudaStream_t s)
{
    TcState st{};
    TcFeLayout L2;
    int rc = fe_state(N, K, D, sms, &st, &L2);
    if (rc != DGTM_OK)
        return rc;
    if (L2.total != L.total) {
        set_error(DGTM_EINVAL, "free-energy workspace plan changed between calls");
        return DGTM_EINVAL;
    }
    if ((rc = fe_bind(L, ws, &st)) != DGTM_OK)
        return rc;
    st.Y32 = const_cast<float *>(Y);
    st.T32 = T;
    DGTM_CUDA_TRY(cudaMemsetAsync(st.status, 0, sizeof(int), s));
    const size_t tpl = (size_t) st.Npad * st.Dp;
    t_split_kernel<float><<<grid_for(tpl), 256, 0, s>>>(T, N, D, st.Dp, st.Npad, 2, st.Tb);
    DGTM_CUDA_TRY(cudaGetLastError());
    y_split_kernel<float><<<grid_for((size_t) st.Kpad * 32, 256, 4096), 256, 0, s>>>(
        Y, K, D, st.Dp, st.Kpad, st.Yb, nullptr);
    DGTM_CUDA_TRY(cudaGetLastError());
    int nl = 0;
    // tc_estep clears the status word again; a failure of this call shows
    // there.  The free energy needs the statistics at `temp` only.
    return tc_estep(&st, nullptr, c1, c2, 1, colstat, part, s, &nl, false);
}

int tc_fe_stats(const TcFeLayout &L, void *ws, int N, int K, int D, int sms, double *G,
                double *RT, cudaStream_t s)
{
    TcState st{};
    TcFeLayout L2;
    int rc = fe_state(N, K, D, sms, &st, &L2);
    if (rc != DGTM_OK || (rc = fe_bind(L, ws, &st)) != DGTM_OK)
        return rc;
    int nl = 0;
    if ((rc = tc_mstep_pass(&st, nullptr, 0.0, s, &nl)) != DGTM_OK)
        return rc;
    return tc_mstep_reduce(&st, G, RT, s, &nl);
}

int tc_fe_rty(const TcFeLayout &L, void *ws, int N, int K, int D, int sms, float *C,
              cudaStream_t s)
{
    TcState st{};
    TcFeLayout L2;
    int rc = fe_state(N, K, D, sms, &st, &L2);
    if (rc != DGTM_OK || (rc = fe_bind(L, ws, &st)) != DGTM_OK)
        return rc;
    P3Params p;
    p.N = N;
    p.D = D;
    p.Npad = st.Npad;
    p.Kpad = st.Kpad;
    p.nchunk = st.Kpad / P3_BK;
    p.nstage = st.nstage3;
    p.nout = round_up(D, PANEL_ELEMS);  // whole 128-byte swizzle atoms of the MN-major Y
    p.colq = st.colq;
    p.C = C;
    p.status = st.status;
    st.pass3<<<st.Npad / P3_TILE, P3_THREADS, st.smem3, s>>>(st.tmY3, st.tmT1, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}

void tc_view(const TcState *st, TcView *v)
{
    v->N = st->N;
    v->D = st->D;
    v->K = st->K;
    v->Dp = st->Dp;
    v->npanel = st->npanel;
    v->Npad = st->Npad;
    v->Kpad = st->Kpad;
    v->nT = st->nT;
    v->binary = st->binary;
    v->ksteps = st->ksteps;
    v->Tb = st->Tb;
    v->Yb = st->Yb;
    v->colq = st->colq;
    v->tt = st->tt;
    v->status = st->status;
}

int *tc_fe_status(const TcFeLayout &L, void *ws)
{
    return reinterpret_cast<int *>(static_cast<char *>(ws) + L.status);
}

}  // namespace dgtm
