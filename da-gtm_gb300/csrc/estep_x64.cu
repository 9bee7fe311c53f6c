// estep_x64.cu -- the exact-slice form of the FP64 E-step and responsibility
// pass for 0/1 data (tcgen05 + TMA + TMEM, sm_103a).
//
// The FP64 form restates comm/comm.c:560-629 (distances) and
// comm/mpicomm.c:316-414 (responsibilities, G, R T) in FP64.  GB300 issues
// FP64 at ~1/64 of its FP32 rate, so this form keeps FP64 accuracy without
// the FP64 pipe in the O(K N D) and O(K N) work:
//
// Distances, exactly.  The centres are written in fixed point on one grid,
// y = Y_int 2^-F with |Y_int| < 2^53 (F from the largest |y| and |y|^2/2),
// and Y_int in seven balanced base-256 digits S0..S6 (|S| <= 128, exact in
// BF16).  With 0/1 data every product of a digit slice with T is a sum of at
// most D_p digits: an integer below 2^15, exact in the tensor pipe's FP32
// accumulation.  Slices are paired in the accumulator (256 S0 + S1, ...,
// 256 S4 + S5, S6: the even slice is stored pre-multiplied by 256), four
// accumulators of integers below 2^23 whose differences are exact in FP32.
// -|y|^2/2 on the same grid is spread over the D_p - D padding columns
// (where T is 1), so the contraction yields
//     acc_kn = t_n . y_k - |y_k|^2 / 2 = I_kn 2^-F,
//     I = A01 2^40 + A23 2^24 + A45 2^8 + P6,
// exact for the rounded centres (the rounding of y to 2^-F is below FP64's).
// -c (d_kn - d_ref) = 2c (acc_kn - acc_ref) is formed from the exact slice
// differences as a double-float (48 bits of the difference itself, so no
// cancellation error), and exp in double-float (df.cuh).
//
// Pass 1 (one CTA per two 128-point tiles, like the split form's pass 1):
// the data tiles live in tensor memory as the MMA A operand; Y's digit
// slices stream through a TMA ring in 32-centre chunks; each point's thread
// keeps a reference centre (the running maximum of acc) and the sums
// s_n = sum_k exp(-c (d_kn - d_ref)) at temperature 1 and at `temp` as 2^-48
// integers (uint64: exact, order-independent) plus the FP32 sum of each
// term's exact rounding remainder, rescaled when the reference moves.  Output: the column statistics (d_ref, log s_n) in FP64,
// the reference's slice partials, and the per-CTA quality terms.
//
// Pass 2 (persistent; units of 16 centres x up to 16384 points): per
// 128-point tile, MMA 1 (M = 128 points, N = 112: the seven slices of the
// 16 centres side by side) gives the slice partials; eight warps form
// R_kn = exp(-c (d_kn - d_ref) - log s_n) in 2^-48 fixed point and write its
// six base-256 digits side by side (96 rows) to shared memory; MMA 2 (M = 128
// data dimensions, A = the same T tile read MN-major, N = 96, K = 128
// points) accumulates R T and, through the ones in the padding columns, G,
// one accumulator per digit.  A digit sum over a whole unit stays below
// 2^22: exact.  At the unit's end the six sums of each (dimension, centre)
// go to global uint64 accumulators (high and low 24-bit parts: exact,
// order-independent).  A last kernel forms G and R T in FP64.
//
// The oracle's FP64 sums round in their own order; this form's results are
// the exact values for the rounded centres to ~2^-47 relative, which is the
// reference's own accuracy (FP64 sums over D, K and N).
#include "common.cuh"
#include "df.cuh"
#include "df2.cuh"
#include "kernels.cuh"
#include "sm100.cuh"
#include "x64.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

namespace dgtm {

int make_tmap_bf16(CUtensorMap *map, const void *ptr, uint64_t rows, uint64_t cols, uint64_t ld,
                   uint32_t box_rows, uint32_t box_cols);

using namespace sm100;

namespace {

constexpr int XS = 7;              // digit slices of the centres
constexpr int PANEL = 64;          // BF16 per 128-byte swizzle row
constexpr int SMEM_LIMIT = 227 * 1024;
constexpr int NPAD_ALIGN = 256;
constexpr int KPAD_ALIGN = 128;
constexpr int X_MAXK = 60000;      // per-point sums of K terms below 2^48 (1 + 2^-7) stay in 64 bits

// pass 1
constexpr int X1_THREADS = 320;    // warp 0 TMA, warp 1 MMA, warps 2-9 statistics
constexpr int X1_TILE = 128;       // points per tile; two tiles per CTA
constexpr int X1_NC = 32;          // centres per chunk (MMA N)
constexpr int X1_XB = 4;           // centres per statistics batch (4: measured faster than 8)
constexpr int X1_ACC = 256;        // TMEM column of the accumulators (2 tiles x 4 x 32)
constexpr int X1_YPANEL = X1_NC * 128;
constexpr int X1_TPANEL = X1_TILE * 128;

// pass 2
constexpr int X2_THREADS = 320;    // warp 0 TMA, warp 1 MMA, warps 2-9 responsibilities
constexpr int X2_TILE = 128;       // points per tile (MMA 1 M, MMA 2 K)
constexpr int X2_NC = 16;          // centres per unit
constexpr int X2_UNIT_TILES = 128; // 16384 points: digit sums below 2^22, unit sums below 2^62
constexpr int X2_N1 = XS * X2_NC;  // MMA 1 N: the seven slices side by side (112)
constexpr int X2_N2 = 6 * X2_NC;   // MMA 2 N: the six digits of R side by side (96)
constexpr int X2_TPANEL = X2_TILE * 128;  // 16 KB
constexpr int X2_YPANEL = X2_N1 * 128;    // 14 KB: 112 rows (slice, centre) x 64 depths
constexpr int X2_RPANEL = X2_N2 * 128;    // 12 KB: 96 rows (digit, centre) x 64 points
constexpr int X2_RBUF = 2 * X2_RPANEL;    // one tile's R digits
constexpr int X2_CONST = X2_TILE * 32;    // per-point constants of a tile: refq, lsq

__host__ __device__ constexpr int rup(int a, int b) { return (a + b - 1) / b * b; }

__device__ __forceinline__ float fu(uint32_t v) { return __uint_as_float(v); }

// ---------------------------------------------------------------------------
// operands
// ---------------------------------------------------------------------------
// flags |= 2 when a value is neither 0 nor 1
__global__ void x_class_kernel(const double *__restrict__ T64, size_t n, int *flags)
{
    int f = 0;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x) {
        const double t = T64[i];
        if (t != 0.0 && t != 1.0)
            f = 2;
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if (f && (threadIdx.x & 31) == 0)
        atomicOr(flags, f);
}

// T in BF16 (Npad x Dp): the 0/1 data, ones in the padding columns, zero rows
// of padding points
__global__ void x_tdata_kernel(const double *__restrict__ T64, int N, int D, int Dp, int Npad,
                               __nv_bfloat16 *__restrict__ Tx)
{
    const size_t total = (size_t) Npad * Dp;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int n = (int) (i / Dp), d = (int) (i % Dp);
        const double v = (n < N) ? ((d < D) ? T64[(size_t) n * D + d] : 1.0) : 0.0;
        Tx[i] = __float2bfloat16_rn((float) v);
    }
}

// the largest of |y_kd| and |y_k|^2 / (2 m) as FP64 bits (positive doubles
// order like their bit patterns)
__global__ void x_qmax_kernel(const double *__restrict__ Y, const double *__restrict__ yy, int K,
                              int D, int m, unsigned long long *qbits)
{
    double q = 0.0;
    const size_t n = (size_t) K * D;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < n;
         i += (size_t) gridDim.x * blockDim.x)
        q = fmax(q, fabs(Y[i]));
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
        q = fmax(q, 0.5 * yy[k] / (double) m);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        q = fmax(q, __shfl_xor_sync(0xffffffffu, q, o));
    if ((threadIdx.x & 31) == 0 && q > 0.0)
        atomicMax(qbits, (unsigned long long) __double_as_longlong(q));
}

__device__ __forceinline__ int x_grid_exponent(unsigned long long qbits)
{
    const double q = __longlong_as_double((long long) qbits);
    return (q > 0.0 && isfinite(q)) ? 52 - ilogb(q) : 0;
}

// the seven digit slices (7 x Kpad x Dp BF16): data columns from y, padding
// columns the pieces of -|y|^2/2, padding rows zero.  Also the grid (XScale).
__global__ void x_digits_kernel(const double *__restrict__ Y, const double *__restrict__ yy, int K,
                                int D, int Dp, int Kpad, const unsigned long long *qbits, XScale *sc,
                                __nv_bfloat16 *__restrict__ Yx)
{
    const int F = x_grid_exponent(*qbits);
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        sc->F = F;
        sc->inv = ldexp(1.0, -F);
    }
    const int m = Dp - D;
    const size_t total = (size_t) Kpad * Dp;
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int k = (int) (i / Dp), d = (int) (i % Dp);
        long long v = 0;
        if (k < K) {
            if (d < D) {
                v = llrint(ldexp(Y[(size_t) k * D + d], F));
            } else {
                const long long H = llrint(ldexp(0.5 * yy[k], F));
                const int j = d - D;
                v = -(H / m + ((long long) j < H % m ? 1 : 0));
            }
        }
        int dig[XS];
#pragma unroll
        for (int s = XS - 1; s >= 1; s--) {
            const int dd = (int) ((v + 128) & 255) - 128;
            dig[s] = dd;
            v = (v - dd) >> 8;
        }
        dig[0] = (int) v;
#pragma unroll
        for (int s = 0; s < XS; s++) {
            const int w = (s < XS - 1 && (s & 1) == 0) ? dig[s] * 256 : dig[s];
            Yx[(size_t) s * total + i] = __float2bfloat16_rn((float) w);
        }
    }
}

// ---------------------------------------------------------------------------
// pass 1
// ---------------------------------------------------------------------------
struct X1Params {
    int N, K, Kpad, Npad, nchunk, nslot, isDA, two_temps;
    double c1, c2;
    const XScale *sc;
    const double *tt;
    double2 *colstat;  // N: (d_ref, log s_n)
    float4 *refq;      // Npad: the reference centre's four slice partials
    float4 *lsq;       // Npad: (-log s_n as a double-float, flag, cut); flag 1: zero column,
                       // 2: padding; R_kn = 0 where I_kn - I_ref < cut (d_kn > dcut)
    double dcut;       // the reference's exp(-beta d / 2) underflows beyond it
    double *part;      // 2 per CTA
    int *status;
};

// A per-point sum: 2^-48 integers plus the FP32 sum of the terms' exact
// rounding remainders (df::fixed48r), so every term counts to ~2^-72.
struct XSum {
    unsigned long long i = 0ull;
    float r = 0.f;
    // adds a batch sum 0 <= E < 2^(SH + 1): df::fixed48r of E 2^-SH (exact
    // scaling), so the integers step by 2^SH and the remainders are exact
    template <int SH>
    __device__ __forceinline__ void add_batch(df::f2x e)
    {
        float rem;
        constexpr float inv = 1.0f / (float) (1 << SH);
        i += df::fixed48r({e.h * inv, e.l * inv}, rem) << SH;
        r += rem * (float) (1 << SH);
    }
    __device__ __forceinline__ double value() const { return ldexp((double) i + (double) r, -48); }
    // s *= E <= 1 (rare: when a point's reference centre moves; FP64, 2^-53)
    __device__ __forceinline__ void scale(df::f2x e)
    {
        i = (unsigned long long) llrint(((double) i + (double) r) * df::to_double(e));
        r = 0.f;
    }
};

// TWO: the sums at both temperatures (annealing with temp != 1), else at one
template <int NP, bool TWO>
__global__ void __launch_bounds__(X1_THREADS, 1)
    x_pass1_kernel(const __grid_constant__ CUtensorMap tmY, const __grid_constant__ CUtensorMap tmT,
                   const X1Params p)
{
    constexpr int ACOL = NP * 32;               // TMEM columns of one data tile
    constexpr int SLOT = NP * X1_YPANEL;        // one digit slice of a chunk
    constexpr int TSTAGE = 2 * NP * X1_TPANEL;  // both data tiles, staged in the ring's last slots
    constexpr int TSLOTS = TSTAGE / SLOT;       // 8
    constexpr int KS = 4 * NP;
    static_assert(ACOL * 2 <= X1_ACC, "tensor memory plan");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    const int nslot = p.nslot;
    unsigned char *ring = base;
    uint64_t *bars = (uint64_t *) (ring + nslot * SLOT);
    uint64_t *y_full = bars;
    uint64_t *y_empty = bars + nslot;
    uint64_t *t_full = bars + 2 * nslot;
    uint64_t *t_done = t_full + 1;
    uint64_t *acc_full = t_done + 1;   // [tile]
    uint64_t *acc_empty = acc_full + 2;
    uint64_t *drain = acc_empty + 2;
    uint32_t *tmem_sh = (uint32_t *) (drain + 1);
    float2 *tab = (float2 *) (tmem_sh + 2);
    double *red = (double *) (tab + 64);  // 2 x 256
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int n0 = blockIdx.x * 2 * X1_TILE;

    if (threadIdx.x < 64) {
        float h, l;
        df::exp_table_entry(threadIdx.x, h, l);
        tab[threadIdx.x] = make_float2(h, l);
    }
    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < nslot; s++) {
            mbar_init(&y_full[s], 1);
            mbar_init(&y_empty[s], 1);
        }
        mbar_init(t_full, 1);
        mbar_init(t_done, 1);
        for (int g = 0; g < 2; g++) {
            mbar_init(&acc_full[g], 1);
            mbar_init(&acc_empty[g], 128);
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

    if (warp == 0 && lane == 0) {
        // ---------------- producer ----------------
        prefetch_tmap(&tmY);
        prefetch_tmap(&tmT);
        unsigned char *tst = ring + (nslot - TSLOTS) * SLOT;
        mbar_expect_tx(t_full, (uint32_t) TSTAGE);
#pragma unroll
        for (int g = 0; g < 2; g++)
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(tst + (g * NP + pn) * X1_TPANEL, &tmT, t_full, PANEL * pn, n0 + g * X1_TILE);
        int q = 0;
        uint32_t ph = 0;
        for (int it = 0; it < XS * p.nchunk; it++) {
            if (it >= nslot && !mbar_wait(&y_empty[q], ph ^ 1u, p.status, 41)) {
                failed = 1;
                break;
            }
            if (it < nslot && q >= nslot - TSLOTS && !mbar_wait(t_done, 0, p.status, 42)) {
                failed = 1;  // the slot still holds a data tile
                break;
            }
            const int c = it / XS, s = it % XS;
            mbar_expect_tx(&y_full[q], (uint32_t) SLOT);
#pragma unroll
            for (int pn = 0; pn < NP; pn++)
                tma_load_2d(ring + q * SLOT + pn * X1_YPANEL, &tmY, &y_full[q], PANEL * pn,
                            s * p.Kpad + c * X1_NC);
            if (++q == nslot) {
                q = 0;
                ph ^= 1u;
            }
        }
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        const uint32_t idesc = idesc_bf16(X1_TILE, X1_NC, 0, 0);
        const uint64_t ydesc0 = sdesc_sw128(smem_u32(ring), 16, 1024);
        bool ok = mbar_wait_w(t_full, 0, p.status, 43);
        if (ok) {
            // the data tiles into tensor memory (tile g from column g ACOL)
            tc_fence_after();
            const uint64_t tdesc = ydesc0 + (uint64_t) (((nslot - TSLOTS) * SLOT) >> 4);
#pragma unroll
            for (int g = 0; g < 2; g++)
#pragma unroll
                for (int pn = 0; pn < NP; pn++)
#pragma unroll
                    for (int kk = 0; kk < 4; kk++)
                        tmem_cp_w(tmem + (uint32_t) (g * ACOL + pn * 32 + kk * 8),
                                  tdesc + (uint64_t) (((g * NP + pn) * X1_TPANEL) >> 4) + 2 * kk);
            mma_commit_w(t_done);
            ok = mbar_wait_w(t_done, 0, p.status, 43);
            tc_fence_after();
        }
        int q0 = 0;
        uint32_t ph0 = 0;
        for (int c = 0; ok && c < p.nchunk; c++) {
            int q = q0;
            uint32_t ph = ph0;
            for (int g = 0; g < 2; g++) {
                if (c > 0 && !mbar_wait_w(&acc_empty[g], (uint32_t) ((c - 1) & 1), p.status, 44)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t d0 = tmem + (uint32_t) (X1_ACC + g * 4 * X1_NC);
                const uint32_t a0 = tmem + (uint32_t) (g * ACOL);
                q = q0;
                ph = ph0;
#pragma unroll
                for (int s = 0; s < XS; s++) {
                    if (g == 0) {
                        if (!mbar_wait_w(&y_full[q], ph, p.status, 45)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                    }
                    const uint64_t bd = ydesc0 + (uint64_t) ((q * SLOT) >> 4);
                    // slices 2a and 2a + 1 into accumulator a; slice 6 alone
#pragma unroll
                    for (int ks = 0; ks < KS; ks++)
                        mma_ts_w(d0 + (uint32_t) ((s >> 1) * X1_NC), a0 + (uint32_t) (ks * 8),
                                 bd + (uint64_t) ((ks / 4) * (X1_YPANEL >> 4) + 2 * (ks % 4)), idesc,
                                 ((s & 1) || ks) ? 1u : 0u);
                    if (g == 1)
                        mma_commit_w(&y_empty[q]);
                    if (++q == nslot) {
                        q = 0;
                        ph ^= 1u;
                    }
                }
                if (!ok)
                    break;
                mma_commit_w(&acc_full[g]);
            }
            q0 = q;
            ph0 = ph;
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- statistics: one thread per point ----------------
        const int q = warp & 3, g = (warp - 2) >> 2;
        const int row = q * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        const int n = n0 + g * X1_TILE + row;
        const double inv = p.sc->inv;
        const df::f2x k1 = df::from_double(2.0 * p.c1 * inv), k2 = df::from_double(2.0 * p.c2 * inv);
        // lanes: the two temperatures of one centre (TWO), else two centres
        const df2::x2 kk = df2::pack(k1, TWO ? k2 : k1);
        // the reference centre's slice partials (and the first three scaled)
        float r0 = 0.f, r1 = 0.f, r2 = 0.f, r3 = 0.f, R0 = 0.f, R1 = 0.f, R2 = 0.f;
        bool have = false;
        // s_n at temperature 1 and at `temp`
        XSum s1, s2;
        bool ok = true;
        for (int c = 0; c < p.nchunk; c++) {
            if (!mbar_wait(&acc_full[g], (uint32_t) (c & 1), p.status, 46)) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int nvalid = min(X1_NC, p.K - c * X1_NC);  // padding centres are skipped
            const uint32_t col = lane_base + (uint32_t) (X1_ACC + g * 4 * X1_NC);
            // X1_XB centres at a time (4 x X1_XB partials in registers), so
            // that several exponential chains fit beside them; the accumulator is
            // released after the last batch is read (the tensor pipe is idle
            // far longer than the next chunk's MMAs take).  The batch loop is
            // not unrolled: one copy of its eight exponentials keeps the
            // kernel inside the instruction cache.
            constexpr int B = X1_XB;
#pragma unroll 1
            for (int bt = 0; bt < X1_NC / B; bt++) {
                uint32_t v[4 * B];
#pragma unroll
                for (int sl = 0; sl < 4; sl++)
                    tmem_ldp<B>(col + (uint32_t) (sl * X1_NC + B * bt), v + B * sl);
                tmem_ld_wait();
                if (bt == X1_NC / B - 1) {
                    tc_fence_before();
                    mbar_arrive(&acc_empty[g]);
                }
                const int nv = nvalid - B * bt;  // valid centres in this batch (padding after them)
                // the batch's largest acc, approximately (FP32 of the top two partials)
                float best = -INFINITY, b0 = 0.f, b1 = 0.f, b2 = 0.f, b3 = 0.f;
#pragma unroll
                for (int j = 0; j < B; j++) {
                    const float a = fmaf(fu(v[j]), 0x1p40f, fu(v[B + j]) * 0x1p24f);
                    if (j < nv && a > best) {
                        best = a;
                        b0 = fu(v[j]);
                        b1 = fu(v[B + j]);
                        b2 = fu(v[2 * B + j]);
                        b3 = fu(v[3 * B + j]);
                    }
                }
                if (best > -INFINITY) {
                    bool take = !have;
                    if (have) {
                        const df::f2x dI = df::sum4(fmaf(b0, 0x1p40f, -R0), fmaf(b1, 0x1p24f, -R1),
                                                    fmaf(b2, 256.f, -R2), b3 - r3);
                        if (dI.h > 0.f) {
                            // the sums move to the new reference: s *= exp(-2c dI 2^-F)
                            const df::f2x nd = {-dI.h, -dI.l};
                            const df2::x2 e = df2::exp_df(df2::mul(df2::pack(nd, nd), kk), tab);
                            s1.scale(df2::lane0(e));
                            if (TWO)
                                s2.scale(df2::lane1(e));
                            take = true;
                        }
                    }
                    if (take) {
                        r0 = b0;
                        r1 = b1;
                        r2 = b2;
                        r3 = b3;
                        R0 = b0 * 0x1p40f;
                        R1 = b1 * 0x1p24f;
                        R2 = b2 * 256.f;
                        have = true;
                    }
                }
                // exact slice differences (each below 2^24), then 48 bits of
                // their sum: centres j and j + 1 in the two lanes
                auto delta2 = [&](int j) {
                    auto pair = [&](int i) { return df2::f2_pack(fu(v[i]), fu(v[i + 1])); };
                    return df2::sum4(df2::fma2(pair(j), df2::splat(0x1p40f), df2::splat(-R0)),
                                     df2::fma2(pair(B + j), df2::splat(0x1p24f), df2::splat(-R1)),
                                     df2::fma2(pair(2 * B + j), df2::splat(256.f), df2::splat(-R2)),
                                     df2::f2_sub(pair(3 * B + j), df2::splat(r3)));
                };
                // straight-line code (one basic block, so the chains overlap);
                // a padding centre's exponential is masked to 0, which adds
                // nothing to the sums.  The batch's terms (each at most 1 plus the FP32
                // pre-scan's error) are summed as double-floats (relative error
                // 3 2^-48 per add, no cancellation) and go to the fixed-point
                // sums once.
                constexpr int SH = (B == 8) ? 3 : 2;  // batch sums below 2^(SH + 1)
                if (TWO) {
                    df2::x2 e[B];
#pragma unroll
                    for (int j = 0; j < B; j += 2) {
                        const df2::x2 d = delta2(j);
                        const df::f2x d0 = df2::lane0(d), d1 = df2::lane1(d);
                        e[j] = df2::exp_df(df2::mul(df2::pack(d0, d0), kk), tab);
                        e[j + 1] = df2::exp_df(df2::mul(df2::pack(d1, d1), kk), tab);
                        const uint64_t keep0 = (j < nv) ? ~0ull : 0ull, keep1 = (j + 1 < nv) ? ~0ull : 0ull;
                        e[j].h.v &= keep0;
                        e[j].l.v &= keep0;
                        e[j + 1].h.v &= keep1;
                        e[j + 1].l.v &= keep1;
                    }
#pragma unroll
                    for (int w = 1; w < B; w *= 2)
#pragma unroll
                        for (int j = 0; j < B; j += 2 * w)
                            e[j] = df2::add(e[j], e[j + w]);
                    s1.add_batch<SH>(df2::lane0(e[0]));
                    s2.add_batch<SH>(df2::lane1(e[0]));
                } else {
                    df2::x2 e[B / 2];
#pragma unroll
                    for (int j = 0; j < B; j += 2) {
                        e[j / 2] = df2::exp_df(df2::mul(delta2(j), kk), tab);
                        const uint64_t keep =
                            ((j < nv) ? 0x00000000FFFFFFFFull : 0ull) | ((j + 1 < nv) ? 0xFFFFFFFF00000000ull : 0ull);
                        e[j / 2].h.v &= keep;
                        e[j / 2].l.v &= keep;
                    }
#pragma unroll
                    for (int w = 1; w < B / 2; w *= 2)
#pragma unroll
                        for (int j = 0; j < B / 2; j += 2 * w)
                            e[j] = df2::add(e[j], e[j + w]);
                    s1.add_batch<SH>(df::add(df2::lane0(e[0]), df2::lane1(e[0])));
                }
            }
        }
        double t1 = 0.0, t2 = 0.0;
        if (ok && n < p.N) {
            const double Iref = (double) r0 * 0x1p40 + (double) r1 * 0x1p24 + (double) r2 * 256.0 + (double) r3;
            const double dstar = p.tt[n] - 2.0 * Iref * inv;
            const double ls1 = log(s1.value());
            const double ls2 = TWO ? log(s2.value()) : ls1;
            const double lsel = p.isDA ? ls2 : ls1;
            t1 = -p.c1 * dstar + ls1;
            t2 = p.isDA ? (-p.c2 * dstar + ls2) : 0.0;
            double lsn = lsel;
            float flag = 0.f;
            // comm/mpicomm.c:382-389 zero-column fallback
            if (p.c1 * dstar > 700.0 && exp(-p.c1 * dstar) == 0.0) {
                lsn = NAN;
                flag = 1.f;
                if (p.isDA) {
                    t1 = -INFINITY;
                    t2 = log((double) p.K);
                } else {
                    t1 = log((double) p.K);
                }
            }
            p.colstat[n] = make_double2(dstar, lsn);
            p.refq[n] = make_float4(r0, r1, r2, r3);
            const df::f2x L = df::from_double(flag != 0.f ? 0.0 : lsel);
            // d_kn > dcut <=> acc_kn < (|t_n|^2 - dcut) / 2 <=> I_kn - I_ref below this
            const double cut = fmax(ldexp(0.5 * (p.tt[n] - p.dcut), p.sc->F) - Iref, -1e38);
            p.lsq[n] = make_float4(-L.h, -L.l, flag, (float) cut);
        } else if (n < p.Npad) {
            p.refq[n] = make_float4(0.f, 0.f, 0.f, 0.f);
            p.lsq[n] = make_float4(0.f, 0.f, 2.f, 0.f);
        }
        if (!ok)
            failed = 1;
        red[g * X1_TILE + row] = t1;
        red[256 + g * X1_TILE + row] = t2;
    }
    __syncthreads();
    if (warp < 2) {
        // fixed-order sums of the CTA's per-point terms (warp 0: temperature
        // 1, warp 1: `temp`), each lane a contiguous run, then a butterfly
        constexpr int PER = 2 * X1_TILE / 32;
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
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 47, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

using X1Kernel = void (*)(const CUtensorMap, const CUtensorMap, const X1Params);

template <bool TWO>
X1Kernel pass1_for(int np)
{
    return np == 1   ? x_pass1_kernel<1, TWO>
           : np == 2 ? x_pass1_kernel<2, TWO>
           : np == 3 ? x_pass1_kernel<3, TWO>
                     : nullptr;
}

// ---------------------------------------------------------------------------
// pass 2
// ---------------------------------------------------------------------------
struct X2Params {
    int K, Kpad, ntiles, unit_tiles, kblocks, nunits;
    double c;
    const XScale *sc;
    const float4 *refq, *lsq;
    unsigned long long *RTacc;  // 2 x Kpad x Dp: sums of the high and low 24 bits
    int *status;
};

// unit v: point-major (all CTAs stream the same point tiles, which stay in L2)
__device__ __forceinline__ void x_unit(const X2Params &p, int v, int &kb, int &t0, int &t1)
{
    const int nu = v / p.kblocks;
    kb = v % p.kblocks;
    t0 = nu * p.unit_tiles;
    t1 = min(p.ntiles, t0 + p.unit_tiles);
}

// BF16 bits of a small non-negative integer (exact: at most 8 significant bits)
__device__ __forceinline__ uint32_t bf16_small(uint32_t v)
{
    return __float_as_uint(__uint_as_float(0x4B000000u | v) - 8388608.0f) >> 16;
}

template <int NP>
__global__ void __launch_bounds__(X2_THREADS, 1)
    x_pass2_kernel(const __grid_constant__ CUtensorMap tmY, const __grid_constant__ CUtensorMap tmT,
                   const X2Params p)
{
    constexpr int DP = NP * PANEL;
    constexpr int KS = 4 * NP;
    constexpr int TSTAGE = NP * X2_TPANEL + X2_CONST;
    constexpr int YBYTES = NP * X2_YPANEL;
    constexpr int NBLK = (DP > 128) ? 2 : 1;       // 128-dimension blocks of R T
    constexpr int MB1 = (DP > 128) ? DP - 128 : 0; // first dimension of block 1
    constexpr int S_COL = 0;                       // 2 buffers of 112 (slice, centre), 128 apart
    constexpr int S_STRIDE = 128;
    constexpr int RT_COL = 256;                    // NBLK blocks x 96 (digit, centre)
    static_assert(X2_N1 <= S_STRIDE && 2 * S_STRIDE <= RT_COL && RT_COL + NBLK * X2_N2 <= 512,
                  "tensor memory plan");
    static_assert(MB1 % PANEL == 0, "block 1 starts on a panel");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    // two T stages (panels + constants), then the R digit buffers, which also
    // keep the MN-major read of a one-panel stage (NP = 1) inside the
    // allocation, then the unit's centre slices
    unsigned char *Tst = base;
    unsigned char *Rbuf = Tst + 2 * TSTAGE;
    unsigned char *Ybuf = Rbuf + 2 * X2_RBUF;
    uint64_t *bars = (uint64_t *) (Ybuf + YBYTES);
    uint64_t *t_full = bars;          // 2
    uint64_t *t_empty = bars + 2;     // 2
    uint64_t *s_full = bars + 4;      // 2
    uint64_t *s_empty = bars + 6;     // 2
    uint64_t *r_full = bars + 8;      // 2
    uint64_t *r_empty = bars + 10;    // 2
    uint64_t *rt_full = bars + 12;
    uint64_t *rt_free = bars + 13;
    uint64_t *y_full = bars + 14;
    uint64_t *y_empty = bars + 15;
    uint64_t *drain = bars + 16;
    uint32_t *tmem_sh = (uint32_t *) (bars + 17);
    float2 *tab = (float2 *) (tmem_sh + 2);
    __shared__ int failed;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x < 64) {
        float h, l;
        df::exp_table_entry(threadIdx.x, h, l);
        tab[threadIdx.x] = make_float2(h, l);
    }
    if (threadIdx.x == 0) {
        failed = 0;
        for (int b = 0; b < 2; b++) {
            mbar_init(&t_full[b], 1);
            mbar_init(&t_empty[b], 1);
            mbar_init(&s_full[b], 1);
            mbar_init(&s_empty[b], 256);
            mbar_init(&r_full[b], 256);
            mbar_init(&r_empty[b], 1);
        }
        mbar_init(rt_full, 1);
        mbar_init(rt_free, 256);
        mbar_init(y_full, 1);
        mbar_init(y_empty, 1);
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
        // ---------------- producer: the unit's centre slices, then its point tiles ----------------
        prefetch_tmap(&tmY);
        prefetch_tmap(&tmT);
        int s = 0, jt = 0, nunit = 0;
        uint32_t ph = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x, nunit++) {
            int kb, t0, t1;
            x_unit(p, v, kb, t0, t1);
            if (nunit > 0 && !mbar_wait(y_empty, (uint32_t) ((nunit - 1) & 1), p.status, 51)) {
                ok = false;
                break;
            }
            // slice sl of the unit's 16 centres into rows 16 sl .. 16 sl + 15 of each panel
            mbar_expect_tx(y_full, (uint32_t) YBYTES);
#pragma unroll
            for (int sl = 0; sl < XS; sl++)
#pragma unroll
                for (int pn = 0; pn < NP; pn++)
                    tma_load_2d(Ybuf + pn * X2_YPANEL + sl * X2_NC * 128, &tmY, y_full, PANEL * pn,
                                sl * p.Kpad + kb * X2_NC);
            for (int t = t0; t < t1; t++, jt++) {
                if (jt >= 2 && !mbar_wait(&t_empty[s], ph ^ 1u, p.status, 52)) {
                    ok = false;
                    break;
                }
                unsigned char *st = Tst + s * TSTAGE;
                mbar_expect_tx(&t_full[s], (uint32_t) (NP * X2_TPANEL + X2_CONST));
#pragma unroll
                for (int pn = 0; pn < NP; pn++)
                    tma_load_2d(st + pn * X2_TPANEL, &tmT, &t_full[s], PANEL * pn, t * X2_TILE);
                bulk_load(st + NP * X2_TPANEL, p.refq + (size_t) t * X2_TILE, X2_TILE * 16, &t_full[s]);
                bulk_load(st + NP * X2_TPANEL + X2_TILE * 16, p.lsq + (size_t) t * X2_TILE, X2_TILE * 16,
                          &t_full[s]);
                if (++s == 2) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        const uint32_t id1 = idesc_bf16(X2_TILE, X2_N1, 0, 0);  // points x (slice, centre)
        const uint32_t id2 = idesc_bf16(128, X2_N2, 1, 0);      // dimensions x (digit, centre), A MN-major
        const uint64_t tdesc_k = sdesc_sw128(smem_u32(Tst), 16, 1024);
        const uint64_t tdesc_mn = sdesc_sw128(smem_u32(Tst), X2_TPANEL, 1024);
        const uint64_t ydesc = sdesc_sw128(smem_u32(Ybuf), 16, 1024);
        const uint64_t rdesc = sdesc_sw128(smem_u32(Rbuf), 16, 1024);
        int jt = 0, s = 0, sp = 0, nunit = 0;
        uint32_t ph = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x, nunit++) {
            int kb, t0, t1;
            x_unit(p, v, kb, t0, t1);
            if (!mbar_wait_w(y_full, (uint32_t) (nunit & 1), p.status, 53)) {
                ok = false;
                break;
            }
            tc_fence_after();
            for (int t = t0; t <= t1; t++) {
                if (t < t1) {
                    // MMA 1: the seven slice partials of tile jt (M = 128 points, N = 112)
                    const int b = jt & 1;
                    if (!mbar_wait_w(&t_full[s], ph, p.status, 54) ||
                        (jt >= 2 && !mbar_wait_w(&s_empty[b], (uint32_t) (((jt - 2) >> 1) & 1), p.status, 55))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem + (uint32_t) (S_COL + b * S_STRIDE);
                    const uint64_t ad = tdesc_k + (uint64_t) ((s * TSTAGE) >> 4);
#pragma unroll
                    for (int ks = 0; ks < KS; ks++)
                        mma_ss_w(d, ad + (uint64_t) ((ks / 4) * (X2_TPANEL >> 4) + 2 * (ks % 4)),
                                 ydesc + (uint64_t) ((ks / 4) * (X2_YPANEL >> 4) + 2 * (ks % 4)), id1,
                                 ks ? 1u : 0u);
                    mma_commit_w(&s_full[b]);
                    if (t == t1 - 1)
                        mma_commit_w(y_empty);  // the unit's centre slices are read
                }
                if (t > t0) {
                    // MMA 2: R T of tile jt - 1 (M = 128 dimensions, N = 96, K = 128 points)
                    const int j = jt - 1, rb = j & 1;
                    const bool first = (t - 1 == t0);
                    if (!mbar_wait_w(&r_full[rb], (uint32_t) ((j >> 1) & 1), p.status, 56) ||
                        (first && nunit > 0 &&
                         !mbar_wait_w(rt_free, (uint32_t) ((nunit - 1) & 1), p.status, 57))) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t ad = tdesc_mn + (uint64_t) ((sp * TSTAGE) >> 4);
                    const uint64_t bd = rdesc + (uint64_t) ((rb * X2_RBUF) >> 4);
#pragma unroll
                    for (int mb = 0; mb < NBLK; mb++)
#pragma unroll
                        for (int kk = 0; kk < X2_TILE / 16; kk++)
                            mma_ss_w(tmem + (uint32_t) (RT_COL + mb * X2_N2),
                                     ad + (uint64_t) ((mb ? (MB1 / PANEL) * (X2_TPANEL >> 4) : 0) +
                                                      kk * (2048 >> 4)),
                                     bd + (uint64_t) ((kk >> 2) * (X2_RPANEL >> 4) + 2 * (kk & 3)), id2,
                                     (!first || kk) ? 1u : 0u);
                    mma_commit_w(&t_empty[sp]);
                    mma_commit_w(&r_empty[rb]);
                    if (t == t1)
                        mma_commit_w(rt_full);  // the unit's R T is complete
                }
                if (t < t1) {
                    sp = s;
                    if (++s == 2) {
                        s = 0;
                        ph ^= 1u;
                    }
                    jt++;
                }
            }
        }
        if (!ok)
            failed = 1;
    } else if (warp >= 2) {
        // ---------------- responsibilities (R digits) and the unit's R T ----------------
        const int q = warp & 3, g = (warp - 2) >> 2;
        const uint32_t lane_base = tmem + ((uint32_t) (q * 32) << 16);
        const int pt = q * 32 + lane;  // point within a tile (digits), row of R T (drain)
        const double inv = p.sc->inv;
        const df::f2x kc = df::from_double(2.0 * p.c * inv);
        const unsigned long long rinvK = ((1ull << 48) + (unsigned long long) (p.K / 2)) / (unsigned long long) p.K;
        // drain ownership: block g, rows 32 q + lane, dimension dim
        const int mb = g;
        const int dim = (mb == 0 ? 0 : MB1) + pt;
        const bool own = (mb < NBLK) && (mb == 0 ? (q * 32 < DP) : (q * 32 >= 256 - DP));
        int jt = 0, s = 0, nunit = 0;
        uint32_t ph = 0;
        bool ok = true;
        for (int v = blockIdx.x; ok && v < p.nunits; v += gridDim.x, nunit++) {
            int kb, t0, t1;
            x_unit(p, v, kb, t0, t1);
            for (int t = t0; t < t1; t++, jt++) {
                const int b = jt & 1;
                if (!mbar_wait(&t_full[s], ph, p.status, 59) ||
                    !mbar_wait(&s_full[b], (uint32_t) ((jt >> 1) & 1), p.status, 60)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // this group's 8 centres of the seven slices: columns 16 sl + 8 g
                uint32_t va[XS * 8];
                {
                    const uint32_t col = lane_base + (uint32_t) (S_COL + b * S_STRIDE + 8 * g);
#pragma unroll
                    for (int sl = 0; sl < XS; sl++)
                        tmem_ld8p(col + (uint32_t) (sl * X2_NC), va + 8 * sl);
                    tmem_ld_wait();
                }
                tc_fence_before();
                mbar_arrive(&s_empty[b]);
                const unsigned char *cb = Tst + s * TSTAGE + NP * X2_TPANEL;
                const float4 rq = ((const float4 *) cb)[pt];
                const float4 lq = ((const float4 *) (cb + X2_TILE * 16))[pt];
                const float R0 = rq.x * 0x1p40f, R1 = rq.y * 0x1p24f, R2 = rq.z * 256.f;
                const df::f2x nls = {lq.x, lq.y};  // -log s_n
                const int flag = (int) lq.z;
                // the R buffer of tile jt is free once MMA 2 of tile jt - 2 completed
                if (jt >= 2 && !mbar_wait(&r_empty[b], (uint32_t) (((jt - 2) >> 1) & 1), p.status, 61)) {
                    ok = false;
                    break;
                }
                unsigned char *rbp = Rbuf + b * X2_RBUF + (pt >> 6) * X2_RPANEL;
                const df2::x2 kc2 = df2::pack(kc, kc), nls2 = df2::pack(nls, nls);
                // two centres at a time in the two lanes; all eight exponentials
                // first, in one basic block (the guards act on the results)
                df2::x2 dI[4];  // centres c and c + 1 in the two lanes
                df2::x2 e4[4];
#pragma unroll
                for (int c = 0; c < 8; c += 2) {
                    auto pair = [&](int i) { return df2::f2_pack(fu(va[i]), fu(va[i + 1])); };
                    // slices side by side: the even one is stored times 256, so
                    // each pair is an exact FP32 sum
                    const df2::f2 a01 = df2::f2_add(pair(c), pair(8 + c));
                    const df2::f2 a23 = df2::f2_add(pair(16 + c), pair(24 + c));
                    const df2::f2 a45 = df2::f2_add(pair(32 + c), pair(40 + c));
                    dI[c / 2] = df2::sum4(df2::fma2(a01, df2::splat(0x1p40f), df2::splat(-R0)),
                                          df2::fma2(a23, df2::splat(0x1p24f), df2::splat(-R1)),
                                          df2::fma2(a45, df2::splat(256.f), df2::splat(-R2)),
                                          df2::f2_sub(pair(48 + c), df2::splat(rq.w)));
                }
#pragma unroll
                for (int c = 0; c < 8; c += 2)
                    e4[c / 2] = df2::exp_df(df2::add(df2::mul(dI[c / 2], kc2), nls2), tab);
#pragma unroll
                for (int c = 0; c < 8; c += 2) {
                    const df2::x2 e = e4[c / 2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        const int cc = c + h;
                        uint32_t tp = 0u, bt = 0u;
                        const int k = kb * X2_NC + 8 * g + cc;
                        if (k < p.K) {
                            // R = 0 where the reference's exp(-beta d / 2) underflows
                            const float dh = h ? df2::f2_hi(dI[c / 2].h) : df2::f2_lo(dI[c / 2].h);
                            if (flag == 0 && !(dh < lq.w)) {
                                df::fixed48_parts(h ? df2::lane1(e) : df2::lane0(e), tp, bt);
                            } else if (flag == 1) {
                                // comm/mpicomm.c:382-389: R = 1/K
                                tp = (uint32_t) (rinvK >> 24);
                                bt = (uint32_t) (rinvK & 0xFFFFFFull);
                            }
                            if (bt >= (1u << 24)) {
                                tp += 1u;
                                bt -= 1u << 24;
                            }
                            if (tp >= (1u << 24)) {  // R = 1: just below 2^48
                                tp = (1u << 24) - 1u;
                                bt = (1u << 24) - 1u;
                            }
                        }
                        // digit d of R at row 16 d + 8 g + cc, column pt (K-major, 128-byte swizzle)
                        const int cr = 8 * g + cc;
                        unsigned char *rowp = rbp + cr * 128 + ((((pt & 63) >> 3) ^ (cr & 7)) << 4) + (pt & 7) * 2;
                        *(uint16_t *) (rowp + 0 * X2_NC * 128) = (uint16_t) bf16_small(tp >> 16);
                        *(uint16_t *) (rowp + 1 * X2_NC * 128) = (uint16_t) bf16_small((tp >> 8) & 255u);
                        *(uint16_t *) (rowp + 2 * X2_NC * 128) = (uint16_t) bf16_small(tp & 255u);
                        *(uint16_t *) (rowp + 3 * X2_NC * 128) = (uint16_t) bf16_small(bt >> 16);
                        *(uint16_t *) (rowp + 4 * X2_NC * 128) = (uint16_t) bf16_small((bt >> 8) & 255u);
                        *(uint16_t *) (rowp + 5 * X2_NC * 128) = (uint16_t) bf16_small(bt & 255u);
                    }
                }
                fence_proxy_async_smem();
                mbar_arrive(&r_full[b]);
                if (++s == 2) {
                    s = 0;
                    ph ^= 1u;
                }
            }
            if (!ok)
                break;
            // the unit's R T: six exact digit sums per (dimension, centre), to
            // the global accumulators (exact, order-independent)
            if (!mbar_wait(rt_full, (uint32_t) (nunit & 1), p.status, 58)) {
                ok = false;
                break;
            }
            tc_fence_after();
            if (own) {
                unsigned long long acc[X2_NC];
#pragma unroll
                for (int c = 0; c < X2_NC; c++)
                    acc[c] = 0ull;
                const uint32_t col = lane_base + (uint32_t) (RT_COL + mb * X2_N2);
#pragma unroll
                for (int dg = 0; dg < 6; dg++) {
                    uint32_t w[X2_NC];
                    tmem_ld16p(col + (uint32_t) (dg * X2_NC), w);
                    tmem_ld_wait();
#pragma unroll
                    for (int c = 0; c < X2_NC; c++)
                        acc[c] += (unsigned long long) __float2uint_rz(fu(w[c])) << (8 * (5 - dg));
                }
                if (dim < DP) {
#pragma unroll
                    for (int c = 0; c < X2_NC; c++) {
                        const int k = kb * X2_NC + c;
                        if (k < p.K) {
                            unsigned long long *dst = p.RTacc + (size_t) k * DP + dim;
                            atomicAdd(dst, acc[c] >> 24);
                            atomicAdd(dst + (size_t) p.Kpad * DP, acc[c] & 0xFFFFFFull);
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(rt_free);
        }
        if (!ok)
            failed = 1;
    }
    __syncthreads();
    if (failed && warp == 1) {
        mma_commit_w(drain);
        mbar_wait_w(drain, 0, p.status, 62, 100000000ull);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

using X2Kernel = void (*)(const CUtensorMap, const CUtensorMap, const X2Params);

X2Kernel pass2_for(int np)
{
    return np == 1 ? x_pass2_kernel<1> : np == 2 ? x_pass2_kernel<2> : np == 3 ? x_pass2_kernel<3> : nullptr;
}

// G and R T in FP64 from the exact sums: value = hi 2^-24 + lo 2^-48
__global__ void x_finish_kernel(const unsigned long long *__restrict__ RTacc, int K, int D, int Dp,
                                int Kpad, double *__restrict__ G, double *__restrict__ RT)
{
    const size_t total = (size_t) K * (D + 1);
    for (size_t i = blockIdx.x * (size_t) blockDim.x + threadIdx.x; i < total;
         i += (size_t) gridDim.x * blockDim.x) {
        const int k = (int) (i / (D + 1)), d = (int) (i % (D + 1));
        const size_t at = (size_t) k * Dp + d;
        const double v = ldexp((double) RTacc[at], -24) + ldexp((double) RTacc[(size_t) Kpad * Dp + at], -48);
        if (d < D)
            RT[(size_t) k * D + d] = v;
        else
            G[k] = v;
    }
}

int grid_for(size_t n, int per = 256, int cap = 8192)
{
    size_t g = (n + per - 1) / per;
    if (g < 1)
        g = 1;
    if (g > (size_t) cap)
        g = cap;
    return (int) g;
}

}  // namespace

struct XState {
    int N = 0, D = 0, K = 0, Dp = 0, npanel = 0, Npad = 0, Kpad = 0, sms = 0;
    int nchunk = 0, nslot = 0, blocks1 = 0;
    int ntiles = 0, kblocks = 0, nunits = 0, grid2 = 0;
    size_t smem1 = 0, smem2 = 0;
    __nv_bfloat16 *Tx = nullptr, *Yx = nullptr;
    unsigned long long *qbits = nullptr;
    XScale *sc = nullptr;
    float4 *refq = nullptr, *lsq = nullptr;
    unsigned long long *RTacc = nullptr;
    int *status = nullptr, *hstatus = nullptr;
    X1Kernel pass1 = nullptr, pass1_two = nullptr;  // one temperature, two
    X2Kernel pass2 = nullptr;
    CUtensorMap tmT, tmY1, tmY2;
};

void x64_destroy(XState *st)
{
    if (!st)
        return;
    cudaFree(st->Tx);
    cudaFree(st->Yx);
    cudaFree(st->qbits);
    cudaFree(st->sc);
    cudaFree(st->refq);
    cudaFree(st->lsq);
    cudaFree(st->RTacc);
    cudaFree(st->status);
    cudaFreeHost(st->hstatus);
    delete st;
}

int x64_create(XState **out, int N, int D, int K, int sms, const double *T64, cudaStream_t s)
{
    *out = nullptr;
    const char *env = getenv("DGTM_X64");
    if (env && strcmp(env, "0") == 0) {
        set_error(DGTM_ENOTSUP, "the exact-slice FP64 form is switched off (DGTM_X64=0)");
        return DGTM_ENOTSUP;
    }
    int dev = 0, major = 0;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    DGTM_CUDA_TRY(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
    if (major != 10) {
        set_error(DGTM_ENOTSUP, "the exact-slice FP64 form needs a Blackwell (sm_10x) GPU");
        return DGTM_ENOTSUP;
    }
    if (D + 3 > 3 * PANEL || K > X_MAXK || N < 1 || K < 1) {
        set_error(DGTM_ENOTSUP, "the exact-slice FP64 form needs D <= 189 and K <= %d", X_MAXK);
        return DGTM_ENOTSUP;
    }
    XState *st = new XState();
    auto fail = [&](int code) {
        x64_destroy(st);
        return code;
    };
    cudaError_t e = cudaMalloc((void **) &st->status, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMallocHost((void **) &st->hstatus, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMemsetAsync(st->status, 0, sizeof(int), s);
    if (e == cudaSuccess) {
        x_class_kernel<<<grid_for((size_t) N * D), 256, 0, s>>>(T64, (size_t) N * D, st->status);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(st->hstatus, st->status, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "x64_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    if (*st->hstatus & 2) {
        set_error(DGTM_ENOTSUP, "the exact-slice FP64 form needs 0/1 data");
        return fail(DGTM_ENOTSUP);
    }
    st->N = N;
    st->D = D;
    st->K = K;
    st->sms = sms;
    st->npanel = (D + 3 + PANEL - 1) / PANEL;
    st->Dp = st->npanel * PANEL;
    st->Npad = rup(N, NPAD_ALIGN);
    st->Kpad = rup(K, KPAD_ALIGN);
    st->pass1 = pass1_for<false>(st->npanel);
    st->pass1_two = pass1_for<true>(st->npanel);
    st->pass2 = pass2_for(st->npanel);
    // pass 1: the ring of digit slices (at least the staged data tiles plus a chunk)
    st->nchunk = (K + X1_NC - 1) / X1_NC;
    st->blocks1 = st->Npad / (2 * X1_TILE);
    const int slot = st->npanel * X1_YPANEL;
    const int fixed1 = 1024 + 512 + 4096 + 256;
    int nslot = (SMEM_LIMIT - fixed1) / (slot + 16);
    if (nslot > 32)
        nslot = 32;
    st->nslot = nslot;
    st->smem1 = (size_t) fixed1 + (size_t) nslot * (slot + 16);
    // pass 2
    st->ntiles = st->Npad / X2_TILE;
    st->kblocks = st->Kpad / X2_NC;
    st->nunits = ((st->ntiles + X2_UNIT_TILES - 1) / X2_UNIT_TILES) * st->kblocks;
    st->grid2 = st->nunits < sms ? st->nunits : sms;
    st->smem2 = 1024 + 2 * (size_t) (st->npanel * X2_TPANEL + X2_CONST) + 2 * (size_t) X2_RBUF +
                (size_t) st->npanel * X2_YPANEL + 17 * 8 + 8 + 512;
    if (nslot < 16 || st->smem2 > (size_t) SMEM_LIMIT || !st->pass1 || !st->pass1_two || !st->pass2) {
        set_error(DGTM_ENOTSUP, "x64_create: no shared-memory plan (D = %d)", D);
        return fail(DGTM_ENOTSUP);
    }
    const size_t tpl = (size_t) st->Npad * st->Dp, ypl = (size_t) st->Kpad * st->Dp;
    e = cudaMalloc((void **) &st->Tx, sizeof(__nv_bfloat16) * tpl);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->Yx, sizeof(__nv_bfloat16) * ypl * XS);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->qbits, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->sc, sizeof(XScale));
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->refq, sizeof(float4) * st->Npad);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->lsq, sizeof(float4) * st->Npad);
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &st->RTacc, sizeof(unsigned long long) * 2 * ypl);
    if (e != cudaSuccess) {
        set_error(DGTM_ENOMEM, "x64_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ENOMEM);
    }
    x_tdata_kernel<<<grid_for(tpl), 256, 0, s>>>(T64, N, D, st->Dp, st->Npad, st->Tx);
    e = cudaGetLastError();
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(st->pass1, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) st->smem1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(st->pass1_two, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) st->smem1);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(st->pass2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) st->smem2);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "x64_create: %s", cudaGetErrorString(e));
        return fail(DGTM_ECUDA);
    }
    int rc = make_tmap_bf16(&st->tmT, st->Tx, (uint64_t) st->Npad, st->Dp, st->Dp, X1_TILE, PANEL);
    if (rc == DGTM_OK)
        rc = make_tmap_bf16(&st->tmY1, st->Yx, (uint64_t) XS * st->Kpad, st->Dp, st->Dp, X1_NC, PANEL);
    if (rc == DGTM_OK)
        rc = make_tmap_bf16(&st->tmY2, st->Yx, (uint64_t) XS * st->Kpad, st->Dp, st->Dp, X2_NC, PANEL);
    if (rc != DGTM_OK)
        return fail(rc);
    *out = st;
    return DGTM_OK;
}

int x64_pass1_blocks(const XState *st) { return st->blocks1; }

int x64_estep(XState *st, const double *Y64, const double *yy, const double *tt, double c1,
              double c2, int isDA, double2 *colstat, double *part, cudaStream_t s, int *nlaunch)
{
    DGTM_CUDA_TRY(cudaMemsetAsync(st->status, 0, sizeof(int), s));
    DGTM_CUDA_TRY(cudaMemsetAsync(st->qbits, 0, sizeof(unsigned long long), s));
    x_qmax_kernel<<<grid_for((size_t) st->K * st->D, 256, 256), 256, 0, s>>>(Y64, yy, st->K, st->D,
                                                                             st->Dp - st->D, st->qbits);
    DGTM_CUDA_TRY(cudaGetLastError());
    x_digits_kernel<<<grid_for((size_t) st->Kpad * st->Dp), 256, 0, s>>>(
        Y64, yy, st->K, st->D, st->Dp, st->Kpad, st->qbits, st->sc, st->Yx);
    DGTM_CUDA_TRY(cudaGetLastError());
    X1Params p;
    p.N = st->N;
    p.K = st->K;
    p.Kpad = st->Kpad;
    p.Npad = st->Npad;
    p.nchunk = st->nchunk;
    p.nslot = st->nslot;
    p.isDA = isDA;
    p.two_temps = isDA && (c1 != c2);
    p.c1 = c1;
    p.c2 = c2;
    p.dcut = ref_dcut(2.0 * c1);
    p.sc = st->sc;
    p.tt = tt;
    p.colstat = colstat;
    p.refq = st->refq;
    p.lsq = st->lsq;
    p.part = part;
    p.status = st->status;
    (p.two_temps ? st->pass1_two : st->pass1)<<<st->blocks1, X1_THREADS, st->smem1, s>>>(st->tmY1, st->tmT, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 3;
    return DGTM_OK;
}

int x64_mstep_pass(XState *st, double c, double *G, double *RT, cudaStream_t s, int *nlaunch)
{
    DGTM_CUDA_TRY(cudaMemsetAsync(st->RTacc, 0, sizeof(unsigned long long) * 2 * (size_t) st->Kpad * st->Dp, s));
    X2Params p;
    p.K = st->K;
    p.Kpad = st->Kpad;
    p.ntiles = st->ntiles;
    p.unit_tiles = X2_UNIT_TILES;
    p.kblocks = st->kblocks;
    p.nunits = st->nunits;
    p.c = c;
    p.sc = st->sc;
    p.refq = st->refq;
    p.lsq = st->lsq;
    p.RTacc = st->RTacc;
    p.status = st->status;
    st->pass2<<<st->grid2, X2_THREADS, st->smem2, s>>>(st->tmY2, st->tmT, p);
    DGTM_CUDA_TRY(cudaGetLastError());
    x_finish_kernel<<<grid_for((size_t) st->K * (st->D + 1)), 256, 0, s>>>(st->RTacc, st->K, st->D, st->Dp,
                                                                            st->Kpad, G, RT);
    DGTM_CUDA_TRY(cudaGetLastError());
    *nlaunch = 2;
    return DGTM_OK;
}

int x64_fetch_status(XState *st, cudaStream_t s)
{
    DGTM_CUDA_TRY(cudaMemcpyAsync(st->hstatus, st->status, sizeof(int), cudaMemcpyDeviceToHost, s));
    return DGTM_OK;
}

int x64_check_status(XState *st)
{
    if (*st->hstatus != 0) {
        set_error(DGTM_ETIMEOUT, "an exact-slice kernel gave up waiting (site %d)", *st->hstatus);
        return DGTM_ETIMEOUT;
    }
    return DGTM_OK;
}

}  // namespace dgtm
