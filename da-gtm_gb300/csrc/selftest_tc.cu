// selftest_tc.cu -- checks the tensor-core building blocks used by the split-
// BF16 kernels on small integer-valued matrices (exact in BF16 and FP32):
//   variant 0: A, B K-major in shared memory (TMA, 128-byte swizzle), 2 panels
//              along K, M = 128, N = 256 (the E-step distance contraction);
//   variant 1: A K-major, B MN-major (row-major data tile), M = 128, N = 192
//              (the R T contraction with B read in its natural orientation);
//   variant 2: as 1 with A in tensor memory written by tcgen05.st (the
//              responsibilities never leave the SM).
// Each launch is one CTA of 128 threads; every wait is bounded.
#include "common.cuh"
#include "df.cuh"
#include "df2.cuh"
#include "sm100.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>
#include <stdlib.h>
#include <string.h>
#include <vector>

namespace dgtm {

using namespace sm100;

namespace {

constexpr int ST_M = 128;

__device__ __forceinline__ bool same_bits(df::f2x a, df::f2x b)
{
    return __float_as_uint(a.h) == __float_as_uint(b.h) && __float_as_uint(a.l) == __float_as_uint(b.l);
}

// The packed double-float operations (df2.cuh) against the scalar ones
// (df.cuh), lane by lane, bitwise: n argument pairs spread over [-45.5, 1]
// with full low parts, table edges and the cut; counts the mismatching lanes.
__global__ void df2_check_kernel(int n, unsigned long long *mismatch)
{
    __shared__ float2 tab[64];
    if (threadIdx.x < 64) {
        float h, l;
        df::exp_table_entry(threadIdx.x, h, l);
        tab[threadIdx.x] = make_float2(h, l);
    }
    __syncthreads();
    unsigned long long bad = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned ua = (unsigned) i * 2654435761u, ub = (unsigned) i * 40503u + 12345u;
        double xa = -45.5 + 46.5 * (double) (ua >> 8) / 16777216.0;
        double xb = (i & 3) ? -45.5 + 46.5 * (double) (ub >> 8) / 16777216.0
                            : -(double) (i % 2900) / 64.0 + 1e-9 * ((double) (ub & 1023) - 512.0);
        const df::f2x a = df::from_double(xa), b = df::from_double(xb);
        const df2::x2 e = df2::exp_df(df2::pack(a, b), tab);
        bad += !same_bits(df2::lane0(e), df::exp_df(a, tab));
        bad += !same_bits(df2::lane1(e), df::exp_df(b, tab));
        const df2::x2 m = df2::mul(df2::pack(a, b), df2::pack(b, a));
        bad += !same_bits(df2::lane0(m), df::mul(a, b)) + !same_bits(df2::lane1(m), df::mul(b, a));
        const df2::x2 s = df2::add(df2::pack(a, b), df2::pack(b, a));
        bad += !same_bits(df2::lane0(s), df::add(a, b)) + !same_bits(df2::lane1(s), df::add(b, a));
        // four FP32 values of mixed size and sign, as the slice differences are
        const float u0 = a.h * 1048576.f, v0 = -b.h * 262144.f, w0 = a.l * 1073741824.f,
                    z0 = (float) (int) (ub & 0xFFFFFu) - 524288.f;
        const df2::x2 q = df2::sum4(df2::f2_pack(u0, v0), df2::f2_pack(v0, u0), df2::f2_pack(w0, z0),
                                    df2::f2_pack(z0, w0));
        bad += !same_bits(df2::lane0(q), df::sum4(u0, v0, w0, z0)) +
               !same_bits(df2::lane1(q), df::sum4(v0, u0, z0, w0));
    }
    if (bad)
        atomicAdd(mismatch, bad);
}

__global__ void __launch_bounds__(128) selftest_kernel(const __grid_constant__ CUtensorMap ta,
                                                       const __grid_constant__ CUtensorMap tb,
                                                       const __nv_bfloat16 *__restrict__ a_rows,
                                                       int variant, float *__restrict__ out,
                                                       int *status)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    // 1024-byte aligned operand region
    unsigned char *base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    unsigned char *As = base;            // up to 2 panels x 128 rows x 128 B = 32 KB
    unsigned char *Bs = base + 32768;    // up to 64 KB
    __shared__ uint64_t bar_tma, bar_mma;
    __shared__ uint32_t tmem_base_sh;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        mbar_init(&bar_tma, 1);
        mbar_init(&bar_mma, 1);
        fence_barrier_init();
    }
    if (warp == 0) {
        tmem_alloc(&tmem_base_sh, 512);
        tc_fence_before();
    }
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const int N = (variant == 0) ? 256 : 192;

    if (variant == 2) {
        // A (128 x 32) into TMEM columns 256..271: lane m holds row m, 2 BF16 per column
        uint32_t r[16];
        const int m = threadIdx.x;
        for (int c = 0; c < 16; c++) {
            const uint32_t lo = *(const uint16_t *) &a_rows[m * 128 + 2 * c];
            const uint32_t hi = *(const uint16_t *) &a_rows[m * 128 + 2 * c + 1];
            r[c] = lo | (hi << 16);
        }
        tmem_st16(tmem + ((uint32_t) (warp * 32) << 16) + 256, r);
        tmem_st_wait();
        tc_fence_before();
    }
    __syncthreads();

    if (threadIdx.x == 0) {
        tc_fence_after();
        uint32_t bytes = 0;
        if (variant == 0) {
            bytes = 2 * 16384 + 2 * 32768;
            mbar_expect_tx(&bar_tma, bytes);
            for (int p = 0; p < 2; p++) {
                tma_load_2d(As + p * 16384, &ta, &bar_tma, 64 * p, 0);
                tma_load_2d(Bs + p * 32768, &tb, &bar_tma, 64 * p, 0);
            }
        } else {
            bytes = 16384 + 3 * 4096;
            mbar_expect_tx(&bar_tma, bytes);
            tma_load_2d(As, &ta, &bar_tma, 0, 0);
            for (int p = 0; p < 3; p++)
                tma_load_2d(Bs + p * 4096, &tb, &bar_tma, 64 * p, 0);
        }
        if (mbar_wait(&bar_tma, 0, status, 1)) {
            tc_fence_after();
            if (variant == 0) {
                const uint32_t id = idesc_bf16(ST_M, 256, 0, 0);
                for (int p = 0; p < 2; p++)
                    for (int kk = 0; kk < 4; kk++) {
                        const uint64_t a = sdesc_sw128(smem_u32(As + p * 16384 + kk * 32), 16, 1024);
                        const uint64_t b = sdesc_sw128(smem_u32(Bs + p * 32768 + kk * 32), 16, 1024);
                        mma_ss(tmem, a, b, id, (p | kk) != 0);
                    }
            } else {
                const uint32_t id = idesc_bf16(ST_M, 192, 0, 1);
                for (int kk = 0; kk < 2; kk++) {
                    const uint64_t b = sdesc_sw128(smem_u32(Bs + kk * 2048), 4096, 1024);
                    if (variant == 1) {
                        const uint64_t a = sdesc_sw128(smem_u32(As + kk * 32), 16, 1024);
                        mma_ss(tmem, a, b, id, kk != 0);
                    } else {
                        mma_ts(tmem, tmem + 256 + kk * 8, b, id, kk != 0);
                    }
                }
            }
            mma_commit(&bar_mma);
        } else {
            mbar_arrive(&bar_mma);  // let the readers go; the status reports the failure
        }
    }
    __syncwarp();
    mbar_wait(&bar_mma, 0, status, 2);
    tc_fence_after();
    const int m = warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem + ((uint32_t) (warp * 32) << 16) + c0, r);
        tmem_ld_wait();
        for (int j = 0; j < 32; j++)
            out[m * N + c0 + j] = __uint_as_float(r[j]);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0)
        tmem_dealloc(tmem, 512);
}

PFN_cuTensorMapEncodeTiled_v12000 get_encode()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000) p;
    }
    return fn;
}

}  // namespace

// 2-D BF16 tensor map: rows x cols (row-major, leading dimension ld elements),
// box box_rows x box_cols, 128-byte swizzle.
int make_tmap_bf16(CUtensorMap *map, const void *ptr, uint64_t rows, uint64_t cols, uint64_t ld,
                   uint32_t box_rows, uint32_t box_cols)
{
    PFN_cuTensorMapEncodeTiled_v12000 enc = get_encode();
    if (!enc) {
        set_error(DGTM_ECUDA, "cuTensorMapEncodeTiled is not available from the driver");
        return DGTM_ECUDA;
    }
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {ld * 2};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims,
                     strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                     CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        set_error(DGTM_ECUDA, "cuTensorMapEncodeTiled failed (%d): rows=%llu cols=%llu box=%ux%u",
                  (int) r, (unsigned long long) rows, (unsigned long long) cols, box_rows, box_cols);
        return DGTM_ECUDA;
    }
    return DGTM_OK;
}

// The failure path of every bounded wait: one thread waits, with the given
// limit, on an mbarrier that nothing arrives at, exactly as the tensor-core
// kernels wait (mbar_wait: hardware-suspended try_wait, wall-clock limit),
// records the probe's site code in the status word when it gives up, and the
// kernel returns normally.
constexpr int WAIT_PROBE_SITE = 90;

__global__ void wait_probe_kernel(int *status, unsigned long long limit_ns,
                                  unsigned long long *waited_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_barrier_init();
        const uint64_t t0 = globaltimer_ns();
        mbar_wait(&bar, 0, status, WAIT_PROBE_SITE, limit_ns);
        *waited_ns = globaltimer_ns() - t0;
    }
}

static uint16_t f2bf(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return (uint16_t) (u >> 16);  // exact for the small integers used here
}

}  // namespace dgtm

using namespace dgtm;

extern "C" int dgtm_selftest(double *errs, int nerrs)
{
    if (!errs || nerrs < 3) {
        set_error(DGTM_EINVAL, "dgtm_selftest needs room for 3 results");
        return DGTM_EINVAL;
    }
    if (nerrs >= 4) {
        // the packed double-float operations against the scalar ones
        unsigned long long *dm = nullptr, hm = 0;
        cudaError_t e = cudaMalloc((void **) &dm, sizeof(unsigned long long));
        if (e == cudaSuccess)
            e = cudaMemset(dm, 0, sizeof(unsigned long long));
        if (e == cudaSuccess) {
            df2_check_kernel<<<256, 256>>>(1 << 20, dm);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess)
            e = cudaMemcpy(&hm, dm, sizeof(hm), cudaMemcpyDeviceToHost);
        cudaFree(dm);
        if (e != cudaSuccess) {
            set_error(DGTM_ECUDA, "selftest: %s", cudaGetErrorString(e));
            return DGTM_ECUDA;
        }
        errs[3] = (double) hm;
    }
    // host data: A 128 x 128, B0 256 x 128 (K-major), B1 32 x 192 (MN-major)
    std::vector<uint16_t> hA(128 * 128), hB0(256 * 128), hB1(32 * 192);
    std::vector<float> fA(128 * 128), fB0(256 * 128), fB1(32 * 192);
    for (int i = 0; i < 128; i++)
        for (int k = 0; k < 128; k++) {
            float v = (float) ((i * 7 + k * 3) % 5 - 2);
            fA[i * 128 + k] = v;
            hA[i * 128 + k] = f2bf(v);
        }
    for (int n = 0; n < 256; n++)
        for (int k = 0; k < 128; k++) {
            float v = (float) ((n * 5 + k * 11) % 7 - 3);
            fB0[n * 128 + k] = v;
            hB0[n * 128 + k] = f2bf(v);
        }
    for (int k = 0; k < 32; k++)
        for (int n = 0; n < 192; n++) {
            float v = (float) ((k * 13 + n * 3) % 9 - 4);
            fB1[k * 192 + n] = v;
            hB1[k * 192 + n] = f2bf(v);
        }
    void *dA = nullptr, *dB0 = nullptr, *dB1 = nullptr;
    float *dOut = nullptr;
    int *dSt = nullptr;
    int rc = DGTM_OK;
    std::vector<float> out(128 * 256);
    const size_t smem = 1024 + 32768 + 65536;
#define ST_CK(expr)                                                                   \
    do {                                                                              \
        cudaError_t _e = (expr);                                                      \
        if (_e != cudaSuccess) {                                                      \
            set_error(DGTM_ECUDA, "selftest: %s: %s", #expr, cudaGetErrorString(_e)); \
            rc = DGTM_ECUDA;                                                          \
            goto done;                                                                \
        }                                                                             \
    } while (0)
    {
        ST_CK(cudaMalloc(&dA, hA.size() * 2));
        ST_CK(cudaMalloc(&dB0, hB0.size() * 2));
        ST_CK(cudaMalloc(&dB1, hB1.size() * 2));
        ST_CK(cudaMalloc(&dOut, out.size() * 4));
        ST_CK(cudaMalloc(&dSt, sizeof(int)));
        ST_CK(cudaMemcpy(dA, hA.data(), hA.size() * 2, cudaMemcpyHostToDevice));
        ST_CK(cudaMemcpy(dB0, hB0.data(), hB0.size() * 2, cudaMemcpyHostToDevice));
        ST_CK(cudaMemcpy(dB1, hB1.data(), hB1.size() * 2, cudaMemcpyHostToDevice));
        ST_CK(cudaFuncSetAttribute(selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int) smem));
        for (int v = 0; v < 3; v++) {
            CUtensorMap ta, tb;
            if (v == 0) {
                if ((rc = make_tmap_bf16(&ta, dA, 128, 128, 128, 128, 64)) != DGTM_OK)
                    goto done;
                if ((rc = make_tmap_bf16(&tb, dB0, 256, 128, 128, 256, 64)) != DGTM_OK)
                    goto done;
            } else {
                // A: first 64 columns of the 128 x 128 matrix (K = 32 used)
                if ((rc = make_tmap_bf16(&ta, dA, 128, 128, 128, 128, 64)) != DGTM_OK)
                    goto done;
                if ((rc = make_tmap_bf16(&tb, dB1, 32, 192, 192, 32, 64)) != DGTM_OK)
                    goto done;
            }
            ST_CK(cudaMemset(dSt, 0, sizeof(int)));
            ST_CK(cudaMemset(dOut, 0, out.size() * 4));
            selftest_kernel<<<1, 128, smem>>>(ta, tb, (const __nv_bfloat16 *) dA, v, dOut, dSt);
            ST_CK(cudaGetLastError());
            ST_CK(cudaDeviceSynchronize());
            int st = 0;
            ST_CK(cudaMemcpy(&st, dSt, sizeof(int), cudaMemcpyDeviceToHost));
            if (st != 0) {
                set_error(DGTM_ETIMEOUT, "selftest variant %d: wait %d gave up", v, st);
                rc = DGTM_ETIMEOUT;
                goto done;
            }
            const int N = (v == 0) ? 256 : 192;
            ST_CK(cudaMemcpy(out.data(), dOut, (size_t) 128 * N * 4, cudaMemcpyDeviceToHost));
            double maxerr = 0.0;
            for (int m = 0; m < 128; m++)
                for (int n = 0; n < N; n++) {
                    double ref = 0.0;
                    if (v == 0) {
                        for (int k = 0; k < 128; k++)
                            ref += (double) fA[m * 128 + k] * fB0[n * 128 + k];
                    } else {
                        for (int k = 0; k < 32; k++)
                            ref += (double) fA[m * 128 + k] * fB1[k * 192 + n];
                    }
                    const double e = fabs(ref - (double) out[m * N + n]);
                    if (e > maxerr)
                        maxerr = e;
                }
            errs[v] = maxerr;
        }
    }
done:
    cudaFree(dA);
    cudaFree(dB0);
    cudaFree(dB1);
    cudaFree(dOut);
    cudaFree(dSt);
    return rc;
#undef ST_CK
}

extern "C" int dgtm_wait_probe(unsigned limit_ms, int *site, double *waited_ms)
{
    if (!site || !waited_ms || limit_ms == 0 || limit_ms > 10000) {
        set_error(DGTM_EINVAL, "dgtm_wait_probe: bad arguments (limit %u ms)", limit_ms);
        return DGTM_EINVAL;
    }
    int *dSt = nullptr;
    unsigned long long *dW = nullptr;
    int st = 0;
    unsigned long long w = 0;
    cudaError_t e = cudaMalloc((void **) &dSt, sizeof(int));
    if (e == cudaSuccess)
        e = cudaMalloc((void **) &dW, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMemset(dSt, 0, sizeof(int));
    if (e == cudaSuccess) {
        wait_probe_kernel<<<1, 32>>>(dSt, (unsigned long long) limit_ms * 1000000ull, dW);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cudaDeviceSynchronize();
    if (e == cudaSuccess)
        e = cudaMemcpy(&st, dSt, sizeof(int), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess)
        e = cudaMemcpy(&w, dW, sizeof(w), cudaMemcpyDeviceToHost);
    cudaFree(dSt);
    cudaFree(dW);
    if (e != cudaSuccess) {
        set_error(DGTM_ECUDA, "dgtm_wait_probe: %s", cudaGetErrorString(e));
        return DGTM_ECUDA;
    }
    *site = st;
    *waited_ms = (double) w * 1e-6;
    if (st != 0) {
        set_error(DGTM_ETIMEOUT, "a wait gave up (site %d) after %.1f ms", st, *waited_ms);
        return DGTM_ETIMEOUT;
    }
    return DGTM_OK;
}
