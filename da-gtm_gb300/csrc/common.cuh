// common.cuh -- shared helpers for the DA-GTM sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/dagtm_gb300.h"

namespace dgtm {

// Host-side error record (thread-local), read through dgtm_last_error_string().
void set_error(int code, const char *fmt, ...);

#define DGTM_CUDA_TRY(expr)                                                     \
    do {                                                                        \
        cudaError_t _e = (expr);                                                \
        if (_e != cudaSuccess) {                                                \
            ::dgtm::set_error(DGTM_ECUDA, "%s:%d %s: %s", __FILE__, __LINE__,   \
                              #expr, cudaGetErrorString(_e));                   \
            return DGTM_ECUDA;                                                  \
        }                                                                       \
    } while (0)

static inline int ceil_div(long long a, long long b) { return (int) ((a + b - 1) / b); }

// Block-wide sum of one double per thread in a fixed order (deterministic).
// blockDim.x must be a multiple of 32 and at most 1024; scratch holds 32 doubles.
__device__ __forceinline__ double block_sum_fixed(double v, double *scratch)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0)
        scratch[warp] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        const int nw = blockDim.x >> 5;
        for (int w = 0; w < nw; w++)
            r += scratch[w];
        scratch[0] = r;
    }
    __syncthreads();
    r = scratch[0];
    __syncthreads();
    return r;
}

}  // namespace dgtm
