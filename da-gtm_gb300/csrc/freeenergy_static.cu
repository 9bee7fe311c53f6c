// freeenergy_static.cu -- the free-energy forward for callers that cannot
// allocate device memory.
//
// dgtm_fe_forward needs a device workspace from its caller.  Some callers
// have no way to provide one: code that runs where cudaMalloc is not
// allowed or not wanted (a host function or stream callback, which may not
// call CUDA at all; a process whose device memory is entirely handed out by
// another allocator, so a fresh cudaMalloc would fail or break its budget; a
// latency-critical loop that cannot afford the implicit synchronisation of an
// allocation).  dgtm_fe_forward_noalloc serves them: it runs the FP32
// CUDA-core kernels of the FP32 form (the FP32 E-step and its reductions),
// with its scratch in one fixed array of DGTM_FE_NOALLOC_BYTES compiled into
// this library.  Every GPU that loads the library holds that array until the
// process exits.  No call allocates anything itself; the first call on a
// device may be the moment the driver loads this library's device code (and
// with it the array), under CUDA's lazy module loading.
#include "common.cuh"
#include "kernels.cuh"

#include <math.h>
#include <mutex>

namespace dgtm {

namespace {

// The library's own scratch for dgtm_fe_forward_noalloc.  In host code this
// name is only a stand-in for the device array: its device address comes from
// cudaGetSymbolAddress (see scratch_on_current_device).
static __device__ __align__(256) unsigned char g_noalloc_scratch[DGTM_FE_NOALLOC_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;

// The array's device address per device, with the ID of the CUDA context it
// was looked up in.  A context that is torn down and created again (after a
// cudaDeviceReset, say) reloads this library's device code, and the array may
// then sit elsewhere: a new context ID triggers a new lookup.
struct ScratchAddr {
    unsigned long long ctx_id;
    void *addr;
};
ScratchAddr g_scratch[kMaxDevices];

typedef int (*PfnCtxGetCurrent)(void **ctx);
typedef int (*PfnCtxGetId)(void *ctx, unsigned long long *id);

// ID of the calling thread's current CUDA context (driver entry points looked
// up through the runtime, so the library does not link the driver library).
// Returns false when the thread has no current context yet.
bool current_context_id(unsigned long long *id)
{
    static PfnCtxGetCurrent get_current = nullptr;
    static PfnCtxGetId get_id = nullptr;
    if (!get_current || !get_id) {
        void *p1 = nullptr, *p2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p1, 12000, cudaEnableDefault,
                                             &q1) != cudaSuccess ||
            q1 != cudaDriverEntryPointSuccess ||
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &p2, 12000, cudaEnableDefault, &q2) !=
                cudaSuccess ||
            q2 != cudaDriverEntryPointSuccess)
            return false;
        get_current = (PfnCtxGetCurrent) p1;
        get_id = (PfnCtxGetId) p2;
    }
    void *ctx = nullptr;
    return get_current(&ctx) == 0 && ctx && get_id(ctx, id) == 0;
}

// Set-up, once per device and context: with that device current, look up the
// array's device address (cudaGetSymbolAddress).  The first lookup in a
// process may make the driver load this library's device code, which is
// when the array is reserved on that device; later calls reuse the address.
int scratch_on_current_device(void **out)
{
    int dev = 0;
    DGTM_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_error(DGTM_ENOTSUP, "device %d is beyond the %d devices this library tracks", dev,
                  kMaxDevices);
        return DGTM_ENOTSUP;
    }
    // a thread that has not used the runtime yet has no current context:
    // the lookup below binds the device's primary context, then it is named
    unsigned long long id = 0;
    bool have_id = current_context_id(&id);
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!have_id || !g_scratch[dev].addr || g_scratch[dev].ctx_id != id) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            set_error(DGTM_ECUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                      cudaGetErrorString(e));
            return DGTM_ECUDA;
        }
        if (!have_id && !current_context_id(&id)) {
            set_error(DGTM_ECUDA, "no current CUDA context for the no-alloc scratch");
            return DGTM_ECUDA;
        }
        g_scratch[dev] = ScratchAddr{id, p};
    }
    *out = g_scratch[dev].addr;
    return DGTM_OK;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t) 255; }

// Scratch carved for one forward call: |t_n|^2, |y_k|^2, the per-point
// statistics, the per-block partial sums and two scalars.
struct NoAllocLayout {
    size_t tt, yy, colstat, part, scal, total;
    int nblk;
};

NoAllocLayout layout(int N, int K)
{
    NoAllocLayout L{};
    L.nblk = pass1_simt_blocks(N);
    size_t o = 0;
    L.tt = o;
    o += align256(sizeof(double) * (size_t) N);
    L.yy = o;
    o += align256(sizeof(double) * (size_t) K);
    L.colstat = o;
    o += align256(sizeof(double2) * (size_t) N);
    L.part = o;
    o += align256(sizeof(double) * 2 * (size_t) L.nblk);
    L.scal = o;
    o += align256(sizeof(double) * 8);
    L.total = o;
    return L;
}

__global__ void noalloc_value_kernel(const double *__restrict__ S, double base, double temp,
                                     double *__restrict__ F)
{
    F[0] = base + temp * S[1];
}

}  // namespace

}  // namespace dgtm

using namespace dgtm;

extern "C" int dgtm_fe_forward_noalloc(const float *Y, const float *T, int N, int K, int D,
                                       double beta, double temp, void *stream, double *F)
{
    if (!Y || !T || !F || N < 1 || K < 1 || D < 1 || D > 256) {
        set_error(DGTM_EINVAL, "bad free-energy arguments (N=%d K=%d D=%d)", N, K, D);
        return DGTM_EINVAL;
    }
    if (!(beta > 0.0) || !isfinite(beta) || !(temp > 0.0) || !isfinite(temp)) {
        set_error(DGTM_EINVAL, "beta (%g) and temp (%g) must be positive and finite", beta, temp);
        return DGTM_EINVAL;
    }
    const NoAllocLayout L = layout(N, K);
    if (L.total > (size_t) DGTM_FE_NOALLOC_BYTES) {
        set_error(DGTM_EINVAL,
                  "N=%d, K=%d need %zu bytes of scratch, more than the %u bytes "
                  "dgtm_fe_forward_noalloc holds; use dgtm_fe_forward with a workspace",
                  N, K, L.total, (unsigned) DGTM_FE_NOALLOC_BYTES);
        return DGTM_EINVAL;
    }
    void *base_ptr = nullptr;
    int r = scratch_on_current_device(&base_ptr);
    if (r != DGTM_OK)
        return r;
    char *ws = static_cast<char *>(base_ptr);
    // Nothing below relies on the scratch starting at zero: every slot is
    // written by one kernel before the next reads it, so the contents a
    // previous call left behind never leak into this one.
    double *tt = reinterpret_cast<double *>(ws + L.tt);
    double *yy = reinterpret_cast<double *>(ws + L.yy);
    double2 *colstat = reinterpret_cast<double2 *>(ws + L.colstat);
    double *part = reinterpret_cast<double *>(ws + L.part);
    double *S = reinterpret_cast<double *>(ws + L.scal);
    cudaStream_t s = (cudaStream_t) stream;
    if ((r = launch_norms_f32(T, N, D, tt, s)) != DGTM_OK ||
        (r = launch_norms_f32(Y, K, D, yy, s)) != DGTM_OK)
        return r;
    Pass1Args<float> a{T, Y, tt, yy, N, D, K, beta / 2.0, beta / (2.0 * temp), 1, colstat, part};
    if ((r = launch_pass1_simt<float>(a, s)) != DGTM_OK)
        return r;
    if ((r = launch_sum_pairs(part, L.nblk, S, s)) != DGTM_OK)
        return r;
    const double base = N * ((D / 2.0) * log(beta / (2.0 * M_PI)) - log((double) K));
    noalloc_value_kernel<<<1, 1, 0, s>>>(S, base, temp, F);
    DGTM_CUDA_TRY(cudaGetLastError());
    return DGTM_OK;
}
