// estep_tc.cu -- split-BF16 tensor-core form (placeholder until the tcgen05
// kernels land): creation reports DGTM_ENOTSUP.
#include "common.cuh"
#include "tc.cuh"

namespace dgtm {

struct TcState {
    int dummy;
};

int tc_create(TcState **out, int, int, int, int, const double *, const double *, cudaStream_t)
{
    *out = nullptr;
    set_error(DGTM_ENOTSUP, "the split-BF16 form is not built yet");
    return DGTM_ENOTSUP;
}
void tc_destroy(TcState *) {}
int tc_prepare_y(TcState *, const double *, cudaStream_t) { return DGTM_ENOTSUP; }
int tc_estep(TcState *, const double *, double, double, int, double2 *, double *, cudaStream_t,
             int *)
{
    return DGTM_ENOTSUP;
}
int tc_pass1_blocks(const TcState *) { return 1; }
int tc_mstep_pass(TcState *, const double2 *, double, cudaStream_t, int *) { return DGTM_ENOTSUP; }
int tc_mstep_reduce(TcState *, double *, double *, cudaStream_t, int *) { return DGTM_ENOTSUP; }
int tc_fetch_status(TcState *, cudaStream_t) { return DGTM_OK; }
int tc_check_status(TcState *) { return DGTM_OK; }

}  // namespace dgtm
