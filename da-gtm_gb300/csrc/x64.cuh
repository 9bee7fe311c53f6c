// x64.cuh -- the exact-slice form of the FP64 E-step and responsibility pass
// for 0/1 data (estep_x64.cu): tensor-core distances from fixed-point digit
// slices of the centres, double-float exponentials, exact fixed-point sums.
#pragma once

#include <cuda_runtime.h>

namespace dgtm {

// the fixed-point grid of the centres of the current E-step: y ~ Y_int 2^-F
struct XScale {
    int F;
    int pad;
    double inv;  // 2^-F
};

struct XState;

// DGTM_ENOTSUP (and no state) unless the data are 0/1, D <= 189, K <= 60000,
// the device is sm_10x and DGTM_X64 is not "0": the caller then keeps the
// CUDA-core FP64 form.
int x64_create(XState **out, int N, int D, int K, int sms, const double *T64, cudaStream_t s);
void x64_destroy(XState *st);
// E-step: the digit slices of Y64, then pass 1: column statistics (d_ref,
// log s_n) as the CUDA-core FP64 pass writes them, and two partial sums per
// CTA of the quality terms into part (x64_pass1_blocks pairs).
int x64_estep(XState *st, const double *Y64, const double *yy, const double *tt, double c1,
              double c2, int isDA, double2 *colstat, double *part, cudaStream_t s, int *nlaunch);
int x64_pass1_blocks(const XState *st);
// Responsibility pass: G (K) and R T (K x D) in FP64, c = beta/(2 temp) or beta/2.
int x64_mstep_pass(XState *st, double c, double *G, double *RT, cudaStream_t s, int *nlaunch);
// the bounded waits' status word, fetched asynchronously and checked after a sync
int x64_fetch_status(XState *st, cudaStream_t s);
int x64_check_status(XState *st);

}  // namespace dgtm
