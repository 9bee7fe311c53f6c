// tc.cuh -- the split-BF16 tensor-core form (tcgen05 + TMA + TMEM, sm_103a).
#pragma once

#include <cuda_runtime.h>

namespace dgtm {

struct TcState;

// Build the device operands of the data: T in BF16 (exact for 0/1 data; a
// second BF16 piece holds the remainder otherwise), |t_n|^2 and the TMA maps.
int tc_create(TcState **out, int N, int D, int K, int sms, const double *T64, const double *tt,
              cudaStream_t s);
void tc_destroy(TcState *st);
// Split the FP64 centres into BF16 pieces (with the folded -|y|^2/2 column).
int tc_prepare_y(TcState *st, const double *Y64, cudaStream_t s);
// Where the M-step writes the BF16 pieces and the FP32 copy of new centres.
struct YCopies;
void tc_y_copies(TcState *st, YCopies *cp);
// E-step: column statistics (exact-minimum shift, log s_n) and per-block
// partial sums of the llh / nfree terms.
int tc_estep(TcState *st, const double *Y64, double c1, double c2, int isDA, double2 *colstat,
             double *part, cudaStream_t s, int *nlaunch);
int tc_pass1_blocks(const TcState *st);
// Responsibility pass (tensor cores): per-slice partial G and RT.
int tc_mstep_pass(TcState *st, const double2 *colstat, double c, cudaStream_t s, int *nlaunch);
// Fixed-order FP64 sum of the slices into G (K) and RT (K x D).
int tc_mstep_reduce(TcState *st, double *G, double *RT, cudaStream_t s, int *nlaunch);
// Device-side status (bounded waits that gave up); fetched asynchronously,
// checked after the stream synchronises.
int tc_fetch_status(TcState *st, cudaStream_t s);
int tc_check_status(TcState *st);

}  // namespace dgtm
