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
// partial sums of the llh / nfree terms (need_llh = false: the nfree terms
// only, half the exponentials when temp != 1).
int tc_estep(TcState *st, const double *Y64, double c1, double c2, int isDA, double2 *colstat,
             double *part, cudaStream_t s, int *nlaunch, bool need_llh = true);
int tc_pass1_blocks(const TcState *st);
// Responsibility pass (tensor cores): per-slice partial G and RT.
int tc_mstep_pass(TcState *st, const double2 *colstat, double c, cudaStream_t s, int *nlaunch);
// Fixed-order FP64 sum of the slices into G (K) and RT (K x D).
int tc_mstep_reduce(TcState *st, double *G, double *RT, cudaStream_t s, int *nlaunch);
// Device-side status (bounded waits that gave up); fetched asynchronously,
// checked after the stream synchronises.
int tc_fetch_status(TcState *st, cudaStream_t s);
int tc_check_status(TcState *st);

// The free energy's tensor-core passes over caller-owned FP32 device arrays
// (the data always in two BF16 pieces).  The layout gives byte offsets into a
// 256-byte aligned region of the caller's workspace that the passes own; the
// column statistics and the pass-1 partial sums are the caller's.
struct TcFeLayout {
    size_t Tb = 0, Yb = 0, colq = 0, RTpart = 0, status = 0, total = 0;
    int pass1_blocks = 0;
};
// DGTM_ENOTSUP when the device or D is outside the split form.
int tc_fe_layout(int N, int K, int D, int sms, TcFeLayout *L);
// The operand pieces of Y and T, then pass 1 at c1 = beta/2, c2 = beta/(2 temp)
// (DA): column statistics, the per-point statistics for passes 2 and 3, and
// per-CTA partial sums of the two per-point terms.  Clears the status word.
int tc_fe_estep(const TcFeLayout &L, void *ws, const float *Y, const float *T, int N, int K, int D,
                int sms, double c1, double c2, double2 *colstat, double *part, cudaStream_t s);
// Pass 2 and the slot sum: G = rowsum R and RT = R T (FP64) of the tempered R.
int tc_fe_stats(const TcFeLayout &L, void *ws, int N, int K, int D, int sms, double *G,
                double *RT, cudaStream_t s);
// Pass 3: C = R^T Y (N x D, FP32), C_n = sum_k R_kn y_k.
int tc_fe_rty(const TcFeLayout &L, void *ws, int N, int K, int D, int sms, float *C,
              cudaStream_t s);
// The device status word (non-zero: a bounded wait gave up).
int *tc_fe_status(const TcFeLayout &L, void *ws);

// The split form's device operands as other passes need them.
struct TcView {
    int N, D, K, Dp, npanel, Npad, Kpad, nT, ksteps;
    int binary;           // every data value is 0 or 1
    const void *Tb;       // nT x Npad x Dp BF16: data pieces, columns D..D+2 = 1
    const void *Yb;       // 2 x Kpad x Dp BF16: centre pieces, -|y|^2/2 at D..D+2 of hi
    const float4 *colq;   // Npad: (m, scale, log2 s) of the last E-step
    const double *tt;     // N: |t_n|^2
    int *status;          // bounded-wait status word
};
void tc_view(const TcState *st, TcView *v);

// The AUTO schedule's scatter as a tensor-core GEMM over pair features
// (ctemp_tc.cu).  Needs 0/1 data (binary: every pair product exact in BF16):
// for centres k, S1_k = sum_n R_kn (t_n - y_k)(t_n - y_k)^T and S2_k (R^2),
// upper triangles, written per batch of centres as the CUDA-core scatter
// writes them; then the eigen filter of ctemp.cu.  out[2 k + w] as in
// launch_ctemp_batch; gsum[k] = row sums of R.
// R_kn = 0 where d_kn > dcut (the reference's exp(-beta d / 2) underflows);
// dmin (Kpad floats): each centre's least distance to a point (FP32).
int tc_ctemp_pairs(const TcView &v, const double *Y64, const double *gg_dev, double lim_scale,
                   size_t budget, double dcut, double *gsum_dev, double *out_dev, float *dmin,
                   cudaStream_t s);

}  // namespace dgtm
