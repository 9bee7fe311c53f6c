// kernels.cuh -- argument blocks and launchers shared by the translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace dgtm {

// ---- CUDA-core (FP64 / FP32) forms -------------------------------------------
template <typename F>
struct Pass1Args {
    const F *T;          // N x D
    const F *Y;          // K x D
    const double *tt;    // N   |t_n|^2
    const double *yy;    // K   |y_k|^2
    int N, D, K;
    double c1, c2;       // beta/2, beta/(2 temp)
    int isDA;
    double2 *colstat;    // N   (dmin_n, log s_n)  (log s_n = NaN: zero column)
    double *part;        // 2 per block: sum of the llh and nfree terms
};

template <typename F>
struct Pass2Args {
    const F *T;
    const F *Y;
    const double *tt;
    const double *yy;
    const double2 *colstat;
    int N, D, K;
    double c;            // beta/(2 temp) (DA) or beta/2
    int n_per_split;
    double *Gpart;       // nsplit x K
    double *RTpart;      // nsplit x K x D
    // R_kn = 0 where d_kn > dcut: the reference forms exp(-beta d / 2) first,
    // which is 0 beyond 745.13 / (beta/2) (ref_dcut); no cut by default
    double dcut = 1e300;
};

// The distance beyond which the reference's responsibility is exactly 0:
// exp(-beta d / 2) underflows in FP64 (comm/mpicomm.c:326-336 scales D by
// -beta/2 and exponentiates before tempering and normalising).
inline double ref_dcut(double beta) { return 745.1332191019412 / (0.5 * beta); }

template <typename F> int launch_pass1_simt(const Pass1Args<F> &a, cudaStream_t s);
// own = true: statistics indexed by the owner rows (see estep_simt.cu).
template <typename F>
int launch_pass2_simt(const Pass2Args<F> &a, int nsplit, cudaStream_t s, bool own = false);
int pass1_simt_blocks(int N);
int pass2_simt_ktiles(int K);
// M = R^T X (N x L, L <= 8) and explicit R blocks, FP64, from the column
// statistics.  With Y2 (and its |y|^2 in yy2) every R_kn is multiplied by the
// squared distance of t_n to the centre k of Y2 (the reference's R o D).
int launch_map(const double *T, const double *Y, const double *tt, const double *yy,
               const double2 *colstat, int N, int D, int K, double c, const double *X, int L,
               double *M, cudaStream_t s, const double *Y2 = nullptr,
               const double *yy2 = nullptr);
int launch_r_block(const double *T, const double *Y, const double *tt, const double *yy,
                   const double2 *colstat, int D, int K, double c, int k0, int nk, int n0, int nn,
                   double *R, cudaStream_t s, const double *Y2 = nullptr,
                   const double *yy2 = nullptr, double dcut = 1e300);

// ---- M-step (FP64, all forms) ---------------------------------------------------
// Sum nsplit slices in a fixed order: G[k] = sum_s Gpart[s][k], RT = sum_s RTpart[s].
int launch_reduce_slices(const double *Gpart, const double *RTpart, int nsplit, int K,
                         int D, double *G, double *RT, cudaStream_t s);
// A = FI^T diag(G) FI (M1 x M1), B = FI^T RT (M1 x D); scratch holds
// form_ab_scratch_doubles(M1, D) doubles of slice partials.
size_t form_ab_scratch_doubles(int M1, int D);
int launch_form_ab(const double *FI, const double *G, const double *RT, int K, int M1,
                   int D, double *A, double *B, double *scratch, cudaStream_t s);
// W = A^{-1} B by Cholesky (solver 0) or symmetric-eigen pseudo-inverse (solver 1).
// work: M1*M1 + M1 doubles (+ M1*M1 for solver 1).  flag[0] != 0 on failure.
// kernel launches of one launch_solve
int solve_launches(int M1, int solver);
int launch_solve(const double *A, const double *B, int M1, int D, int solver, double *W,
                 double *work, int *flag, cudaStream_t s);
// Copies of the centres that the E-step of a form reads, written by
// launch_update_y with Y (each may be null): the FP32 copy (K x D) and the
// split-BF16 pieces (two planes of Kpad x Dp: hi with -|y_hi + y_lo|^2 / 2 in
// three BF16 pieces at columns D .. D+2, then lo).
struct YCopies {
    float *Y32 = nullptr;
    uint16_t *Yb = nullptr;  // BF16 bit patterns
    int Dp = 0, Kpad = 0;
};
// Y = FI W, yy = |y|^2, bterm_k = G_k yy_k - 2 y_k.RT_k (G/RT may be null: no
// bterm), and the copies in cp.  FIp: FI as (hi, lo) FP32 pairs for the
// compensated FP32 product (FP32 and split forms), or null for FP64 FMAs.
// ticket: one device int of scratch.  scratch (scratch_doubles doubles, may be
// null): room for W as FP32 pairs when W is too large for shared memory, so
// that the compensated product does not convert it per centre; *nlaunch
// receives the kernels launched.
int launch_update_y(const double *FI, const float2 *FIp, const double *W, const double *G,
                    const double *RT, int K, int M1, int D, double *Y, double *yy,
                    double *bterm, const YCopies &cp, int *ticket, double *scratch,
                    size_t scratch_doubles, int *nlaunch, cudaStream_t s);
// dst[i] = src[i] as an unevaluated sum of two FP32 (hi, lo).
int launch_to_pairs(const double *src, size_t n, float2 *dst, cudaStream_t s);
// AUTO cooling (ctemp.cu).  A plan fixes the batch of centres (kb), the chunk
// of points (nn), the arithmetic (FP32 for the FP32 and split forms) and the
// scratch bytes one batch needs, within a budget of scratch bytes.
struct CtempPlan {
    int kb = 1, nn = 1;
    bool f32 = false, eig_in_smem = true;
    size_t scratch_bytes = 0;
};
CtempPlan ctemp_plan(int N, int D, int K, bool f32, bool have_t32, size_t budget, int nn_max);
// For centres k0 .. k0+kb-1: gsum = row sums of R, out[2 i + w] = largest
// eigenvalue of 2 S1 (w = 0) / 2 (S1 - S2) (w = 1) below lim_scale * gg_i
// (eigenvalues at or above it count as 0).  gg_dev null: gg = gsum.  T32: the
// context's FP32 copy of T, or null (an FP32 plan then converts each chunk).
// R is the FP64 R of the R blocks, 0 where d > dcut (ref_dcut).
int launch_ctemp_batch(const CtempPlan &pl, const double *T64, const float *T32, const double *Y,
                       const double *tt, const double *yy, const double2 *colstat, int N, int D,
                       int K, double c, int k0, int kb, const double *gg_dev, double lim_scale,
                       void *scratch, double *gsum_dev, double *out_dev, double dcut,
                       bool scale_r, cudaStream_t s);
// Rows idx[0..n) of Y (K x D), and of yy and gg (gg may be null), packed.
int launch_gather_centres(const double *Y, const double *yy, const double *gg, const int *idx,
                          int n, int D, double *Ys, double *yys, double *ggs, cudaStream_t s);
// yy = |y|^2 for a given Y.
int launch_norms(const double *X, int rows, int D, double *out, cudaStream_t s);
// out[r] = |x_r|^2 in FP64 for an FP32 row-major matrix (rows x D).
int launch_norms_f32(const float *X, int rows, int D, double *out, cudaStream_t s);
// out[0] = sum_i v[i] (fixed order) + add; out[1] = num / out[0].
int launch_sum_ratio(const double *v, int n, double add, double num, double *out,
                     cudaStream_t s);
// out[0] = sum_i v[i] (fixed order) + add_dev[0].
int launch_sum_ratio_dev(const double *v, int n, const double *add_dev, double *out,
                         cudaStream_t s);
// Sum of the pass-1 block partials: out[0] = sum part[2b], out[1] = sum part[2b+1].
int launch_sum_pairs(const double *part, int nblocks, double *out, cudaStream_t s);
// Element-wise conversion to FP32.
int launch_to_f32(const double *src, size_t n, float *dst, cudaStream_t s);

}  // namespace dgtm
