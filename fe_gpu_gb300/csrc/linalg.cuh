// Tall-skinny reductions (Gram and cross products), residual/score rows and
// single-block k x k kernels (Cholesky solve and inverse, small GEMM,
// sandwich accumulation, PSD fix). All reductions use a fixed summation order
// and are run-to-run deterministic.
#pragma once

#include "common.cuh"

namespace fegb {

// Strided matrix view: element (r, c) at ptr[r * rs + c * cs].
struct MatView {
    const double* ptr;
    long long rs;
    long long cs;
    int cols;
};

// out (a x b, column-major, ld = ldo) = A^T B over n rows. If gram (A == B),
// only pairs i <= j are computed and the result is mirrored to both triangles
// unless upper_only (then only the upper triangle is written).
// alpha/beta: out = alpha * A^T B + beta * out.
int crossprod(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha, double beta,
              double* out, int ldo, cudaStream_t s, Scratch& scr);

// Same result through the FP32 pipe: every FP64 value is split into an FP32
// pair (hi + lo, 48 significant bits), products are formed error-free
// (TwoProd by FMA plus the cross terms), summed with TwoSum into an FP32 pair
// per output and folded into FP64 every tile of rows. Relative error per term
// about 2^-47, against 2^-53 for FP64 products; GB300 issues FP32 at about 60x
// its FP64 rate, so cross products whose FP64 form is bound by the FP64 pipe
// (outputs at least "split_gram_pairs_per_col" times the input columns; the
// knob's default is CROSSPROD_SPLIT_PAIRS_PER_COL)
// run several times faster. The FP64 values are split while a tile is loaded;
// a value beyond the split range sends the whole product to the FP64 path.
constexpr long long CROSSPROD_SPLIT_PAIRS_PER_COL = 3;
int crossprod_split(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha,
                    double beta, double* out, int ldo, cudaStream_t s, Scratch& scr);
// crossprod_split when the output is large enough, else crossprod.
int crossprod_auto(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha,
                   double beta, double* out, int ldo, cudaStream_t s, Scratch& scr);

// Residual and score rows from the AoS block X (n x C, col 0 = y, 1..k = W):
// r_i = y_i - sum_j W_ij beta_j; if S != null, S[i][t] = r_i * X[i][score_cols[t]]
// (t < n_score); if resid != null, resid[i] = r_i. rss (device scalar) = sum r_i^2.
int residual_scores(const double* X, int C, long long n, const double* beta, int k, const int* score_cols_dev,
                    int n_score, double* S, double* resid, double* rss_dev, cudaStream_t s, Scratch& scr);

// ---- single-block k x k kernels (matrices column-major in device memory) ----

// Q_sel = Q[idx, idx] (k x k from ld=ldq), Cholesky (upper), solve for
// b_sel = b[idx], inverse. beta_out[t] = solution, Qinv (k x k). info (device):
// 0 ok, j > 0 when the leading minor j is not positive definite.
int dense_chol_solve_inv(int k, const double* Q, int ldq, const int* idx_dev, const double* b, double* beta_out,
                         double* Qinv, int* info_dev, double* work, cudaStream_t s);

// C (m x n, ldc) = alpha * op(A) op(B) + beta * C for small matrices.
int dense_gemm(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
               double beta, double* C, int ldc, cudaStream_t s);

// acc (k x k) += w * Qinv * M[idx, idx] * Qinv; M has leading dimension ldm.
int dense_sandwich_acc(int k, const double* Qinv, const double* M, int ldm, const int* idx_dev, double w, double* acc,
                       double* work, cudaStream_t s);

// acc *= scalar; mirror upper to lower; PSD fix (clamp negative eigenvalues,
// reconstruct V diag V^T); se[t] = sqrt(max(0, acc[t,t])). psd_applied (device
// int) set to 1 if an eigenvalue was clamped. do_psd = 0 skips the eigen step
// and instead symmetrizes by averaging (the CPU-path convention).
int dense_finalize_cov(int k, double* acc, double scalar, int do_psd, double* se_out, int* psd_applied, double* work,
                       cudaStream_t s);

}  // namespace fegb
