// Device routines shared by the dense kernels of linalg.cu and the batched
// estimator (batch_est.cu): double-single products, and single-block k x k
// Cholesky solve and inverse, Jacobi eigensolver and covariance finalize (each
// run by one block of DN_THREADS threads).
#pragma once

#include "common.cuh"

namespace fegb {

constexpr int DN_THREADS = 256;

// acc_hi/acc_lo (+)= x * y in double-single arithmetic:
// (xh + xl)(yh + yl) = ph + pe + cross with ph + pe exact (TwoProd by FMA);
// TwoSum of the running high part and ph, its rounding error into the low part.
// (The _rn intrinsics are never contracted into FMAs, which TwoSum relies on.)
__device__ __forceinline__ void ds_fma(float2 x, float2 y, float& sh, float& sl) {
    const float ph = __fmul_rn(x.x, y.x);
    const float pe = fmaf(x.x, y.x, -ph);
    const float cr = fmaf(x.x, y.y, x.y * y.x);
    const float s1 = __fadd_rn(sh, ph);
    const float bb = __fsub_rn(s1, sh);
    const float err = __fadd_rn(__fsub_rn(sh, __fsub_rn(s1, bb)), __fsub_rn(ph, bb));
    sh = s1;
    sl += err + (pe + cr);
}

// One block of DN_THREADS threads: Q_sel = Q[idx, idx] (or the leading k x k
// block), upper Cholesky factor, solve for b_sel and the inverse. info: 0 ok,
// j > 0 when the leading minor j is not positive definite. work: 2 k^2.
__device__ inline void chol_solve_inv_block(int k, const double* __restrict__ Q, int ldq, const int* __restrict__ idx,
                                     const double* __restrict__ b, double* __restrict__ beta,
                                     double* __restrict__ Qinv, int* __restrict__ info, double* __restrict__ work) {
    double* U = work;
    double* Ui = work + (size_t)k * k;
    __shared__ int s_info;
    __shared__ double s_d;
    const int t = threadIdx.x;
    for (int e = t; e < k * k; e += DN_THREADS) {
        int i = e % k, j = e / k;
        int qi = idx ? idx[i] : i, qj = idx ? idx[j] : j;
        U[e] = Q[qi + (long long)qj * ldq];
    }
    if (t == 0) s_info = 0;
    __syncthreads();
    for (int j = 0; j < k; ++j) {
        for (int c = j + t; c < k; c += DN_THREADS) {
            double v = U[j + c * k];
            for (int p = 0; p < j; ++p) v -= U[p + j * k] * U[p + c * k];
            U[j + c * k] = v;
        }
        __syncthreads();
        if (t == 0) {
            double d = U[j + j * k];
            if (!(d > 0.0)) {
                s_info = j + 1;
            } else {
                s_d = sqrt(d);
                U[j + j * k] = s_d;
            }
        }
        __syncthreads();
        if (s_info) break;
        for (int c = j + 1 + t; c < k; c += DN_THREADS) U[j + c * k] /= s_d;
        __syncthreads();
    }
    if (s_info) {
        if (t == 0) *info = s_info;
        return;
    }
    // U^{-1}: column j by thread j (back substitution on the upper factor)
    for (int j = t; j < k; j += DN_THREADS) {
        for (int i = 0; i < k; ++i) Ui[i + j * k] = 0.0;
        Ui[j + j * k] = 1.0 / U[j + j * k];
        for (int i = j - 1; i >= 0; --i) {
            double s = 0.0;
            for (int p = i + 1; p <= j; ++p) s += U[i + p * k] * Ui[p + j * k];
            Ui[i + j * k] = -s / U[i + i * k];
        }
    }
    __syncthreads();
    // beta = U^{-1} U^{-T} b_sel, Qinv = U^{-1} U^{-T}
    for (int e = t; e < k * k; e += DN_THREADS) {
        int i = e % k, j = e / k;
        if (i > j) continue;
        double s = 0.0;
        for (int p = j; p < k; ++p) s += Ui[i + p * k] * Ui[j + p * k];
        Qinv[i + j * k] = s;
        Qinv[j + i * k] = s;
    }
    __syncthreads();
    if (t == 0) {
        // forward then backward substitution (dpotrs order)
        for (int i = 0; i < k; ++i) {
            double v = b[idx ? idx[i] : i];
            for (int p = 0; p < i; ++p) v -= U[p + i * k] * beta[p];
            beta[i] = v / U[i + i * k];
        }
        for (int i = k - 1; i >= 0; --i) {
            double v = beta[i];
            for (int p = i + 1; p < k; ++p) v -= U[i + p * k] * beta[p];
            beta[i] = v / U[i + i * k];
        }
        *info = 0;
    }
}

// One block: whether the symmetric k x k matrix A (upper triangle read) has an
// upper Cholesky factor with positive pivots, i.e. is positive definite; the
// factor is formed in U (k^2 doubles). The answer is the same on every thread.
__device__ inline bool block_cholesky_ok(int k, const double* __restrict__ A, double* __restrict__ U) {
    __shared__ int s_fail;
    __shared__ double s_d;
    const int t = threadIdx.x;
    for (int e = t; e < k * k; e += DN_THREADS) U[e] = A[e];
    if (t == 0) s_fail = 0;
    __syncthreads();
    for (int j = 0; j < k; ++j) {
        for (int c = j + t; c < k; c += DN_THREADS) {
            double v = U[j + c * k];
            for (int p = 0; p < j; ++p) v -= U[p + j * k] * U[p + c * k];
            U[j + c * k] = v;
        }
        __syncthreads();
        if (t == 0) {
            const double d = U[j + j * k];
            if (!(d > 0.0))
                s_fail = 1;
            else
                s_d = sqrt(d);
        }
        __syncthreads();
        if (s_fail) break;
        for (int c = j + 1 + t; c < k; c += DN_THREADS) U[j + c * k] /= s_d;
        __syncthreads();
    }
    const bool ok = s_fail == 0;
    __syncthreads();
    return ok;
}

// Parallel cyclic Jacobi on a k x k symmetric matrix A (in place; global
// memory), eigenvectors accumulated in V; the round-robin pairing makes all
// rotations of one round touch disjoint rows/columns.
__device__ inline void block_jacobi(int k, double* A, double* V) {
    __shared__ int sp[DN_THREADS], sq[DN_THREADS];
    __shared__ double sc[DN_THREADS], ss[DN_THREADS];
    __shared__ double s_off, s_tot;
    __shared__ double red[DN_THREADS / 32];
    const int t = threadIdx.x;
    for (int e = t; e < k * k; e += DN_THREADS) V[e] = (e % k == e / k) ? 1.0 : 0.0;
    const int kk = (k % 2) ? k + 1 : k;
    const int m = kk / 2;
    __syncthreads();
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int e = t; e < k * k; e += DN_THREADS) {
            double a = A[e] * A[e];
            tot += a;
            if (e % k != e / k) off += a;
        }
        for (int pass = 0; pass < 2; ++pass) {
            double v = pass == 0 ? off : tot;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if ((t & 31) == 0) red[t >> 5] = v;
            __syncthreads();
            if (t == 0) {
                double s = 0.0;
                for (int w = 0; w < DN_THREADS / 32; ++w) s += red[w];
                if (pass == 0)
                    s_off = s;
                else
                    s_tot = s;
            }
            __syncthreads();
        }
        if (s_off == 0.0 || s_off <= 1e-30 * (s_tot > 0.0 ? s_tot : 1.0)) break;
        for (int round = 0; round < kk - 1; ++round) {
            for (int i = t; i < m; i += DN_THREADS) {
                int p, q;
                if (i == 0) {
                    p = round;
                    q = kk - 1;
                } else {
                    p = (round + i) % (kk - 1);
                    q = (round - i + (kk - 1)) % (kk - 1);
                }
                if (p > q) {
                    int tmp = p;
                    p = q;
                    q = tmp;
                }
                double c = 1.0, s = 0.0;
                if (q < k) {
                    double apq = A[p + q * k];
                    if (apq != 0.0) {
                        double app = A[p + p * k], aqq = A[q + q * k];
                        double theta = (aqq - app) / (2.0 * apq);
                        double tt = (theta >= 0.0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                        c = 1.0 / sqrt(tt * tt + 1.0);
                        s = tt * c;
                    }
                }
                sp[i] = p;
                sq[i] = q;
                sc[i] = c;
                ss[i] = s;
            }
            __syncthreads();
            // columns: A <- A J, V <- V J
            for (int e = t; e < m * k; e += DN_THREADS) {
                int i = e / k, r = e % k;
                int p = sp[i], q = sq[i];
                if (q >= k || ss[i] == 0.0) continue;
                double c = sc[i], s = ss[i];
                double arp = A[r + p * k], arq = A[r + q * k];
                A[r + p * k] = c * arp - s * arq;
                A[r + q * k] = s * arp + c * arq;
                double vrp = V[r + p * k], vrq = V[r + q * k];
                V[r + p * k] = c * vrp - s * vrq;
                V[r + q * k] = s * vrp + c * vrq;
            }
            __syncthreads();
            // rows: A <- J^T A
            for (int e = t; e < m * k; e += DN_THREADS) {
                int i = e / k, col = e % k;
                int p = sp[i], q = sq[i];
                if (q >= k || ss[i] == 0.0) continue;
                double c = sc[i], s = ss[i];
                double apc = A[p + col * k], aqc = A[q + col * k];
                A[p + col * k] = c * apc - s * aqc;
                A[q + col * k] = s * apc + c * aqc;
            }
            __syncthreads();
        }
    }
}

// One block: acc *= scalar, then the PSD fix (mirror, Jacobi, clamp
// negative eigenvalues, rebuild) or the CPU path's symmetrisation; se[i] =
// sqrt(max(0, acc[i, i])). work: 2 k^2.
__device__ inline void finalize_cov_block(int k, double* __restrict__ acc, double scalar, int do_psd,
                                   double* __restrict__ se, int* __restrict__ psd_applied,
                                   double* __restrict__ work) {
    const int t = threadIdx.x;
    double* A = work;
    double* V = work + (size_t)k * k;
    __shared__ int s_applied;
    if (t == 0) s_applied = 0;
    for (int e = t; e < k * k; e += DN_THREADS) acc[e] *= scalar;
    __syncthreads();
    if (!do_psd) {
        // 0.5 (A + A^T), as the CPU path does (fe_pipeline.f90:476)
        for (int e = t; e < k * k; e += DN_THREADS) {
            int i = e % k, j = e / k;
            A[e] = 0.5 * (acc[i + j * k] + acc[j + i * k]);
        }
        __syncthreads();
        for (int e = t; e < k * k; e += DN_THREADS) acc[e] = A[e];
        __syncthreads();
        for (int i = t; i < k; i += DN_THREADS) se[i] = sqrt(fmax(0.0, acc[i + i * k]));
        if (t == 0) *psd_applied = 0;
        return;
    }
    // mirror the upper triangle to the lower (fe_pipeline.f90:1366, 1802-1811)
    for (int e = t; e < k * k; e += DN_THREADS) {
        int i = e % k, j = e / k;
        if (i > j) acc[e] = acc[j + i * k];
    }
    __syncthreads();
    for (int e = t; e < k * k; e += DN_THREADS) A[e] = acc[e];
    __syncthreads();
    // A positive definite matrix has no negative eigenvalue to clamp, and its
    // reconstruction V diag(lambda) V' is the matrix itself up to rounding:
    // the eigensolver (about 24 ms at k = 90) runs only when the Cholesky
    // factorisation fails
    if (block_cholesky_ok(k, A, V)) {
        for (int i = t; i < k; i += DN_THREADS) se[i] = sqrt(fmax(0.0, acc[i + i * k]));
        if (t == 0) *psd_applied = 0;
        return;
    }
    block_jacobi(k, A, V);
    __syncthreads();
    // lambda_j = A[j,j]; scale eigenvector columns by sqrt(max(lambda,0))
    for (int e = t; e < k * k; e += DN_THREADS) {
        int j = e / k;
        double lam = A[j + j * k];
        if (lam < 0.0) {
            s_applied = 1;
            lam = 0.0;
        }
        V[e] *= lam > 0.0 ? sqrt(lam) : 0.0;
    }
    __syncthreads();
    for (int e = t; e < k * k; e += DN_THREADS) {
        int i = e % k, j = e / k;
        double s = 0.0;
        for (int p = 0; p < k; ++p) s += V[i + p * k] * V[j + p * k];
        acc[e] = s;
    }
    __syncthreads();
    for (int i = t; i < k; i += DN_THREADS) se[i] = sqrt(fmax(0.0, acc[i + i * k]));
    if (t == 0) *psd_applied = s_applied;
}

}  // namespace fegb
