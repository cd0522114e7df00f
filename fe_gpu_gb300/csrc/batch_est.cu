// Batched estimation of stacked specifications (fegb_estimate_batch).
//
// After a column class's shared within-transform every specification still
// needs its own normal equations, solve, residuals, scores and clustered SEs
// (the reference path: fe_pipeline.f90:947-1420). Fitting them one by one
// costs a row sort per specification and per cluster subset and a few dozen
// launches and host round trips each. Here the whole class is estimated with
// a fixed number of launches:
//
//   1. Gram products of every specification: a persistent kernel drains a
//      device work queue of (specification, row range) items; each item's
//      double-single partial Gram goes to its own slot, and the slots of a
//      specification are folded in item order (deterministic).
//   2. One block per specification: 2SLS normal equations, column filter,
//      Cholesky solve and inverse (the single-fit routines of linalg_dev.cuh).
//   3. Residuals and score columns, item by item (RSS per item, folded).
//   4. Per cluster subset (bit mask over each specification's cluster
//      dimensions): one 64-bit key sort of all the class's rows (specification
//      index in the high bits, the specification's mixed-radix cluster key in
//      the low bits), cluster score sums, and the meats as Gram products of
//      the cluster sums through the same work queue; one block per
//      specification accumulates the CGM sandwich with its sign.
//   5. One block per specification: scalar, PSD fix, SEs; dof and R^2 on the
//      host from a few copied scalars.
#include "batch_est.cuh"
#include "linalg_dev.cuh"
#include "prep.cuh"

#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace fegb {

namespace {

using BeClock = std::chrono::steady_clock;
double be_seconds_since(BeClock::time_point t0) {
    return std::chrono::duration<double>(BeClock::now() - t0).count();
}

constexpr int BE_THREADS = 256;
constexpr int BE_ITEM_ROWS = 16384;  // rows (or clusters) per work item
// rows per shared-memory tile of the Gram: about 4096 values (32 KB as FP64),
// a multiple of 32 between 32 and 256
__host__ __device__ inline int be_tile_rows(int Cw) {
    int tr = 4096 / (Cw > 0 ? Cw : 1);
    tr = tr > 256 ? 256 : tr;
    tr = tr / 32 * 32;
    return tr < 32 ? 32 : tr;
}
// output pairs per thread: 1 up to 22 columns (253 pairs), else 2, 4 or 9
// (64 columns: 2080 pairs)
inline int be_ppt(int Cw) {
    const int P = Cw * (Cw + 1) / 2;
    const int npt = (P + 255) / 256;
    return npt <= 1 ? 1 : npt <= 2 ? 2 : npt <= 4 ? 4 : 9;
}

struct BeItem {
    int spec;
    long long r0, r1;
};

// Per-specification state on the device.
struct BeSpecDev {
    long long row0, n;
    int k, l, cs;      // cs = 1 + k + l columns used
    // set by the solve kernel
    int use_iv, na, kk, info;
    int za[BE_MAX_COLS];    // X columns (1-based into [y W Z]) of Z_aug = [exogenous W, selected Z]
    int kept[BE_MAX_COLS];  // kept regressors (0-based)
    int endog_mask[2];      // bit j: regressor j (0-based) endogenous
    int sel[BE_MAX_COLS];   // selected instruments (1-based into Z)
    int n_sel;
    double tss_within;
};

// Columns of the class: column 0 = y, column c >= 1 = W block column c - 1.
struct ColMajorX {
    const double* y;
    const double* W;
    long long ld;
    __device__ __forceinline__ double operator()(long long r, int c) const {
        return c == 0 ? y[r] : W[(long long)(c - 1) * ld + r];
    }
};
// Row-major rows of width ld (cluster score sums).
struct RowMajor {
    const double* S;
    int ld;
    __device__ __forceinline__ double operator()(long long r, int c) const { return S[r * ld + c]; }
};

// Gram of the item's rows over the specification's first `width` columns,
// pairs p = j (j + 1) / 2 + i (i <= j) over Cw columns: partials[item][p].
// Items are taken from a device counter (*queue), so the persistent blocks
// stay busy whatever the items' sizes; the arithmetic of an item does not
// depend on the block that takes it. SPLIT: double-single products on the
// FP32 pipe (a value outside the split range sets *bad); else FP64.
template <class Acc, bool SPLIT, int BE_PPT>
__global__ void __launch_bounds__(BE_THREADS)
    be_gram_kernel(Acc X, const BeItem* __restrict__ items, int n_items, const int* __restrict__ width_of,
                   int Cw, double* __restrict__ partials, int* __restrict__ queue, int* __restrict__ bad) {
    extern __shared__ __align__(16) unsigned char be_smem[];
    __shared__ int s_item;
    __shared__ double s_fold[BE_THREADS];
    const int t = threadIdx.x;
    const int P = Cw * (Cw + 1) / 2;
    // pair assignment: P <= BE_THREADS: thread = (pair, row phase); else pairs t + j * BE_THREADS
    const bool one = P <= BE_THREADS;
    const int phases = one ? BE_THREADS / P : 1;
    const int npt = one ? 1 : (P + BE_THREADS - 1) / BE_THREADS;
    int pi[BE_PPT], pj[BE_PPT];
    bool pv[BE_PPT];
    const int phase = one ? t / P : 0;
#pragma unroll
    for (int q = 0; q < BE_PPT; ++q) {
        const int p = one ? t % P : t + q * BE_THREADS;
        pv[q] = q < npt && p < P && phase < phases;
        int j = 0;
        while ((j + 1) * (j + 2) / 2 <= (pv[q] ? p : 0)) ++j;
        pj[q] = j;
        pi[q] = (pv[q] ? p : 0) - j * (j + 1) / 2;
    }
    bool oor = false;
    while (true) {
        if (t == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const BeItem item = items[it];
        const int width = min(Cw, width_of[item.spec]);
        double acc[BE_PPT];
#pragma unroll
        for (int q = 0; q < BE_PPT; ++q) acc[q] = 0.0;
        const int TR = be_tile_rows(Cw);
        for (long long r0 = item.r0; r0 < item.r1; r0 += TR) {
            const int rows = (int)min((long long)TR, item.r1 - r0);
            __syncthreads();  // the previous tile is consumed
            for (int e = t; e < TR * Cw; e += BE_THREADS) {
                const int r = e % TR, c = e / TR;  // consecutive threads walk rows of a column
                const double v = (r < rows && c < width) ? X(r0 + r, c) : 0.0;
                if (SPLIT)
                    reinterpret_cast<float2*>(be_smem)[r * Cw + c] = split_f64<56>(v, oor);
                else
                    reinterpret_cast<double*>(be_smem)[r * Cw + c] = v;
            }
            __syncthreads();
            if (SPLIT) {
                // two rows per step into two sets of sums (independent chains)
                const float2* x = reinterpret_cast<const float2*>(be_smem);
                float sh[BE_PPT], sl[BE_PPT], sh2[BE_PPT], sl2[BE_PPT];
#pragma unroll
                for (int q = 0; q < BE_PPT; ++q) sh[q] = sl[q] = sh2[q] = sl2[q] = 0.f;
                int r = phase;
                for (; r + phases < rows; r += 2 * phases) {
                    const int r2 = r + phases;
#pragma unroll
                    for (int q = 0; q < BE_PPT; ++q)
                        if (pv[q]) {
                            ds_fma(x[r * Cw + pi[q]], x[r * Cw + pj[q]], sh[q], sl[q]);
                            ds_fma(x[r2 * Cw + pi[q]], x[r2 * Cw + pj[q]], sh2[q], sl2[q]);
                        }
                }
                if (r < rows) {
#pragma unroll
                    for (int q = 0; q < BE_PPT; ++q)
                        if (pv[q]) ds_fma(x[r * Cw + pi[q]], x[r * Cw + pj[q]], sh[q], sl[q]);
                }
#pragma unroll
                for (int q = 0; q < BE_PPT; ++q) acc[q] += ((double)sh[q] + (double)sl[q]) + ((double)sh2[q] + (double)sl2[q]);
            } else {
                const double* x = reinterpret_cast<const double*>(be_smem);
                for (int r = phase; r < rows; r += phases) {
#pragma unroll
                    for (int q = 0; q < BE_PPT; ++q)
                        if (pv[q]) acc[q] = fma(x[r * Cw + pi[q]], x[r * Cw + pj[q]], acc[q]);
                }
            }
        }
        double* out = partials + (long long)it * P;
        if (one) {
            s_fold[t] = pv[0] ? acc[0] : 0.0;
            __syncthreads();
            if (t < P) {
                double v = 0.0;
                for (int ph = 0; ph < phases; ++ph) v += s_fold[ph * P + t];
                out[t] = v;
            }
        } else {
#pragma unroll
            for (int q = 0; q < BE_PPT; ++q)
                if (pv[q]) out[t + q * BE_THREADS] = acc[q];
        }
        __syncthreads();  // s_item and s_fold are reused
    }
    if (SPLIT && __any_sync(0xffffffffu, oor) && (t & 31) == 0) atomicOr(bad, 1);
}

// The double-single Gram in 4 x 4 output blocks: thread t takes block
// q = t % NB (bi <= bj over the class's Cw columns padded to Cw4) and row phase
// t / NB, so each tile row costs it 4 + 4 shared-memory reads (two 32-byte
// runs) for 16 products instead of two reads per product. Per item the
// blocks' sums are folded over the phases in phase order. Same items, queue
// and partial layout as be_gram_kernel.
template <class Acc>
__global__ void __launch_bounds__(BE_THREADS)
    be_gram_blocked_kernel(Acc X, const BeItem* __restrict__ items, int n_items, const int* __restrict__ width_of,
                           int Cw, double* __restrict__ partials, int* __restrict__ queue, int* __restrict__ bad) {
    extern __shared__ __align__(16) unsigned char be_smem[];
    __shared__ int s_item;
    __shared__ double s_fold[BE_THREADS][17];  // a thread's 16 sums (odd stride: no bank conflicts)
    const int t = threadIdx.x;
    const int Cw4 = (Cw + 3) / 4 * 4;
    const int nbk = Cw4 / 4;
    const int NB = nbk * (nbk + 1) / 2;
    const int phases = BE_THREADS / NB;
    const int q = t % NB, phase = t / NB;
    const bool active = phase < phases;
    int bi = 0, bj = 0;
    {
        int j = 0;
        while ((j + 1) * (j + 2) / 2 <= q) ++j;
        bj = j;
        bi = q - j * (j + 1) / 2;
    }
    const int P = Cw * (Cw + 1) / 2;
    bool oor = false;
    float2* tile = reinterpret_cast<float2*>(be_smem);  // [TR][Cw4]
    while (true) {
        if (t == 0) s_item = atomicAdd(queue, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const BeItem item = items[it];
        const int width = min(Cw, width_of[item.spec]);
        double acc[16];
#pragma unroll
        for (int e = 0; e < 16; ++e) acc[e] = 0.0;
        const int TR = be_tile_rows(Cw);
        for (long long r0 = item.r0; r0 < item.r1; r0 += TR) {
            const int rows = (int)min((long long)TR, item.r1 - r0);
            __syncthreads();  // the previous tile is consumed
            for (int e = t; e < TR * Cw4; e += BE_THREADS) {
                const int r = e % TR, c = e / TR;  // consecutive threads walk rows of a column
                const double v = (r < rows && c < width) ? X(r0 + r, c) : 0.0;
                tile[r * Cw4 + c] = split_f64<56>(v, oor);
            }
            __syncthreads();
            if (active) {
                float sh[16], sl[16];
#pragma unroll
                for (int e = 0; e < 16; ++e) sh[e] = sl[e] = 0.f;
                const float4* row = reinterpret_cast<const float4*>(tile);
                for (int r = phase; r < rows; r += phases) {
                    const float4 i01 = row[(r * Cw4 + 4 * bi) / 2], i23 = row[(r * Cw4 + 4 * bi) / 2 + 1];
                    const float4 j01 = row[(r * Cw4 + 4 * bj) / 2], j23 = row[(r * Cw4 + 4 * bj) / 2 + 1];
                    const float2 xi[4] = {make_float2(i01.x, i01.y), make_float2(i01.z, i01.w),
                                          make_float2(i23.x, i23.y), make_float2(i23.z, i23.w)};
                    const float2 xj[4] = {make_float2(j01.x, j01.y), make_float2(j01.z, j01.w),
                                          make_float2(j23.x, j23.y), make_float2(j23.z, j23.w)};
#pragma unroll
                    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
                        for (int jj = 0; jj < 4; ++jj) ds_fma(xi[ii], xj[jj], sh[ii * 4 + jj], sl[ii * 4 + jj]);
                }
#pragma unroll
                for (int e = 0; e < 16; ++e) acc[e] += (double)sh[e] + (double)sl[e];
            }
        }
#pragma unroll
        for (int e = 0; e < 16; ++e) s_fold[t][e] = active ? acc[e] : 0.0;
        __syncthreads();
        double* out = partials + (long long)it * P;
        for (int w = t; w < NB * 16; w += BE_THREADS) {
            const int qq = w / 16, e = w % 16;
            int jb = 0;
            while ((jb + 1) * (jb + 2) / 2 <= qq) ++jb;
            const int ib = qq - jb * (jb + 1) / 2;
            const int i = 4 * ib + e / 4, j = 4 * jb + e % 4;
            if (i <= j && j < Cw) {
                double v = 0.0;
                for (int ph = 0; ph < phases; ++ph) v += s_fold[ph * NB + qq][e];
                out[j * (j + 1) / 2 + i] = v;
            }
        }
        __syncthreads();  // s_item and s_fold are reused
    }
    if (__any_sync(0xffffffffu, oor) && (t & 31) == 0) atomicOr(bad, 1);
}

// out[s][p] = sum over the items of specification s (in order) of partials[item][p]
__global__ void be_fold_kernel(const double* __restrict__ partials, const int* __restrict__ item0,
                               const int* __restrict__ item1, int P, double* __restrict__ out) {
    const int s = blockIdx.x;
    for (int p = threadIdx.x; p < P; p += blockDim.x) {
        double v = 0.0;
        for (int it = item0[s]; it < item1[s]; ++it) v += partials[(long long)it * P + p];
        out[(long long)s * P + p] = v;
    }
}

__device__ __forceinline__ double gram_at(const double* G, int i, int j) {
    if (i > j) {
        const int tmp = i;
        i = j;
        j = tmp;
    }
    return G[j * (j + 1) / 2 + i];
}

// Per-specification scratch (doubles): Q, Qzz, Qzx, Pi, Qinv_zz, Qinv, work (2), vectors.
__host__ __device__ inline long long be_scratch_per_spec(int Kb) { return 10LL * Kb * Kb + 8LL * Kb; }

// One block per specification: build_iv_normal_equations
// (fe_pipeline.f90:947-1032), solve_with_column_filter (fe_pipeline.f90:
// 1034-1107), as the single-fit path computes them.
__global__ void __launch_bounds__(DN_THREADS)
    be_solve_kernel(BeSpecDev* __restrict__ specs, const double* __restrict__ gram, int Cw, int Kb,
                    double* __restrict__ scratch, double* __restrict__ beta_full, double* __restrict__ Qinv_out,
                    double* __restrict__ Pi_out) {
    BeSpecDev& S = specs[blockIdx.x];
    const double* G = gram + (long long)blockIdx.x * (Cw * (Cw + 1) / 2);
    double* sc = scratch + (long long)blockIdx.x * be_scratch_per_spec(Kb);
    double* Q = sc;
    double* Qzz = Q + Kb * Kb;
    double* Qzx = Qzz + Kb * Kb;
    double* Pi = Pi_out + (long long)blockIdx.x * Kb * Kb;
    double* Qiz = Qzx + Kb * Kb;
    double* Qinv = Qinv_out + (long long)blockIdx.x * Kb * Kb;
    double* work = Qiz + Kb * Kb;  // 2 Kb^2
    double* b = work + 2 * Kb * Kb;
    double* zy = b + Kb;
    double* rhs = zy + Kb;
    double* bsel = rhs + Kb;
    double* beta = beta_full + (long long)blockIdx.x * Kb;
    __shared__ int s_info;
    __shared__ int s_kept[BE_MAX_COLS];
    __shared__ int s_kk;
    const int t = threadIdx.x;
    const int k = S.k, l = S.l;
    for (int j = t; j < Kb; j += DN_THREADS) beta[j] = 0.0;
    if (t == 0) {
        S.tss_within = G[0];
        S.info = 0;
        S.kk = 0;
        // endogenous columns and instruments (fe_pipeline.f90:672-746)
        int n_endog = 0;
        for (int j = 0; j < k; ++j) n_endog += (S.endog_mask[j >> 5] >> (j & 31)) & 1;
        int nsel = S.n_sel;
        int na = 0;
        S.use_iv = n_endog > 0 && l > 0 && nsel >= n_endog;
        if (S.use_iv) {
            for (int j = 0; j < k; ++j)
                if (!((S.endog_mask[j >> 5] >> (j & 31)) & 1)) S.za[na++] = 1 + j;
            for (int q = 0; q < nsel; ++q) S.za[na++] = 1 + k + (S.sel[q] - 1);
        }
        S.na = S.use_iv ? na : 0;
    }
    __syncthreads();
    const int na = S.na;
    // Q = W'W, b = W'y
    for (int e = t; e < k * k; e += DN_THREADS) Q[(e % k) + (e / k) * k] = gram_at(G, 1 + e % k, 1 + e / k);
    for (int j = t; j < k; j += DN_THREADS) b[j] = gram_at(G, 1 + j, 0);
    __syncthreads();
    if (S.use_iv) {
        for (int e = t; e < na * na; e += DN_THREADS) Qzz[e] = gram_at(G, S.za[e % na], S.za[e / na]);
        for (int e = t; e < na * k; e += DN_THREADS) Qzx[e] = gram_at(G, S.za[e % na], 1 + e / na);
        for (int j = t; j < na; j += DN_THREADS) zy[j] = gram_at(G, S.za[j], 0);
        __syncthreads();
        chol_solve_inv_block(na, Qzz, na, nullptr, zy, rhs, Qiz, &s_info, work);
        __syncthreads();
        if (s_info != 0) {
            if (t == 0) S.info = s_info;
            return;
        }
        // Pi = Qzz^-1 Qzx (na x k); Q = 0.5 (Qzx' Pi + Pi' Qzx); b = Qzx' rhs
        for (int e = t; e < na * k; e += DN_THREADS) {
            const int i = e % na, j = e / na;
            double v = 0.0;
            for (int p = 0; p < na; ++p) v += Qiz[i + p * na] * Qzx[p + j * na];
            Pi[i + j * na] = v;
        }
        __syncthreads();
        for (int e = t; e < k * k; e += DN_THREADS) {
            const int i = e % k, j = e / k;
            double v1 = 0.0, v2 = 0.0;
            for (int p = 0; p < na; ++p) {
                v1 += Qzx[p + i * na] * Pi[p + j * na];
                v2 += Pi[p + i * na] * Qzx[p + j * na];
            }
            Q[i + j * k] = 0.5 * v1 + 0.5 * v2;
        }
        for (int j = t; j < k; j += DN_THREADS) {
            double v = 0.0;
            for (int p = 0; p < na; ++p) v += Qzx[p + j * na] * rhs[p];
            b[j] = v;
        }
        __syncthreads();
    }
    // column filter on the diagonal of W'W
    if (t == 0) {
        double dmax = 0.0;
        for (int j = 0; j < k; ++j) dmax = fmax(dmax, fabs(gram_at(G, 1 + j, 1 + j)));
        dmax = fmax(dmax, 1.0);
        const double tol = 1.0e-10 * dmax;
        int kk = 0;
        for (int j = 0; j < k; ++j)
            if (!(fabs(gram_at(G, 1 + j, 1 + j)) <= tol)) s_kept[kk++] = j;
        s_kk = kk;
        S.kk = kk;
        for (int q = 0; q < kk; ++q) S.kept[q] = s_kept[q];
        if (kk == 0) S.info = -1;
    }
    __syncthreads();
    const int kk = s_kk;
    if (kk == 0) return;
    chol_solve_inv_block(kk, Q, k, s_kept, b, bsel, Qinv, &s_info, work);
    __syncthreads();
    if (s_info != 0) {
        if (t == 0) S.info = s_info;
        return;
    }
    for (int q = t; q < kk; q += DN_THREADS) beta[s_kept[q]] = bsel[q];
}

__device__ __forceinline__ int be_spec_of(const long long* __restrict__ row0, int ns, long long i) {
    int lo = 0, hi = ns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (row0[mid] <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Residual r = y - W beta and score rows S[row][t] = r * x_{score col t}
// (regressors for OLS, Z_aug for 2SLS; zeros past the specification's count),
// one block per item; per-item RSS partials. Score rows are row-major with Sb
// (even) values each.
__global__ void __launch_bounds__(BE_THREADS)
    be_resid_kernel(ColMajorX X, const BeSpecDev* __restrict__ specs, const BeItem* __restrict__ items,
                    const double* __restrict__ beta_full, int Kb, int Sb, long long N, double* __restrict__ S,
                    double* __restrict__ rss_part) {
    const BeItem item = items[blockIdx.x];
    const BeSpecDev& sp = specs[item.spec];
    __shared__ double s_beta[BE_MAX_COLS];
    __shared__ int s_col[BE_MAX_COLS];
    __shared__ double red[BE_THREADS / 32];
    const int k = sp.k;
    const int nsc = sp.use_iv ? sp.na : k;
    for (int j = threadIdx.x; j < Kb; j += BE_THREADS) s_beta[j] = beta_full[(long long)item.spec * Kb + j];
    for (int j = threadIdx.x; j < Sb; j += BE_THREADS) s_col[j] = j < nsc ? (sp.use_iv ? sp.za[j] : 1 + j) : -1;
    __syncthreads();
    double acc = 0.0;
    for (long long r = item.r0 + threadIdx.x; r < item.r1; r += BE_THREADS) {
        double v = X(r, 0);
        for (int j = 0; j < k; ++j) v -= X(r, 1 + j) * s_beta[j];
        acc += v * v;
        if (S) {
            // row-major rows of Sb scores (the cluster sums read whole rows)
            double* srow = S + r * Sb;
            for (int tcol = 0; tcol < Sb; tcol += 2) {
                const double a = s_col[tcol] >= 0 ? v * X(r, s_col[tcol]) : 0.0;
                const double b2 = (tcol + 1 < Sb && s_col[tcol + 1] >= 0) ? v * X(r, s_col[tcol + 1]) : 0.0;
                *reinterpret_cast<double2*>(srow + tcol) = make_double2(a, b2);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < BE_THREADS / 32; ++w) v += red[w];
        rss_part[blockIdx.x] = v;
    }
}

// Sums (mean == nullptr) or squared deviations from the specification's mean
// of its raw y, one block per item.
__global__ void __launch_bounds__(BE_THREADS)
    be_tss_kernel(const double* const* __restrict__ y_raw, const long long* __restrict__ row0,
                  const BeItem* __restrict__ items, const double* __restrict__ mean, double* __restrict__ part) {
    const BeItem item = items[blockIdx.x];
    const double* y = y_raw[item.spec];
    const long long base = row0[item.spec];
    const double m = mean ? mean[item.spec] : 0.0;
    __shared__ double red[BE_THREADS / 32];
    double acc = 0.0;
    for (long long r = item.r0 + threadIdx.x; r < item.r1; r += BE_THREADS) {
        const double v = y[r - base];
        acc += mean ? (v - m) * (v - m) : v;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < BE_THREADS / 32; ++w) v += red[w];
        part[blockIdx.x] = v;
    }
}

// out[s] = sum of part[item] over the items of s (in order); scale[s] (optional) divides
__global__ void be_fold_scalar_kernel(const double* __restrict__ part, const int* __restrict__ item0,
                                      const int* __restrict__ item1, int ns, const long long* __restrict__ divisor,
                                      double* __restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= ns) return;
    double v = 0.0;
    for (int it = item0[s]; it < item1[s]; ++it) v += part[it];
    out[s] = divisor ? v / (double)max(1LL, divisor[s]) : v;
}

// Cluster-subset keys: (specification << LB) | its mixed-radix key over the
// subset's dimensions (0-based local ids), rows of non-participating
// specifications get (ns << LB).
struct BeKeyDims {
    const int32_t* ids[BE_MAX_FE];  // stacked 1-based ids per class dimension
};
__global__ void be_key_kernel(BeKeyDims dims, const long long* __restrict__ row0, int ns, long long N,
                              const int* __restrict__ sub_dim,            // [ns][3] class dimension of subset part j (-1 past m)
                              const unsigned long long* __restrict__ sub_stride,  // [ns][3]
                              const int* __restrict__ goff,                // [ns][BE_MAX_FE]
                              const int* __restrict__ part_spec, int LB, unsigned long long* __restrict__ keys) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < N; i += st) {
        const int s = be_spec_of(row0, ns, i);
        unsigned long long key = (unsigned long long)ns << LB;
        if (part_spec[s]) {
            unsigned long long local = 0;
            for (int j = 0; j < 3; ++j) {
                const int d = sub_dim[s * 3 + j];
                if (d < 0) break;
                const long long v = (long long)dims.ids[d][i] - 1 - goff[s * BE_MAX_FE + d];
                local += (unsigned long long)v * sub_stride[s * 3 + j];
            }
            key = ((unsigned long long)s << LB) | local;
        }
        keys[i] = key;
    }
}

__global__ void be_cluster_flags_kernel(const unsigned long long* __restrict__ skeys, long long n, int ns, int LB,
                                        uint32_t* __restrict__ flags) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; p < n; p += st) {
        const bool valid = (int)(skeys[p] >> LB) < ns;
        flags[p] = (valid && (p == 0 || skeys[p] != skeys[p - 1])) ? 1u : 0u;
    }
}

__global__ void be_cluster_offsets_kernel(const unsigned long long* __restrict__ skeys,
                                          const uint32_t* __restrict__ flags, const uint32_t* __restrict__ excl,
                                          long long n, int LB, int32_t* __restrict__ off,
                                          int32_t* __restrict__ cl_spec) {
    long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; p < n; p += st)
        if (flags[p]) {
            off[excl[p]] = (int32_t)p;
            cl_spec[excl[p]] = (int32_t)(skeys[p] >> LB);
        }
}

// first and one-past-last cluster of every specification (clusters are in specification order)
__global__ void be_cluster_ranges_kernel(const int32_t* __restrict__ cl_spec, int n_cl, int* __restrict__ c0,
                                         int* __restrict__ c1) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    const int st = gridDim.x * blockDim.x;
    for (; c < n_cl; c += st) {
        const int s = cl_spec[c];
        if (c == 0 || cl_spec[c - 1] != s) c0[s] = c;
        if (c == n_cl - 1 || cl_spec[c + 1] != s) c1[s] = c + 1;
    }
}

// Sc[c][t] = sum over the rows of cluster c (in sorted order) of S[row][t]:
// one warp per cluster, lanes over the columns, so every row is one
// contiguous read.
__global__ void be_cluster_sums_kernel(const double* __restrict__ S, int Sb, const int32_t* __restrict__ perm,
                                       const int32_t* __restrict__ off, int n_cl, double* __restrict__ Sc) {
    const int lane = threadIdx.x & 31;
    long long c = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long st = ((long long)gridDim.x * blockDim.x) >> 5;
    for (; c < n_cl; c += st) {
        double a0 = 0.0, a1 = 0.0;
        for (int p = off[c]; p < off[c + 1]; ++p) {
            const double* row = S + (long long)perm[p] * Sb;
            if (lane < Sb) a0 += row[lane];
            if (lane + 32 < Sb) a1 += row[lane + 32];
        }
        if (lane < Sb) Sc[c * Sb + lane] = a0;
        if (lane + 32 < Sb) Sc[c * Sb + lane + 32] = a1;
    }
}

// acc (kk x kk) += w Qinv M_sel Qinv, M = the meat (pairs over Cw) of the
// score columns; 2SLS: M_k = Pi' M Pi first. One block per participating
// specification.
__global__ void __launch_bounds__(DN_THREADS)
    be_sandwich_kernel(const BeSpecDev* __restrict__ specs, const int* __restrict__ part_spec,
                       const double* __restrict__ meat, int Cw, int Kb, const double* __restrict__ Qinv_all,
                       const double* __restrict__ Pi_all, double w, double* __restrict__ acc_all,
                       double* __restrict__ scratch) {
    const int s = blockIdx.x;
    if (!part_spec[s]) return;
    const BeSpecDev& S = specs[s];
    if (S.info != 0 || S.kk == 0) return;
    const int k = S.k, kk = S.kk;
    const int nsc = S.use_iv ? S.na : k;
    const double* G = meat + (long long)s * (Cw * (Cw + 1) / 2);
    const double* Qinv = Qinv_all + (long long)s * Kb * Kb;
    const double* Pi = Pi_all + (long long)s * Kb * Kb;
    double* acc = acc_all + (long long)s * Kb * Kb;
    double* M = scratch + (long long)s * be_scratch_per_spec(Kb);  // reuses the solve scratch (free by now)
    double* Mk = M + Kb * Kb;
    double* T = Mk + Kb * Kb;
    const int t = threadIdx.x;
    for (int e = t; e < nsc * nsc; e += DN_THREADS) M[e] = gram_at(G, e % nsc, e / nsc);
    __syncthreads();
    if (S.use_iv) {
        const int na = S.na;
        // T = M Pi (na x k), Mk = Pi' T (k x k)
        for (int e = t; e < na * k; e += DN_THREADS) {
            const int i = e % na, j = e / na;
            double v = 0.0;
            for (int p = 0; p < na; ++p) v += M[i + p * na] * Pi[p + j * na];
            T[i + j * na] = v;
        }
        __syncthreads();
        for (int e = t; e < k * k; e += DN_THREADS) {
            const int i = e % k, j = e / k;
            double v = 0.0;
            for (int p = 0; p < na; ++p) v += Pi[p + i * na] * T[p + j * na];
            Mk[i + j * k] = v;
        }
    } else {
        for (int e = t; e < k * k; e += DN_THREADS) Mk[e] = M[e];
    }
    __syncthreads();
    // T = M_sel Qinv, acc += w Qinv T
    for (int e = t; e < kk * kk; e += DN_THREADS) {
        const int i = e % kk, j = e / kk;
        double v = 0.0;
        for (int p = 0; p < kk; ++p) v += Mk[S.kept[i] + S.kept[p] * k] * Qinv[p + j * kk];
        T[i + j * kk] = v;
    }
    __syncthreads();
    for (int e = t; e < kk * kk; e += DN_THREADS) {
        const int i = e % kk, j = e / kk;
        double v = 0.0;
        for (int p = 0; p < kk; ++p) v += Qinv[i + p * kk] * T[p + j * kk];
        acc[i + j * kk] += w * v;
    }
}

// SEs of every specification: clustered (scalar[s] > 0: scaled sandwich and
// the PSD fix) or homoskedastic (sigma2[s] Qinv_jj).
__global__ void __launch_bounds__(DN_THREADS)
    be_finalize_kernel(const BeSpecDev* __restrict__ specs, int Kb, const double* __restrict__ Qinv_all,
                       double* __restrict__ acc_all, const double* __restrict__ scalar, const double* __restrict__ rss,
                       const long long* __restrict__ df_homo, double* __restrict__ se_all, int* __restrict__ psd,
                       double* __restrict__ scratch) {
    const int s = blockIdx.x;
    const BeSpecDev& S = specs[s];
    double* se = se_all + (long long)s * Kb;
    const int t = threadIdx.x;
    for (int j = t; j < Kb; j += DN_THREADS) se[j] = 0.0;
    if (t == 0) psd[s] = 0;
    __syncthreads();
    if (S.info != 0 || S.kk == 0) return;
    const int kk = S.kk;
    double* sel = scratch + (long long)s * be_scratch_per_spec(Kb);
    double* work = sel + Kb;
    if (scalar[s] > 0.0) {
        __shared__ int s_psd;
        finalize_cov_block(kk, acc_all + (long long)s * Kb * Kb, scalar[s], 1, sel, &s_psd, work);
        __syncthreads();
        for (int q = t; q < kk; q += DN_THREADS) se[S.kept[q]] = sel[q];
        if (t == 0) psd[s] = s_psd;
    } else {
        const double sigma2 = rss[s] / (double)max(1LL, df_homo[s]);
        const double* Qinv = Qinv_all + (long long)s * Kb * Kb;
        for (int q = t; q < kk; q += DN_THREADS) se[S.kept[q]] = sqrt(fmax(0.0, sigma2 * Qinv[q + q * kk]));
    }
}

int be_sync_copy(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s, const char* what) {
    if (bytes == 0) return 0;
    FEGB_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, s), what);
    FEGB_CUDA(cudaStreamSynchronize(s), what);
    return 0;
}

// Gram products through the work queue: split-FP32 first, FP64 again when a
// value is outside the split range; folded per specification into out.
template <class Acc>
int be_gram(Acc X, const std::vector<BeItem>& hitems, const std::vector<int>& item0, const std::vector<int>& item1,
            const int* d_width, int ns, int Cw, double* out, cudaStream_t s, Scratch& scr) {
    const int P = Cw * (Cw + 1) / 2;
    const int n_items = (int)hitems.size();
    if (n_items == 0) {
        FEGB_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * (size_t)ns * P, s), "batch gram zero");
        return 0;
    }
    BeItem* d_items = nullptr;
    int *d_i0 = nullptr, *d_i1 = nullptr, *d_q = nullptr, *d_bad = nullptr;
    double* part = nullptr;
    FEGB_TRY(scr.alloc(&d_items, hitems.size(), "batch items"));
    FEGB_TRY(scr.alloc(&d_i0, (size_t)ns, "batch item0"));
    FEGB_TRY(scr.alloc(&d_i1, (size_t)ns, "batch item1"));
    FEGB_TRY(scr.alloc(&d_q, 2, "batch queue"));
    FEGB_TRY(scr.alloc(&d_bad, 1, "batch split flag"));
    FEGB_TRY(scr.alloc(&part, (size_t)n_items * P, "batch gram partials"));
    FEGB_CUDA(cudaMemcpyAsync(d_items, hitems.data(), sizeof(BeItem) * hitems.size(), cudaMemcpyHostToDevice, s),
              "batch items copy");
    FEGB_CUDA(cudaMemcpyAsync(d_i0, item0.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s), "batch item0 copy");
    FEGB_CUDA(cudaMemcpyAsync(d_i1, item1.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s), "batch item1 copy");
    FEGB_CUDA(cudaMemsetAsync(d_q, 0, sizeof(int) * 2, s), "batch queue reset");
    FEGB_CUDA(cudaMemsetAsync(d_bad, 0, sizeof(int), s), "batch flag reset");
    const int grid = std::min(n_items, num_sms() * 4);
    const size_t smem = sizeof(double) * (size_t)be_tile_rows(Cw) * Cw;  // float2 and double are both 8 bytes
    auto launch = [&](bool split, int* q) -> int {
        const int ppt = be_ppt(Cw);
#define BE_GRAM_CASE(NPT)                                                                                          \
    if (ppt == NPT) {                                                                                              \
        if (split)                                                                                                 \
            be_gram_kernel<Acc, true, NPT><<<grid, BE_THREADS, smem, s>>>(X, d_items, n_items, d_width, Cw, part, q, \
                                                                          d_bad);                                  \
        else                                                                                                       \
            be_gram_kernel<Acc, false, NPT><<<grid, BE_THREADS, smem, s>>>(X, d_items, n_items, d_width, Cw, part,   \
                                                                           q, d_bad);                              \
    }
        BE_GRAM_CASE(1)
        BE_GRAM_CASE(2)
        BE_GRAM_CASE(4)
        BE_GRAM_CASE(9)
#undef BE_GRAM_CASE
        FEGB_LAUNCH_CHECK("batch gram");
        return 0;
    };
    if (Cw >= 16) {
        // the blocked double-single form (16 products per 8 shared-memory reads);
        // below 16 columns there are too few 4 x 4 blocks per row and the
        // phases' folds cost more than the reads saved (8 columns: 25 -> 30 ms)
        const int cw4 = (Cw + 3) / 4 * 4;
        const size_t bsmem = sizeof(float2) * (size_t)be_tile_rows(Cw) * cw4;
        // the tile (up to 64 KB) beside the 35 KB of static fold space
        static const cudaError_t attr = cudaFuncSetAttribute(be_gram_blocked_kernel<Acc>,
                                                             cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        if (attr != cudaSuccess) return set_cuda_error(attr, "batch gram (blocked) attr");
        be_gram_blocked_kernel<Acc><<<grid, BE_THREADS, bsmem, s>>>(X, d_items, n_items, d_width, Cw, part, d_q,
                                                                    d_bad);
        FEGB_LAUNCH_CHECK("batch gram (blocked)");
    } else {
        FEGB_TRY(launch(true, d_q));
    }
    int hbad = 0;
    FEGB_TRY(be_sync_copy(&hbad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, s, "batch split flag copy"));
    if (hbad) FEGB_TRY(launch(false, d_q + 1));
    be_fold_kernel<<<ns, 256, 0, s>>>(part, d_i0, d_i1, P, out);
    FEGB_LAUNCH_CHECK("batch gram fold");
    return 0;
}

void be_items(const std::vector<long long>& begin, const std::vector<long long>& end, std::vector<BeItem>& items,
              std::vector<int>& item0, std::vector<int>& item1) {
    const int ns = (int)begin.size();
    items.clear();
    item0.assign(ns, 0);
    item1.assign(ns, 0);
    for (int s = 0; s < ns; ++s) {
        item0[s] = (int)items.size();
        for (long long r = begin[s]; r < end[s]; r += BE_ITEM_ROWS) items.push_back({s, r, std::min(end[s], r + BE_ITEM_ROWS)});
        item1[s] = (int)items.size();
    }
}

}  // namespace

bool batch_est_eligible(const fegb_config& cfg, int Cw, const std::vector<BeSpecHost>& specs) {
    if (cfg.se_convention != FEGB_SE_GPU || Cw > BE_MAX_COLS || specs.empty()) return false;
    const int sb = bits_for((unsigned long long)specs.size() + 1);
    for (const BeSpecHost& S : specs) {
        if (S.n_fe > BE_MAX_FE || S.n_cd > 3 || S.k < 1 || S.k + S.l + 1 > Cw || S.k > BE_MAX_COLS) return false;
        if (S.n > 0x7fffffffLL) return false;
        unsigned long long span = 1;
        for (int j = 0; j < S.n_cd; ++j) {
            const unsigned long long g = (unsigned long long)std::max(1, S.G[S.cd[j]]);
            if (span > (1ULL << 62) / g) return false;
            span *= g;
        }
        if (bits_for(span) + sb > 63) return false;
    }
    return true;
}

int estimate_class_batched(const fegb_config& cfg, const std::vector<BeSpecHost>& specs, long long N, int Cw,
                           const double* yb, const double* Wb, const int32_t* const* ids_b, int n_fe_b,
                           double* const* beta, double* const* se, fegb_result* const* results, cudaStream_t s) {
    const int ns = (int)specs.size();
    if (ns == 0) return 0;
    Scratch scr(s);
    // FEGB_TRACE=1: the stream is synchronised after each phase and its time printed
    static const bool trace = [] {
        const char* v = std::getenv("FEGB_TRACE");
        return v && v[0] && v[0] != '0';
    }();
    auto tp = BeClock::now();
    auto phase = [&](const char* what) -> int {
        if (!trace) return 0;
        FEGB_CUDA(cudaStreamSynchronize(s), "trace sync");
        std::fprintf(stderr, "fegb batch est: %-28s %8.2f ms\n", what, be_seconds_since(tp) * 1e3);
        tp = BeClock::now();
        return 0;
    };
    const int Kb = Cw;  // regressors and score columns per specification: at most Cw - 1
    const int P = Cw * (Cw + 1) / 2;
    auto t0 = BeClock::now();
    // ---- specification records ----
    std::vector<BeSpecDev> hd(ns);
    std::vector<long long> rb(ns), re(ns), row0(ns), nrow(ns);
    std::vector<int> width(ns);
    for (int i = 0; i < ns; ++i) {
        const BeSpecHost& S = specs[i];
        BeSpecDev& D = hd[i];
        std::memset(&D, 0, sizeof(D));
        D.row0 = S.row0;
        D.n = S.n;
        D.k = S.k;
        D.l = S.l;
        D.cs = 1 + S.k + S.l;
        for (int v : S.endog)
            if (v >= 1 && v <= S.k) D.endog_mask[(v - 1) >> 5] |= 1 << ((v - 1) & 31);
        int nsel = 0;
        if (S.l > 0) {
            for (int v : S.instr)
                if (v >= 1 && v <= S.l && nsel < BE_MAX_COLS) D.sel[nsel++] = v;
            if (nsel == 0)
                for (int v = 1; v <= S.l && nsel < BE_MAX_COLS; ++v) D.sel[nsel++] = v;
        }
        D.n_sel = nsel;
        rb[i] = S.row0;
        re[i] = S.row0 + S.n;
        row0[i] = S.row0;
        nrow[i] = S.n;
        width[i] = D.cs;
    }
    BeSpecDev* d_specs = nullptr;
    long long *d_row0 = nullptr, *d_n = nullptr;
    int* d_width = nullptr;
    FEGB_TRY(scr.alloc(&d_specs, (size_t)ns, "batch spec records"));
    FEGB_TRY(scr.alloc(&d_row0, (size_t)ns, "batch row0"));
    FEGB_TRY(scr.alloc(&d_n, (size_t)ns, "batch rows"));
    FEGB_TRY(scr.alloc(&d_width, (size_t)ns, "batch widths"));
    FEGB_CUDA(cudaMemcpyAsync(d_specs, hd.data(), sizeof(BeSpecDev) * ns, cudaMemcpyHostToDevice, s), "spec copy");
    FEGB_CUDA(cudaMemcpyAsync(d_row0, row0.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, s), "row0 copy");
    FEGB_CUDA(cudaMemcpyAsync(d_n, nrow.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, s), "rows copy");
    FEGB_CUDA(cudaMemcpyAsync(d_width, width.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s), "width copy");
    std::vector<BeItem> items;
    std::vector<int> item0, item1;
    be_items(rb, re, items, item0, item1);
    const int n_items = (int)items.size();
    BeItem* d_items = nullptr;
    int *d_i0 = nullptr, *d_i1 = nullptr;
    FEGB_TRY(scr.alloc(&d_items, (size_t)std::max(1, n_items), "row items"));
    FEGB_TRY(scr.alloc(&d_i0, (size_t)ns, "row item0"));
    FEGB_TRY(scr.alloc(&d_i1, (size_t)ns, "row item1"));
    if (n_items)
        FEGB_CUDA(cudaMemcpyAsync(d_items, items.data(), sizeof(BeItem) * n_items, cudaMemcpyHostToDevice, s),
                  "row items copy");
    FEGB_CUDA(cudaMemcpyAsync(d_i0, item0.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s), "item0 copy");
    FEGB_CUDA(cudaMemcpyAsync(d_i1, item1.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s), "item1 copy");

    // ---- total sum of squares of each raw y ----
    std::vector<const double*> yraw(ns);
    for (int i = 0; i < ns; ++i) yraw[i] = specs[i].y_raw;
    const double** d_yraw = nullptr;
    double *d_part = nullptr, *d_mean = nullptr, *d_tss = nullptr;
    FEGB_TRY(scr.alloc(&d_yraw, (size_t)ns, "raw y pointers"));
    FEGB_TRY(scr.alloc(&d_part, (size_t)std::max(1, n_items), "item partials"));
    FEGB_TRY(scr.alloc(&d_mean, (size_t)ns, "y means"));
    FEGB_TRY(scr.alloc(&d_tss, (size_t)ns, "tss"));
    FEGB_CUDA(cudaMemcpyAsync(d_yraw, yraw.data(), sizeof(double*) * ns, cudaMemcpyHostToDevice, s), "yraw copy");
    if (n_items) {
        be_tss_kernel<<<n_items, BE_THREADS, 0, s>>>(d_yraw, d_row0, d_items, nullptr, d_part);
        be_fold_scalar_kernel<<<(ns + 127) / 128, 128, 0, s>>>(d_part, d_i0, d_i1, ns, d_n, d_mean);
        be_tss_kernel<<<n_items, BE_THREADS, 0, s>>>(d_yraw, d_row0, d_items, d_mean, d_part);
        be_fold_scalar_kernel<<<(ns + 127) / 128, 128, 0, s>>>(d_part, d_i0, d_i1, ns, nullptr, d_tss);
        FEGB_LAUNCH_CHECK("batch tss");
    } else {
        FEGB_CUDA(cudaMemsetAsync(d_tss, 0, sizeof(double) * ns, s), "tss zero");
    }
    FEGB_TRY(phase("records and tss"));

    // ---- Gram products and solves ----
    double *d_gram = nullptr, *d_scratch = nullptr, *d_beta = nullptr, *d_Qinv = nullptr, *d_Pi = nullptr;
    FEGB_TRY(scr.alloc(&d_gram, (size_t)ns * P, "batch grams"));
    FEGB_TRY(scr.alloc(&d_scratch, (size_t)ns * be_scratch_per_spec(Kb), "batch dense scratch"));
    FEGB_TRY(scr.alloc(&d_beta, (size_t)ns * Kb, "batch beta"));
    FEGB_TRY(scr.alloc(&d_Qinv, (size_t)ns * Kb * Kb, "batch Qinv"));
    FEGB_TRY(scr.alloc(&d_Pi, (size_t)ns * Kb * Kb, "batch Pi"));
    ColMajorX X{yb, Wb, N};
    FEGB_TRY(be_gram(X, items, item0, item1, d_width, ns, Cw, d_gram, s, scr));
    FEGB_TRY(phase("gram"));
    be_solve_kernel<<<ns, DN_THREADS, 0, s>>>(d_specs, d_gram, Cw, Kb, d_scratch, d_beta, d_Qinv, d_Pi);
    FEGB_LAUNCH_CHECK("batch solve");
    FEGB_CUDA(cudaStreamSynchronize(s), "batch solve sync");
    const double t_regression = be_seconds_since(t0);
    t0 = BeClock::now();

    // ---- residuals, scores, RSS ----
    bool any_cluster = false;
    for (const BeSpecHost& S : specs) any_cluster = any_cluster || S.n_cd > 0;
    const int Sb = (Cw + 1) / 2 * 2;  // score values per row (at most Cw - 1 used), even for 16-byte stores
    double* d_S = nullptr;
    double* d_rss = nullptr;
    if (any_cluster) FEGB_TRY(scr.alloc(&d_S, (size_t)N * Sb, "batch score columns"));
    FEGB_TRY(scr.alloc(&d_rss, (size_t)ns, "batch rss"));
    if (n_items) {
        be_resid_kernel<<<n_items, BE_THREADS, 0, s>>>(X, d_specs, d_items, d_beta, Kb, Sb, N, d_S, d_part);
        FEGB_LAUNCH_CHECK("batch residuals");
        be_fold_scalar_kernel<<<(ns + 127) / 128, 128, 0, s>>>(d_part, d_i0, d_i1, ns, nullptr, d_rss);
        FEGB_LAUNCH_CHECK("batch rss fold");
    } else {
        FEGB_CUDA(cudaMemsetAsync(d_rss, 0, sizeof(double) * ns, s), "rss zero");
    }
    FEGB_TRY(phase("residuals and scores"));
    // solve outcomes (kept columns and dof) for the host
    std::vector<BeSpecDev> hs(ns);
    FEGB_TRY(be_sync_copy(hs.data(), d_specs, sizeof(BeSpecDev) * ns, cudaMemcpyDeviceToHost, s, "spec results copy"));

    // ---- clustered SEs: one pass per subset mask ----
    double* d_acc = nullptr;
    FEGB_TRY(scr.alloc(&d_acc, (size_t)ns * Kb * Kb, "batch sandwich"));
    FEGB_CUDA(cudaMemsetAsync(d_acc, 0, sizeof(double) * (size_t)ns * Kb * Kb, s), "sandwich zero");
    std::vector<long long> min_single(ns, LLONG_MAX);
    if (any_cluster) {
        BeKeyDims kd{};
        for (int d = 0; d < n_fe_b && d < BE_MAX_FE; ++d) kd.ids[d] = ids_b[d];
        int *d_subdim = nullptr, *d_goff = nullptr, *d_part_spec = nullptr;
        unsigned long long* d_stride = nullptr;
        FEGB_TRY(scr.alloc(&d_subdim, (size_t)ns * 3, "subset dims"));
        FEGB_TRY(scr.alloc(&d_stride, (size_t)ns * 3, "subset strides"));
        FEGB_TRY(scr.alloc(&d_goff, (size_t)ns * BE_MAX_FE, "group offsets"));
        FEGB_TRY(scr.alloc(&d_part_spec, (size_t)ns, "participating specs"));
        std::vector<int> hgoff((size_t)ns * BE_MAX_FE, 0);
        for (int i = 0; i < ns; ++i)
            for (int d = 0; d < BE_MAX_FE; ++d) hgoff[(size_t)i * BE_MAX_FE + d] = specs[i].goff[d];
        FEGB_CUDA(cudaMemcpyAsync(d_goff, hgoff.data(), sizeof(int) * hgoff.size(), cudaMemcpyHostToDevice, s),
                  "goff copy");
        unsigned long long *keys = nullptr, *skeys = nullptr;
        int32_t *perm = nullptr, *off = nullptr, *cl_spec = nullptr;
        uint32_t *flags = nullptr, *excl = nullptr, *total = nullptr;
        int *d_c0 = nullptr, *d_c1 = nullptr;
        FEGB_TRY(scr.alloc(&keys, (size_t)N, "cluster keys"));
        FEGB_TRY(scr.alloc(&skeys, (size_t)N, "sorted cluster keys"));
        FEGB_TRY(scr.alloc(&perm, (size_t)N, "cluster perm"));
        FEGB_TRY(scr.alloc(&flags, (size_t)N, "cluster flags"));
        FEGB_TRY(scr.alloc(&excl, (size_t)N, "cluster scan"));
        FEGB_TRY(scr.alloc(&total, 1, "cluster count"));
        FEGB_TRY(scr.alloc(&off, (size_t)N + 1, "cluster offsets"));
        FEGB_TRY(scr.alloc(&cl_spec, (size_t)N, "cluster specs"));
        FEGB_TRY(scr.alloc(&d_c0, (size_t)ns, "cluster begin"));
        FEGB_TRY(scr.alloc(&d_c1, (size_t)ns, "cluster end"));
        double* d_meat = nullptr;
        FEGB_TRY(scr.alloc(&d_meat, (size_t)ns * P, "batch meats"));
        double* Sc = nullptr;
        FEGB_TRY(scr.alloc(&Sc, (size_t)N * Sb, "cluster score sums"));
        const int SB = bits_for((unsigned long long)ns + 1);
        for (int mask = 1; mask < 8; ++mask) {
            const int m = __builtin_popcount((unsigned)mask);
            std::vector<int> subdim((size_t)ns * 3, -1), part(ns, 0);
            std::vector<unsigned long long> stride((size_t)ns * 3, 0);
            int LB = 1;
            long long n_valid = 0;
            bool any = false;
            for (int i = 0; i < ns; ++i) {
                const BeSpecHost& S = specs[i];
                if (hs[i].info != 0 || hs[i].kk == 0 || S.n_cd == 0 || (mask >> S.n_cd) != 0) continue;
                part[i] = 1;
                any = true;
                n_valid += S.n;
                unsigned long long st = 1;
                int j2 = 0;
                for (int j = 0; j < S.n_cd; ++j) {
                    if (!((mask >> j) & 1)) continue;
                    subdim[(size_t)i * 3 + j2] = S.cd[j];
                    stride[(size_t)i * 3 + j2] = st;
                    st *= (unsigned long long)std::max(1, S.G[S.cd[j]]);
                    ++j2;
                }
                LB = std::max(LB, bits_for(st));
                if (m == 1) min_single[i] = std::min(min_single[i], (long long)S.G[S.cd[__builtin_ctz((unsigned)mask)]]);
            }
            if (!any) continue;
            FEGB_CUDA(cudaMemcpyAsync(d_subdim, subdim.data(), sizeof(int) * subdim.size(), cudaMemcpyHostToDevice, s),
                      "subset dims copy");
            FEGB_CUDA(cudaMemcpyAsync(d_stride, stride.data(), sizeof(unsigned long long) * stride.size(),
                                      cudaMemcpyHostToDevice, s),
                      "subset strides copy");
            FEGB_CUDA(cudaMemcpyAsync(d_part_spec, part.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s),
                      "participants copy");
            be_key_kernel<<<grid_stride_blocks(N, 256), 256, 0, s>>>(kd, d_row0, ns, N, d_subdim, d_stride, d_goff,
                                                                    d_part_spec, LB, keys);
            FEGB_LAUNCH_CHECK("cluster keys");
            FEGB_TRY(phase("cluster keys"));
            FEGB_TRY(radix_sort_u64(keys, nullptr, skeys, perm, N, LB + SB, s, scr));
            FEGB_TRY(phase("cluster sort"));
            be_cluster_flags_kernel<<<grid_stride_blocks(N, 256), 256, 0, s>>>(skeys, N, ns, LB, flags);
            FEGB_LAUNCH_CHECK("cluster flags");
            FEGB_TRY(scan_exclusive_u32(flags, excl, N, total, s, scr));
            uint32_t h_ncl = 0;
            FEGB_TRY(be_sync_copy(&h_ncl, total, sizeof(uint32_t), cudaMemcpyDeviceToHost, s, "cluster count copy"));
            const int n_cl = (int)h_ncl;
            be_cluster_offsets_kernel<<<grid_stride_blocks(N, 256), 256, 0, s>>>(skeys, flags, excl, N, LB, off,
                                                                                cl_spec);
            FEGB_LAUNCH_CHECK("cluster offsets");
            const int32_t nv = (int32_t)n_valid;
            FEGB_CUDA(cudaMemcpyAsync(off + n_cl, &nv, sizeof(int32_t), cudaMemcpyHostToDevice, s), "offsets end");
            FEGB_CUDA(cudaMemsetAsync(d_c0, 0, sizeof(int) * ns, s), "cluster begin zero");
            FEGB_CUDA(cudaMemsetAsync(d_c1, 0, sizeof(int) * ns, s), "cluster end zero");
            if (n_cl > 0) {
                be_cluster_ranges_kernel<<<grid_stride_blocks(n_cl, 256), 256, 0, s>>>(cl_spec, n_cl, d_c0, d_c1);
                be_cluster_sums_kernel<<<grid_stride_blocks((long long)n_cl * 32, 256), 256, 0, s>>>(d_S, Sb, perm,
                                                                                                  off, n_cl, Sc);
                FEGB_LAUNCH_CHECK("cluster score sums");
            }
            std::vector<int> c0(ns), c1(ns);
            FEGB_TRY(be_sync_copy(c0.data(), d_c0, sizeof(int) * ns, cudaMemcpyDeviceToHost, s, "cluster begin copy"));
            FEGB_TRY(be_sync_copy(c1.data(), d_c1, sizeof(int) * ns, cudaMemcpyDeviceToHost, s, "cluster end copy"));
            std::vector<long long> cb(ns), ce(ns);
            std::vector<int> swidth(ns);
            for (int i = 0; i < ns; ++i) {
                cb[i] = part[i] ? c0[i] : 0;
                ce[i] = part[i] ? c1[i] : 0;
                swidth[i] = hs[i].use_iv ? hs[i].na : hs[i].k;
            }
            std::vector<BeItem> citems;
            std::vector<int> ci0, ci1;
            be_items(cb, ce, citems, ci0, ci1);
            int* d_swidth = nullptr;
            FEGB_TRY(scr.alloc(&d_swidth, (size_t)ns, "score widths"));
            FEGB_CUDA(cudaMemcpyAsync(d_swidth, swidth.data(), sizeof(int) * ns, cudaMemcpyHostToDevice, s),
                      "score widths copy");
            FEGB_TRY(phase("cluster sums"));
            RowMajor R{Sc, Sb};
            FEGB_TRY(be_gram(R, citems, ci0, ci1, d_swidth, ns, Cw, d_meat, s, scr));
            FEGB_TRY(phase("meat gram"));
            be_sandwich_kernel<<<ns, DN_THREADS, 0, s>>>(d_specs, d_part_spec, d_meat, Cw, Kb, d_Qinv, d_Pi,
                                                         (m % 2 == 1) ? 1.0 : -1.0, d_acc, d_scratch);
            FEGB_LAUNCH_CHECK("batch sandwich");
            FEGB_TRY(phase("sandwich"));
        }
    }

    // ---- SEs, dof and statistics ----
    std::vector<double> hscalar(ns, 0.0);
    std::vector<long long> hdf(ns, 1);
    std::vector<double> hrss(ns), htss(ns);
    FEGB_TRY(be_sync_copy(hrss.data(), d_rss, sizeof(double) * ns, cudaMemcpyDeviceToHost, s, "rss copy"));
    FEGB_TRY(be_sync_copy(htss.data(), d_tss, sizeof(double) * ns, cudaMemcpyDeviceToHost, s, "tss copy"));
    std::vector<int> dof_fes(ns, 0);
    for (int i = 0; i < ns; ++i) {
        const BeSpecHost& S = specs[i];
        for (int d = 0; d < S.n_fe; ++d) dof_fes[i] += std::max(0, S.G[d] - 1);
        const long long pc = (long long)std::max(0, hs[i].kk) + std::max(0, dof_fes[i]) + 1;
        hdf[i] = std::max(1LL, S.n - pc);
        if (S.n_cd > 0 && hs[i].info == 0 && hs[i].kk > 0 && min_single[i] != LLONG_MAX) {
            int nested = 0;
            for (int j = 0; j < S.n_cd; ++j) nested += std::max(0, S.G[S.cd[j]] - 1);
            const long long pce = (long long)hs[i].kk + (nested > 0 ? 1 : 0);
            double scalar = (double)std::max(1LL, S.n - 1) / (double)std::max(1LL, S.n - pce);
            const long long ms = min_single[i];
            if (ms > 1) scalar *= (double)ms / (double)(ms - 1);
            hscalar[i] = scalar;
        }
    }
    double* d_scalar = nullptr;
    long long* d_df = nullptr;
    double* d_se = nullptr;
    int* d_psd = nullptr;
    FEGB_TRY(scr.alloc(&d_scalar, (size_t)ns, "batch scalars"));
    FEGB_TRY(scr.alloc(&d_df, (size_t)ns, "batch dof"));
    FEGB_TRY(scr.alloc(&d_se, (size_t)ns * Kb, "batch se"));
    FEGB_TRY(scr.alloc(&d_psd, (size_t)ns, "batch psd"));
    FEGB_CUDA(cudaMemcpyAsync(d_scalar, hscalar.data(), sizeof(double) * ns, cudaMemcpyHostToDevice, s), "scalar copy");
    FEGB_CUDA(cudaMemcpyAsync(d_df, hdf.data(), sizeof(long long) * ns, cudaMemcpyHostToDevice, s), "dof copy");
    be_finalize_kernel<<<ns, DN_THREADS, 0, s>>>(d_specs, Kb, d_Qinv, d_acc, d_scalar, d_rss, d_df, d_se, d_psd,
                                                 d_scratch);
    FEGB_LAUNCH_CHECK("batch finalize");
    std::vector<double> hbeta((size_t)ns * Kb), hse((size_t)ns * Kb);
    std::vector<int> hpsd(ns);
    FEGB_CUDA(cudaMemcpyAsync(hbeta.data(), d_beta, sizeof(double) * hbeta.size(), cudaMemcpyDeviceToHost, s), "beta");
    FEGB_CUDA(cudaMemcpyAsync(hse.data(), d_se, sizeof(double) * hse.size(), cudaMemcpyDeviceToHost, s), "se");
    FEGB_TRY(be_sync_copy(hpsd.data(), d_psd, sizeof(int) * ns, cudaMemcpyDeviceToHost, s, "psd copy"));
    FEGB_TRY(phase("finalize"));
    const double t_se = be_seconds_since(t0);
    for (int i = 0; i < ns; ++i) {
        const BeSpecHost& S = specs[i];
        fegb_result* r = results[i];
        for (int j = 0; j < S.k; ++j) {
            beta[i][j] = hbeta[(size_t)i * Kb + j];
            se[i][j] = hse[(size_t)i * Kb + j];
        }
        r->solver_info = hs[i].info;
        r->rank = hs[i].info == 0 ? hs[i].kk : 0;
        r->dof_model = hs[i].kk;
        r->dof_fes = dof_fes[i];
        r->is_iv = hs[i].use_iv;
        r->n_instruments = hs[i].use_iv ? hs[i].na : 0;
        r->tss_total = htss[i];
        r->tss_within = hs[i].tss_within;
        r->rss = hrss[i];
        r->n_obs_used = S.n;
        r->dof_resid = hdf[i];
        if (hscalar[i] > 0.0) {
            const long long ms = min_single[i];
            r->psd_fix_applied = hpsd[i];
            r->n_cluster_dims_used = S.n_cd;
            r->min_single_cluster = (int)ms;
            if (ms > 0) r->dof_resid = std::max(1LL, ms - 1);
        }
        r->time_regression = t_regression / ns;
        r->time_se = t_se / ns;
    }
    return 0;
}

}  // namespace fegb
