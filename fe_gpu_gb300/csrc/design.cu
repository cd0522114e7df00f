// Formula design-matrix expansion on the device.
//
// The reference expands Stata-style factor notation on the host
// (build_formula_design_matrix, src/src_main.f90:595-736): every regressor of
// the expanded matrix is a product of factors taken left to right, a factor
// being either a raw column or the dummy (nint(x) == level) of a categorical
// column (append_main_term_columns :1178-1231, build_factor_block :1322-1380,
// products in append_interaction_columns :1269-1320). Here the host only
// plans the columns; the per-row work (level collection over the raw column
// and the products) runs in the kernels below, writing the expanded columns
// straight into the device matrix the estimator reads.
#include "common.cuh"
#include "prep.cuh"

#include <algorithm>
#include <climits>
#include <cmath>

#include "fegb.h"

namespace fegb {
namespace {

// Category test of the reference (src/src_main.f90:1400-1402): a value counts
// as an integer level when it lies within 1e-6 of nint(x). Values whose
// nearest integer does not fit int32 never count (the reference's int(nint())
// would overflow there).
constexpr double CATEGORY_TOL = 1.0e-6;

__device__ __forceinline__ bool nearest_int32(double x, int* out) {
    const double r = round(x);  // halves away from zero, as Fortran nint
    if (!(fabs(r) <= 2147483647.0)) return false;
    *out = (int)r;
    return true;
}

// flag[i] = 1 when row i holds an integer level; key[i] = its order-preserving
// unsigned code (sign bit flipped).
__global__ void level_flags_kernel(const double* __restrict__ col, long long n, uint32_t* __restrict__ flag,
                                   uint32_t* __restrict__ key) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        const double x = col[i];
        int v = 0;
        const bool ok = nearest_int32(x, &v) && fabs(x - (double)v) <= CATEGORY_TOL;
        flag[i] = ok ? 1u : 0u;
        key[i] = (uint32_t)v ^ 0x80000000u;
    }
}

// Compacts the flagged rows: (key, row) pairs in row order.
__global__ void level_compact_kernel(const uint32_t* __restrict__ flag, const uint32_t* __restrict__ pos,
                                     const uint32_t* __restrict__ key, long long n, uint32_t* __restrict__ ckey,
                                     int32_t* __restrict__ crow) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        if (flag[i]) {
            ckey[pos[i]] = key[i];
            crow[pos[i]] = (int32_t)i;
        }
    }
}

// head[j] = 1 at the first entry of each run of equal keys (keys sorted).
__global__ void level_heads_kernel(const uint32_t* __restrict__ skey, long long m, uint32_t* __restrict__ head) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; j < m; j += st) head[j] = (j == 0 || skey[j] != skey[j - 1]) ? 1u : 0u;
}

// Distinct levels with the row of their first appearance. The sort is
// stable and rows entered in increasing order, so a run's first entry holds
// the smallest row.
__global__ void level_distinct_kernel(const uint32_t* __restrict__ head, const uint32_t* __restrict__ hpos,
                                      const uint32_t* __restrict__ skey, const int32_t* __restrict__ srow, long long m,
                                      uint32_t* __restrict__ first_row, int32_t* __restrict__ level) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; j < m; j += st) {
        if (head[j]) {
            first_row[hpos[j]] = (uint32_t)srow[j];
            level[hpos[j]] = (int32_t)(skey[j] ^ 0x80000000u);
        }
    }
}

constexpr int DESIGN_COLS_PER_BLOCK = 16;

// Order-preserving unsigned key of a double: -0 just below +0, NaNs beyond
// the infinities, so an interval test on doubles becomes two integer
// compares (no FP64 instruction, the slow pipe on this part).
__device__ __forceinline__ unsigned long long order_key(double d) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Keys [lo, hi) of the values that round (half away from zero, as Fortran
// nint) to the level L: [L - 0.5, L + 0.5) for L > 0, (L - 0.5, L + 0.5] for
// L < 0, (-0.5, 0.5) for L = 0; L +- 0.5 are exact doubles.
__device__ __forceinline__ void level_interval(int L, unsigned long long& lo, unsigned long long& hi) {
    const unsigned long long kl = order_key((double)L - 0.5), kh = order_key((double)L + 0.5);
    lo = L > 0 ? kl : kl + 1;
    hi = L < 0 ? kh + 1 : kh;
}

struct DesignRecipe {
    fegb_design_column col;
    unsigned long long lo[FEGB_DESIGN_MAX_FACTORS], hi[FEGB_DESIGN_MAX_FACTORS];
};

// out[c * ld + i] = prod_f factor_f(i) for the columns of this block's column
// chunk; factors multiply left to right as in the reference. A dummy factor
// is 1.0 when the value rounds to its level: an integer interval test on the
// value's order key. A product of dummies is 1.0 or 0.0 with no FP64
// multiply (1 x 1, 1 x 0, 0 x 0 are exact); a continuous value still
// multiplies in FP64, so the result keeps its bits (signed zeros, NaN).
__global__ void __launch_bounds__(256) build_design_kernel(const double* const* __restrict__ src,
                                                           const fegb_design_column* __restrict__ cols, int n_cols,
                                                           long long n, double* __restrict__ out, long long ld) {
    __shared__ DesignRecipe sc[DESIGN_COLS_PER_BLOCK];
    const int c0 = blockIdx.y * DESIGN_COLS_PER_BLOCK;
    const int nc = min(DESIGN_COLS_PER_BLOCK, n_cols - c0);
    if (threadIdx.x < nc) {
        DesignRecipe& r = sc[threadIdx.x];
        r.col = cols[c0 + threadIdx.x];
        for (int f = 0; f < r.col.n_factors; ++f) level_interval(r.col.factors[f].level, r.lo[f], r.hi[f]);
    }
    __syncthreads();
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        for (int c = 0; c < nc; ++c) {
            const DesignRecipe& r = sc[c];
            double v = 0.0;
            bool dummies = true;  // v is the product of dummy factors so far: 1.0 iff hit
            bool hit = true;
            for (int f = 0; f < r.col.n_factors; ++f) {
                const fegb_design_factor& fa = r.col.factors[f];
                const double x = __ldg(src[fa.src] + i);
                if (fa.is_dummy) {
                    const unsigned long long k = order_key(x);
                    const bool in = k >= r.lo[f] && k < r.hi[f];
                    if (dummies) {
                        hit = hit && in;
                        v = hit ? 1.0 : 0.0;
                    } else {
                        v = v * (in ? 1.0 : 0.0);
                    }
                } else {
                    v = (f == 0) ? x : v * x;
                    dummies = false;
                }
            }
            out[(long long)(c0 + c) * ld + i] = v;
        }
    }
}

}  // namespace

int design_levels(const double* col, long long n, int max_levels, int* levels, int* n_levels, cudaStream_t s) {
    *n_levels = 0;
    if (n <= 0 || max_levels <= 0) return set_ok();
    Scratch scr(s);
    uint32_t *flag = nullptr, *pos = nullptr, *key = nullptr, *ckey = nullptr, *skey = nullptr;
    int32_t *crow = nullptr, *srow = nullptr;
    uint32_t* total = nullptr;
    FEGB_TRY(scr.alloc(&flag, (size_t)n, "level flags"));
    FEGB_TRY(scr.alloc(&pos, (size_t)n, "level positions"));
    FEGB_TRY(scr.alloc(&key, (size_t)n, "level keys"));
    FEGB_TRY(scr.alloc(&total, 1, "level count"));
    level_flags_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(col, n, flag, key);
    FEGB_LAUNCH_CHECK("level flags");
    FEGB_TRY(scan_exclusive_u32(flag, pos, n, total, s, scr));
    uint32_t m32 = 0;
    FEGB_CUDA(cudaMemcpyAsync(&m32, total, sizeof(m32), cudaMemcpyDeviceToHost, s), "level count copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "level count sync");
    const long long m = m32;
    if (m == 0) return set_ok();
    FEGB_TRY(scr.alloc(&ckey, (size_t)m, "level compact keys"));
    FEGB_TRY(scr.alloc(&crow, (size_t)m, "level compact rows"));
    FEGB_TRY(scr.alloc(&skey, (size_t)m, "level sorted keys"));
    FEGB_TRY(scr.alloc(&srow, (size_t)m, "level sorted rows"));
    level_compact_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(flag, pos, key, n, ckey, crow);
    FEGB_LAUNCH_CHECK("level compact");
    FEGB_TRY(radix_sort_u32(ckey, crow, skey, srow, m, 32, s, scr));
    // distinct levels: reuse flag/pos as run heads and their positions
    level_heads_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(skey, m, flag);
    FEGB_LAUNCH_CHECK("level heads");
    FEGB_TRY(scan_exclusive_u32(flag, pos, m, total, s, scr));
    uint32_t d32 = 0;
    FEGB_CUDA(cudaMemcpyAsync(&d32, total, sizeof(d32), cudaMemcpyDeviceToHost, s), "distinct count copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "distinct count sync");
    const long long D = d32;
    uint32_t *first_row = nullptr, *sfirst = nullptr;
    int32_t *lvl = nullptr, *slvl = nullptr;
    FEGB_TRY(scr.alloc(&first_row, (size_t)D, "level first rows"));
    FEGB_TRY(scr.alloc(&lvl, (size_t)D, "levels"));
    FEGB_TRY(scr.alloc(&sfirst, (size_t)D, "levels by appearance (rows)"));
    FEGB_TRY(scr.alloc(&slvl, (size_t)D, "levels by appearance"));
    level_distinct_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(flag, pos, skey, srow, m, first_row, lvl);
    FEGB_LAUNCH_CHECK("level distinct");
    // order the distinct levels by first appearance and keep the first max_levels
    FEGB_TRY(radix_sort_u32(first_row, lvl, sfirst, slvl, D, bits_for((unsigned long long)n), s, scr));
    const int keep = (int)std::min<long long>(D, max_levels);
    std::vector<int32_t> h(keep);
    FEGB_CUDA(cudaMemcpyAsync(h.data(), slvl, sizeof(int32_t) * keep, cudaMemcpyDeviceToHost, s), "levels copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "levels sync");
    std::sort(h.begin(), h.end());
    for (int i = 0; i < keep; ++i) levels[i] = h[i];
    *n_levels = keep;
    return set_ok();
}

int build_design(const double* const* src, int n_src, long long n, const fegb_design_column* cols, int n_cols,
                 double* out, long long ld, cudaStream_t s) {
    if (n_cols <= 0 || n <= 0) return set_ok();
    if (!src || !cols || !out) return set_error("build_design: null argument");
    if (ld < n) return set_error("build_design: leading dimension %lld < n %lld", ld, n);
    for (int c = 0; c < n_cols; ++c) {
        const fegb_design_column& col = cols[c];
        if (col.n_factors < 1 || col.n_factors > FEGB_DESIGN_MAX_FACTORS)
            return set_error("build_design: column %d has %d factors", c, col.n_factors);
        for (int f = 0; f < col.n_factors; ++f)
            if (col.factors[f].src < 0 || col.factors[f].src >= n_src)
                return set_error("build_design: column %d factor %d reads source %d of %d", c, f,
                                 col.factors[f].src, n_src);
    }
    for (int j = 0; j < n_src; ++j)
        if (!src[j]) return set_error("build_design: source column %d is null", j);
    Scratch scr(s);
    const double** d_src = nullptr;
    fegb_design_column* d_cols = nullptr;
    FEGB_TRY(scr.alloc(&d_src, (size_t)n_src, "design sources"));
    FEGB_TRY(scr.alloc(&d_cols, (size_t)n_cols, "design columns"));
    FEGB_CUDA(cudaMemcpyAsync(d_src, src, sizeof(double*) * n_src, cudaMemcpyHostToDevice, s), "design sources copy");
    FEGB_CUDA(cudaMemcpyAsync(d_cols, cols, sizeof(fegb_design_column) * n_cols, cudaMemcpyHostToDevice, s),
              "design columns copy");
    const unsigned gy = (unsigned)((n_cols + DESIGN_COLS_PER_BLOCK - 1) / DESIGN_COLS_PER_BLOCK);
    // about eight resident blocks per SM over all column chunks; rows are grid-strided
    const unsigned gx = (unsigned)std::min<long long>((n + 255) / 256, std::max(1, num_sms() * 8 / (int)gy));
    build_design_kernel<<<dim3(gx, gy), 256, 0, s>>>(d_src, d_cols, n_cols, n, out, ld);
    FEGB_LAUNCH_CHECK("design columns");
    // the host arrays above stay valid until the copies complete
    FEGB_CUDA(cudaStreamSynchronize(s), "design sync");
    return set_ok();
}

}  // namespace fegb

extern "C" int fegb_design_levels(const double* d_col, long long n, int max_levels, int* levels, int* n_levels,
                                  void* stream) {
    if (!levels || !n_levels) return fegb::set_error("fegb_design_levels: null output");
    if (n < 0) return fegb::set_error("fegb_design_levels: n < 0");
    if (n > 0 && !d_col) return fegb::set_error("fegb_design_levels: null column");
    if (n > INT_MAX) return fegb::set_error("fegb_design_levels: n exceeds the int32 row range");
    return fegb::design_levels(d_col, n, max_levels, levels, n_levels, (cudaStream_t)stream);
}

extern "C" int fegb_build_design(const double* const* d_src, int n_src, long long n, const fegb_design_column* cols,
                                 int n_cols, double* d_out, long long ld_out, void* stream) {
    return fegb::build_design(d_src, n_src, n, cols, n_cols, d_out, ld_out, (cudaStream_t)stream);
}
