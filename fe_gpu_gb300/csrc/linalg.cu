// Tall-skinny reductions and small dense kernels (see linalg.cuh).
#include "linalg.cuh"
#include "linalg_dev.cuh"

#include <algorithm>
#include <cmath>
#include <mutex>

namespace fegb {

namespace {

constexpr int CP_THREADS = 256;
constexpr int CP_TR = 16;
constexpr int CP_MAXPAIRS_LAUNCH = 8192;

struct CPParams {
    const double* A;
    long long ars, acs;
    int a;
    const double* B;
    long long brs, bcs;
    int b;
    long long n;
    int gram;
    long long p0;      // first pair index of this launch
    int npairs;        // pairs in this launch
    int phases;        // row phases (PPT == 1 mode)
    long long rows_per_block;
    double* partials;  // nblocks x npairs
};

__device__ __forceinline__ void pair_ij(long long p, int gram, int a, int& i, int& j) {
    if (gram) {
        int jj = (int)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
        while ((long long)(jj + 1) * (jj + 2) / 2 <= p) ++jj;
        while ((long long)jj * (jj + 1) / 2 > p) --jj;
        j = jj;
        i = (int)(p - (long long)jj * (jj + 1) / 2);
    } else {
        i = (int)(p % a);
        j = (int)(p / a);
    }
}

__device__ __forceinline__ void load_tile(double* dst, const double* src, long long rs, long long cs, int width,
                                          long long row0, int rows) {
    const int total = rows * width;
    if (rs == 1) {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            int r = e % rows, c = e / rows;
            dst[r * width + c] = src[(row0 + r) + (long long)c * cs];
        }
    } else {
        for (int e = threadIdx.x; e < total; e += blockDim.x) {
            int r = e / width, c = e % width;
            dst[r * width + c] = src[(row0 + r) * rs + (long long)c * cs];
        }
    }
}

template <int PPT>
__global__ void __launch_bounds__(CP_THREADS) crossprod_kernel(CPParams p) {
    extern __shared__ double sm[];
    double* sA = sm;
    double* sB = p.gram ? sm : sm + CP_TR * p.a;
    const int t = threadIdx.x;
    int pi[PPT], pj[PPT];
    bool pv[PPT];
    double acc[PPT];
    int phase = 0;
    if (PPT == 1) {
        int local = t % p.npairs;
        phase = t / p.npairs;
        pv[0] = phase < p.phases;
        pair_ij(p.p0 + local, p.gram, p.a, pi[0], pj[0]);
        acc[0] = 0.0;
    } else {
#pragma unroll
        for (int s = 0; s < PPT; ++s) {
            int local = t + s * CP_THREADS;
            pv[s] = local < p.npairs;
            pair_ij(p.p0 + (pv[s] ? local : 0), p.gram, p.a, pi[s], pj[s]);
            acc[s] = 0.0;
        }
    }
    const long long r0 = (long long)blockIdx.x * p.rows_per_block;
    const long long r1 = min(p.n, r0 + p.rows_per_block);
    for (long long tile = r0; tile < r1; tile += CP_TR) {
        const int rows = (int)min((long long)CP_TR, r1 - tile);
        load_tile(sA, p.A, p.ars, p.acs, p.a, tile, rows);
        if (!p.gram) load_tile(sB, p.B, p.brs, p.bcs, p.b, tile, rows);
        __syncthreads();
        if (PPT == 1) {
            if (pv[0])
                for (int r = phase; r < rows; r += p.phases) acc[0] += sA[r * p.a + pi[0]] * sB[r * p.b + pj[0]];
        } else {
            for (int r = 0; r < rows; ++r) {
#pragma unroll
                for (int s = 0; s < PPT; ++s)
                    if (pv[s]) acc[s] += sA[r * p.a + pi[s]] * sB[r * p.b + pj[s]];
            }
        }
        __syncthreads();
    }
    if (PPT == 1) {
        // fold row phases in a fixed order
        __shared__ double fold[CP_THREADS];
        fold[t] = pv[0] ? acc[0] : 0.0;
        __syncthreads();
        if (t < p.npairs) {
            double v = 0.0;
            for (int ph = 0; ph < p.phases; ++ph) v += fold[ph * p.npairs + t];
            p.partials[(long long)blockIdx.x * p.npairs + t] = v;
        }
    } else {
#pragma unroll
        for (int s = 0; s < PPT; ++s)
            if (pv[s]) p.partials[(long long)blockIdx.x * p.npairs + t + s * CP_THREADS] = acc[s];
    }
}

// One warp per output entry: lanes take the row blocks b = lane, lane + 32, ...
// in order, then a fixed shuffle tree.
__global__ void crossprod_reduce_kernel(const double* __restrict__ partials, int nblocks, int npairs, long long p0,
                                        int gram, int upper_only, int a, double alpha, double beta, double* out,
                                        int ldo) {
    const long long t = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (t >= npairs) return;
    double v = 0.0;
    for (int b = lane; b < nblocks; b += 32) v += partials[(long long)b * npairs + t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane != 0) return;
    int i, j;
    pair_ij(p0 + t, gram, a, i, j);
    double* o = out + i + (long long)j * ldo;
    *o = alpha * v + (beta != 0.0 ? beta * (*o) : 0.0);
    if (gram && !upper_only && i != j) {
        double* o2 = out + j + (long long)i * ldo;
        *o2 = alpha * v + (beta != 0.0 ? beta * (*o2) : 0.0);
    }
}

inline unsigned reduce_blocks(long long npairs) { return (unsigned)((npairs * 32 + 255) / 256); }

constexpr int RS_THREADS = 256;

__global__ void __launch_bounds__(RS_THREADS)
    residual_scores_kernel(const double* __restrict__ X, int C, long long n, const double* __restrict__ beta, int k,
                           const int* __restrict__ score_cols, int n_score, double* __restrict__ S,
                           double* __restrict__ resid, double* __restrict__ partials) {
    __shared__ double red[RS_THREADS / 32];
    double local = 0.0;
    long long i = (long long)blockIdx.x * RS_THREADS + threadIdx.x;
    const long long stride = (long long)gridDim.x * RS_THREADS;
    for (; i < n; i += stride) {
        const double* row = X + i * C;
        double r = row[0];
        for (int j = 0; j < k; ++j) r -= row[1 + j] * beta[j];
        if (resid) resid[i] = r;
        if (S)
            for (int t = 0; t < n_score; ++t) S[i * n_score + t] = r * row[score_cols[t]];
        local += r * r;
    }
    // fixed-shape tree: warp then block
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < RS_THREADS / 32; ++w) v += red[w];
        partials[blockIdx.x] = v;
    }
}

// The same for wide rows (many regressors): one warp per row, lanes over the
// columns, so that reads of X and writes of S are contiguous runs (a thread
// per row made every load and store instruction touch 32 rows); the lanes'
// partial products are summed by a fixed xor tree.
__global__ void __launch_bounds__(RS_THREADS)
    residual_scores_wide_kernel(const double* __restrict__ X, int C, long long n, const double* __restrict__ beta,
                                int k, const int* __restrict__ score_cols, int n_score, double* __restrict__ S,
                                double* __restrict__ resid, double* __restrict__ partials) {
    __shared__ double red[RS_THREADS / 32];
    const int lane = threadIdx.x & 31;
    double local = 0.0;
    long long i = ((long long)blockIdx.x * RS_THREADS + threadIdx.x) >> 5;
    const long long stride = ((long long)gridDim.x * RS_THREADS) >> 5;
    for (; i < n; i += stride) {
        const double* row = X + i * C;
        double dot = 0.0;
        for (int j = lane; j < k; j += 32) dot += row[1 + j] * beta[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) dot += __shfl_xor_sync(0xffffffffu, dot, o);
        const double r = row[0] - dot;
        if (resid && lane == 0) resid[i] = r;
        if (S)
            for (int t = lane; t < n_score; t += 32) S[i * n_score + t] = r * row[score_cols[t]];
        if (lane == 0) local += r * r;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
    if (lane == 0) red[threadIdx.x >> 5] = local;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < RS_THREADS / 32; ++w) v += red[w];
        partials[blockIdx.x] = v;
    }
}

__global__ void sum_partials_kernel(const double* __restrict__ partials, int nb, double* out) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double v = 0.0;
        for (int b = 0; b < nb; ++b) v += partials[b];
        *out = v;
    }
}

// ---------------------------- dense kernels ------------------------------


__global__ void __launch_bounds__(DN_THREADS)
    chol_solve_inv_kernel(int k, const double* __restrict__ Q, int ldq, const int* __restrict__ idx,
                          const double* __restrict__ b, double* __restrict__ beta, double* __restrict__ Qinv,
                          int* __restrict__ info, double* __restrict__ work) {
    chol_solve_inv_block(k, Q, ldq, idx, b, beta, Qinv, info, work);
}

__global__ void gemm_small_kernel(int ta, int tb, int m, int n, int k, double alpha, const double* __restrict__ A,
                                  int lda, const double* __restrict__ B, int ldb, double beta, double* __restrict__ C,
                                  int ldc) {
    long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)m * n) return;
    int i = (int)(e % m), j = (int)(e / m);
    double s = 0.0;
    for (int p = 0; p < k; ++p) {
        double av = ta ? A[p + (long long)i * lda] : A[i + (long long)p * lda];
        double bv = tb ? B[j + (long long)p * ldb] : B[p + (long long)j * ldb];
        s += av * bv;
    }
    double* o = C + i + (long long)j * ldc;
    *o = alpha * s + (beta != 0.0 ? beta * (*o) : 0.0);
}

__global__ void select_kernel(int k, const double* __restrict__ M, int ldm, const int* __restrict__ idx,
                              double* __restrict__ out) {
    int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= k * k) return;
    int i = e % k, j = e / k;
    int mi = idx ? idx[i] : i, mj = idx ? idx[j] : j;
    out[e] = M[mi + (long long)mj * ldm];
}

__global__ void __launch_bounds__(DN_THREADS)
    finalize_cov_kernel(int k, double* __restrict__ acc, double scalar, int do_psd, double* __restrict__ se,
                        int* __restrict__ psd_applied, double* __restrict__ work) {
    finalize_cov_block(k, acc, scalar, do_psd, se, psd_applied, work);
}

}  // namespace

int crossprod(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha, double beta,
              double* out, int ldo, cudaStream_t s, Scratch& scr) {
    const int a = A.cols, b = gram ? A.cols : B.cols;
    if (a <= 0 || b <= 0) return 0;
    const long long total_pairs = gram ? (long long)a * (a + 1) / 2 : (long long)a * b;
    if (n <= 0) {
        // A^T B over zero rows is the zero matrix
        for (long long p0 = 0; p0 < total_pairs; p0 += CP_MAXPAIRS_LAUNCH) {
            int np = (int)std::min<long long>(CP_MAXPAIRS_LAUNCH, total_pairs - p0);
            double* zeros = nullptr;
            FEGB_TRY(scr.alloc(&zeros, (size_t)np, "crossprod zeros"));
            FEGB_CUDA(cudaMemsetAsync(zeros, 0, sizeof(double) * np, s), "crossprod zero");
            crossprod_reduce_kernel<<<reduce_blocks(np), 256, 0, s>>>(zeros, 1, np, p0, gram, upper_only, a, alpha,
                                                                      beta, out, ldo);
            FEGB_LAUNCH_CHECK("crossprod zero reduce");
        }
        return 0;
    }
    long long nb = std::min<long long>((n + CP_TR - 1) / CP_TR, (long long)num_sms() * 4);
    long long rpb = (n + nb - 1) / nb;
    rpb = ((rpb + CP_TR - 1) / CP_TR) * CP_TR;
    nb = (n + rpb - 1) / rpb;
    size_t smem = sizeof(double) * CP_TR * (gram ? a : a + b);
    if (smem > 200 * 1024) return set_error("crossprod: %d x %d columns exceed the shared-memory tile", a, b);
    // set once (thread-safe static initialisation) before any launch with a large tile
    static const cudaError_t attr_status = []() {
        cudaError_t e = cudaSuccess;
        const int lim = 200 * 1024;
        if (e == cudaSuccess) e = cudaFuncSetAttribute(crossprod_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(crossprod_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (e == cudaSuccess) e = cudaFuncSetAttribute(crossprod_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(crossprod_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(crossprod_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, lim);
        return e;
    }();
    if (attr_status != cudaSuccess) return set_cuda_error(attr_status, "crossprod attr");
    for (long long p0 = 0; p0 < total_pairs; p0 += CP_MAXPAIRS_LAUNCH) {
        const int np = (int)std::min<long long>(CP_MAXPAIRS_LAUNCH, total_pairs - p0);
        double* partials = nullptr;
        FEGB_TRY(scr.alloc(&partials, (size_t)nb * np, "crossprod partials"));
        CPParams p;
        p.A = A.ptr;
        p.ars = A.rs;
        p.acs = A.cs;
        p.a = a;
        p.B = gram ? A.ptr : B.ptr;
        p.brs = gram ? A.rs : B.rs;
        p.bcs = gram ? A.cs : B.cs;
        p.b = b;
        p.n = n;
        p.gram = gram ? 1 : 0;
        p.p0 = p0;
        p.npairs = np;
        p.phases = np <= 128 ? CP_THREADS / np : 1;
        p.rows_per_block = rpb;
        p.partials = partials;
        if (np <= 128)
            crossprod_kernel<1><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        else if (np <= 4 * CP_THREADS)
            crossprod_kernel<4><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        else if (np <= 8 * CP_THREADS)
            crossprod_kernel<8><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        else if (np <= 16 * CP_THREADS)
            crossprod_kernel<16><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        else
            crossprod_kernel<32><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        FEGB_LAUNCH_CHECK("crossprod");
        crossprod_reduce_kernel<<<reduce_blocks(np), 256, 0, s>>>(partials, (int)nb, np, p0, gram, upper_only, a, alpha,
                                                                  beta, out, ldo);
        FEGB_LAUNCH_CHECK("crossprod reduce");
    }
    return 0;
}

// ------------------------- split-FP32 cross products -------------------------

namespace {

constexpr int DS_TR_MAX = 256;  // rows per shared-memory tile (and per FP64 fold), at most
constexpr int DS_SMEM = 48 * 1024;  // tile bytes aimed at (several blocks per SM)
constexpr int DS_PPT = 4;       // output entries per thread
constexpr int DS_PAIRS_PER_BLOCK = CP_THREADS * DS_PPT;

// The split path accepts magnitudes below 2^57: products and 256-row partial
// sums then stay inside the FP32 range (2^127); see split_bits for the small end.

struct DSParams {
    const double* A;  // FP64 source, element (r, c) at A[r * ars + c * acs]
    long long ars, acs;
    int a;
    const double* B;  // == A for a Gram
    long long brs, bcs;
    int b;
    long long n;
    int gram;
    long long p0;     // first pair of this launch
    int npairs;
    int phases;       // row phases (PPT == 1)
    long long rows_per_block;
    int tr;            // rows per tile
    double* partials;  // row blocks x npairs
    int* bad;          // set when a value is outside the split range (split_bits)
};

// The cross products split values below 2^57 (split_f64): a product and its
// 256-row partial sums stay inside the FP32 range. Outside it (and for
// non-finite values) bad is set and the product is formed in FP64 instead.
__device__ __forceinline__ float2 split_bits(double v, bool& bad) { return split_f64<56>(v, bad); }

// Tile rows [row0, row0 + rows) of an FP64 source into shared memory as
// (hi, lo) FP32 pairs: hi = fl32(x), lo = fl32(x - hi) (x - hi is exact in FP64).
__device__ __forceinline__ bool load_split_tile(float2* dst, const double* src, long long rs, long long cs, int width,
                                                long long row0, int rows) {
    const int total = rows * width;
    bool out_of_range = false;
    for (int e = threadIdx.x; e < total; e += blockDim.x) {
        int r, c;
        if (rs == 1) {  // column-major source: consecutive threads walk rows
            r = e % rows;
            c = e / rows;
        } else {
            r = e / width;
            c = e - r * width;
        }
        dst[r * width + c] = split_bits(src[(row0 + r) * rs + (long long)c * cs], out_of_range);
    }
    return out_of_range;
}

// PPT output entries per thread; PPT == 1: few pairs, the threads of a block
// split each tile's rows into p.phases row phases (folded in a fixed order).
// Each tile's double-single sums are folded into FP64 accumulators.
template <int PPT>
__global__ void __launch_bounds__(CP_THREADS) crossprod_split_kernel(DSParams p) {
    extern __shared__ float2 dsm[];
    float2* sA = dsm;
    float2* sB = p.gram ? dsm : dsm + p.tr * p.a;
    const int t = threadIdx.x;
    const int chunk0 = PPT == 1 ? 0 : blockIdx.y * CP_THREADS * PPT;
    int pi[PPT], pj[PPT];
    bool pv[PPT];
    double acc[PPT];
    int phase = 0;
    if (PPT == 1) {
        const int local = t % p.npairs;
        phase = t / p.npairs;
        pv[0] = phase < p.phases;
        pair_ij(p.p0 + local, p.gram, p.a, pi[0], pj[0]);
        acc[0] = 0.0;
    } else {
#pragma unroll
        for (int s = 0; s < PPT; ++s) {
            const int local = chunk0 + t + s * CP_THREADS;
            pv[s] = local < p.npairs;
            pair_ij(p.p0 + (pv[s] ? local : 0), p.gram, p.a, pi[s], pj[s]);
            acc[s] = 0.0;
        }
    }
    bool bad = false;
    const long long r0 = (long long)blockIdx.x * p.rows_per_block;
    const long long r1 = min(p.n, r0 + p.rows_per_block);
    for (long long tile = r0; tile < r1; tile += p.tr) {
        const int rows = (int)min((long long)p.tr, r1 - tile);
        bad |= load_split_tile(sA, p.A, p.ars, p.acs, p.a, tile, rows);
        if (!p.gram) bad |= load_split_tile(sB, p.B, p.brs, p.bcs, p.b, tile, rows);
        __syncthreads();
        if (PPT == 1) {
            if (pv[0]) {
                float sh = 0.f, sl = 0.f;
                for (int r = phase; r < rows; r += p.phases) ds_fma(sA[r * p.a + pi[0]], sB[r * p.b + pj[0]], sh, sl);
                acc[0] += (double)sh + (double)sl;
            }
        } else {
            float sh[PPT], sl[PPT];
#pragma unroll
            for (int s = 0; s < PPT; ++s) sh[s] = sl[s] = 0.f;
            for (int r = 0; r < rows; ++r) {
#pragma unroll
                for (int s = 0; s < PPT; ++s)
                    if (pv[s]) ds_fma(sA[r * p.a + pi[s]], sB[r * p.b + pj[s]], sh[s], sl[s]);
            }
#pragma unroll
            for (int s = 0; s < PPT; ++s) acc[s] += (double)sh[s] + (double)sl[s];
        }
        __syncthreads();
    }
    if (__any_sync(0xffffffffu, bad) && (t & 31) == 0) atomicOr(p.bad, 1);
    if (PPT == 1) {
        __shared__ double fold[CP_THREADS];
        fold[t] = pv[0] ? acc[0] : 0.0;
        __syncthreads();
        if (t < p.npairs) {
            double v = 0.0;
            for (int ph = 0; ph < p.phases; ++ph) v += fold[ph * p.npairs + t];
            p.partials[(long long)blockIdx.x * p.npairs + t] = v;
        }
    } else {
#pragma unroll
        for (int s = 0; s < PPT; ++s)
            if (pv[s]) p.partials[(long long)blockIdx.x * p.npairs + chunk0 + t + s * CP_THREADS] = acc[s];
    }
}

// Wide Gram products (more than DS_ROWS_MAX_A columns): thread q of the grid's
// y range owns the 4 x 4 block (bi, bj), bi <= bj, of output entries
// (4 bi + ii, 4 bj + jj), so per tile row it reads 4 + 4 split values from
// shared memory (two 32-byte runs) for 16 double-single products, four
// times fewer shared-memory reads per product than one pair per thread, whose
// kernel the wide Grams saturated shared memory with. Columns past a are zero
// in the tile; entries with i > j or past a are not written. The
// double-single sums span DSB_FOLD rows (DSB_FOLD / DSB_TR tiles) and are then
// folded into FP64 sums kept in shared memory, so that a thread holds only
// its 32 FP32 sums in registers and three blocks fit on an SM.
constexpr int DSB_TR = 32;    // rows per tile
constexpr int DSB_FOLD = 128; // rows per double-single sum

__device__ __forceinline__ void pair_block(int q, int& bi, int& bj) {
    int jj = (int)((sqrt(8.0 * (double)q + 1.0) - 1.0) * 0.5);
    while ((jj + 1) * (jj + 2) / 2 <= q) ++jj;
    while (jj * (jj + 1) / 2 > q) --jj;
    bj = jj;
    bi = q - jj * (jj + 1) / 2;
}

__global__ void __launch_bounds__(CP_THREADS, 3)
    crossprod_split_blocked_kernel(const double* __restrict__ A, long long rs, long long cs, int a, long long n,
                                   long long rows_per_block, double* __restrict__ partials, int* __restrict__ bad) {
    extern __shared__ float4 dsb[];
    const int a4 = (a + 3) / 4 * 4;
    double* acc = reinterpret_cast<double*>(dsb);                                  // [16][CP_THREADS]
    float2* tile = reinterpret_cast<float2*>(acc + 16 * CP_THREADS);                // [DSB_TR][a4]
    const int nbk = a4 / 4;
    const int nbp = nbk * (nbk + 1) / 2;
    const int q = blockIdx.y * CP_THREADS + threadIdx.x;
    const bool active = q < nbp;
    int bi = 0, bj = 0;
    if (active) pair_block(q, bi, bj);
#pragma unroll
    for (int e = 0; e < 16; ++e) acc[e * CP_THREADS + threadIdx.x] = 0.0;
    float sh[16], sl[16];
#pragma unroll
    for (int e = 0; e < 16; ++e) sh[e] = sl[e] = 0.f;
    bool oor = false;
    const long long r0 = (long long)blockIdx.x * rows_per_block;
    const long long r1 = min(n, r0 + rows_per_block);
    int since_fold = 0;
    for (long long t0 = r0; t0 < r1; t0 += DSB_TR) {
        const int rows = (int)min((long long)DSB_TR, r1 - t0);
        for (int e = threadIdx.x; e < DSB_TR * a4; e += CP_THREADS) {
            int r, c;
            if (rs == 1) {  // column-major source: consecutive threads walk rows
                r = e % DSB_TR;
                c = e / DSB_TR;
            } else {
                r = e / a4;
                c = e - r * a4;
            }
            tile[r * a4 + c] = (r < rows && c < a) ? split_bits(A[(t0 + r) * rs + (long long)c * cs], oor)
                                                   : make_float2(0.f, 0.f);
        }
        __syncthreads();
        if (active) {
            const float4* row = reinterpret_cast<const float4*>(tile);
            for (int r = 0; r < rows; ++r) {
                const float4 i01 = row[(r * a4 + 4 * bi) / 2], i23 = row[(r * a4 + 4 * bi) / 2 + 1];
                const float4 j01 = row[(r * a4 + 4 * bj) / 2], j23 = row[(r * a4 + 4 * bj) / 2 + 1];
                const float2 xi[4] = {make_float2(i01.x, i01.y), make_float2(i01.z, i01.w), make_float2(i23.x, i23.y),
                                      make_float2(i23.z, i23.w)};
                const float2 xj[4] = {make_float2(j01.x, j01.y), make_float2(j01.z, j01.w), make_float2(j23.x, j23.y),
                                      make_float2(j23.z, j23.w)};
#pragma unroll
                for (int ii = 0; ii < 4; ++ii)
#pragma unroll
                    for (int jj = 0; jj < 4; ++jj) ds_fma(xi[ii], xj[jj], sh[ii * 4 + jj], sl[ii * 4 + jj]);
            }
            since_fold += DSB_TR;
            if (since_fold >= DSB_FOLD || t0 + DSB_TR >= r1) {
#pragma unroll
                for (int e = 0; e < 16; ++e) {
                    acc[e * CP_THREADS + threadIdx.x] += (double)sh[e] + (double)sl[e];
                    sh[e] = sl[e] = 0.f;
                }
                since_fold = 0;
            }
        }
        __syncthreads();
    }
    if (__any_sync(0xffffffffu, oor) && (threadIdx.x & 31) == 0) atomicOr(bad, 1);
    if (!active) return;
    const long long np = (long long)a * (a + 1) / 2;
#pragma unroll
    for (int ii = 0; ii < 4; ++ii)
#pragma unroll
        for (int jj = 0; jj < 4; ++jj) {
            const int i = 4 * bi + ii, j = 4 * bj + jj;
            if (i <= j && j < a)
                partials[(long long)blockIdx.x * np + (long long)j * (j + 1) / 2 + i] =
                    acc[(ii * 4 + jj) * CP_THREADS + threadIdx.x];
        }
}

// Thin Gram products (A <= DS_ROWS_MAX_A columns): each row is handled by
// SPLIT threads (one per warp of a warp group), thread part q holding the
// pairs [q NPP, (q + 1) NPP) in registers as double-single sums; each thread
// sums at most DS_ROWS_PER_THREAD rows, so the FP32 parts stay in range. The
// threads' FP64 totals are reduced per block in a fixed order (warp shuffle
// tree, then the row groups in order). Pair p = j (j + 1) / 2 + i, i <= j.
constexpr int DS_ROWS_GROUPS = 2;        // row groups (of 32 rows) per block
constexpr int DS_ROWS_PER_THREAD = 64;
constexpr int DS_ROWS_MAX_A = 10;
constexpr int DSB_MAX_A = 640;  // widest Gram of the blocked kernel (its 32-row tile and sums: 192 KB of shared memory)

__host__ __device__ constexpr int ds_rows_split(int A) { return A * (A + 1) / 2 <= 16 ? 1 : (A * (A + 1) / 2 + 15) / 16; }

template <int A, int SPLIT, int PART>
__device__ __forceinline__ void split_rows_part(const double* __restrict__ X, long long rs, long long r0,
                                                long long r1, int lane, double (*red)[A * (A + 1) / 2], int rg,
                                                bool& oor) {
    constexpr int NP = A * (A + 1) / 2;
    constexpr int NPP = (NP + SPLIT - 1) / SPLIT;
    constexpr int LO = PART * NPP;
    constexpr int HI = (LO + NPP < NP) ? LO + NPP : NP;
    float sh[NPP], sl[NPP];
#pragma unroll
    for (int q = 0; q < NPP; ++q) sh[q] = sl[q] = 0.f;
    for (long long r = r0 + lane; r < r1; r += 32) {
        float2 x[A];
#pragma unroll
        for (int i = 0; i < A; ++i) x[i] = split_bits(X[r * rs + i], oor);
        int q = 0;
#pragma unroll
        for (int j = 0; j < A; ++j)
#pragma unroll
            for (int i = 0; i <= j; ++i, ++q)
                if (q >= LO && q < HI) ds_fma(x[i], x[j], sh[q - LO], sl[q - LO]);
    }
#pragma unroll
    for (int q = LO; q < HI; ++q) {
        double v = (double)sh[q - LO] + (double)sl[q - LO];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[rg][q] = v;
    }
}

template <int A, int SPLIT, int PART>
__device__ __forceinline__ void split_rows_select(int part, const double* X, long long rs, long long r0, long long r1,
                                                  int lane, double (*red)[A * (A + 1) / 2], int rg, bool& oor) {
    if constexpr (PART < SPLIT) {
        if (part == PART)
            split_rows_part<A, SPLIT, PART>(X, rs, r0, r1, lane, red, rg, oor);
        else
            split_rows_select<A, SPLIT, PART + 1>(part, X, rs, r0, r1, lane, red, rg, oor);
    }
}

template <int A>
__global__ void __launch_bounds__(32 * ds_rows_split(A) * DS_ROWS_GROUPS)
    crossprod_split_rows_kernel(const double* __restrict__ X, long long rs, long long n, double* __restrict__ partials,
                                int* __restrict__ bad) {
    constexpr int NP = A * (A + 1) / 2;
    constexpr int SPLIT = ds_rows_split(A);
    __shared__ double red[DS_ROWS_GROUPS][NP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int part = warp % SPLIT, rg = warp / SPLIT;
    const long long rows_rg = 32LL * DS_ROWS_PER_THREAD;
    const long long r0 = ((long long)blockIdx.x * DS_ROWS_GROUPS + rg) * rows_rg;
    const long long r1 = min(n, r0 + rows_rg);
    bool oor = false;
    split_rows_select<A, SPLIT, 0>(part, X, rs, r0, r1, lane, red, rg, oor);
    if (__any_sync(0xffffffffu, oor) && lane == 0) atomicOr(bad, 1);
    __syncthreads();
    for (int q = threadIdx.x; q < NP; q += blockDim.x) {
        double v = 0.0;
        for (int g = 0; g < DS_ROWS_GROUPS; ++g) v += red[g][q];
        partials[(long long)blockIdx.x * NP + q] = v;
    }
}

template <int A>
int split_rows_launch(const double* X, long long rs, long long n, double* partials, int* bad, int nb, cudaStream_t s) {
    crossprod_split_rows_kernel<A><<<nb, 32 * ds_rows_split(A) * DS_ROWS_GROUPS, 0, s>>>(X, rs, n, partials, bad);
    FEGB_LAUNCH_CHECK("split crossprod (rows)");
    return 0;
}

int split_rows_dispatch(int a, const double* X, long long rs, long long n, double* partials, int* bad, int nb,
                        cudaStream_t s) {
    switch (a) {
        case 2: return split_rows_launch<2>(X, rs, n, partials, bad, nb, s);
        case 3: return split_rows_launch<3>(X, rs, n, partials, bad, nb, s);
        case 4: return split_rows_launch<4>(X, rs, n, partials, bad, nb, s);
        case 5: return split_rows_launch<5>(X, rs, n, partials, bad, nb, s);
        case 6: return split_rows_launch<6>(X, rs, n, partials, bad, nb, s);
        case 7: return split_rows_launch<7>(X, rs, n, partials, bad, nb, s);
        case 8: return split_rows_launch<8>(X, rs, n, partials, bad, nb, s);
        case 9: return split_rows_launch<9>(X, rs, n, partials, bad, nb, s);
        case 10: return split_rows_launch<10>(X, rs, n, partials, bad, nb, s);
        default: return set_error("split crossprod (rows): %d columns", a);
    }
}

}  // namespace

int crossprod_split(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha,
                    double beta, double* out, int ldo, cudaStream_t s, Scratch& scr) {
    const int a = A.cols, b = gram ? A.cols : B.cols;
    if (a <= 0 || b <= 0) return 0;
    if (n <= 0) return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
    const int width = gram ? a : a + b;
    if (sizeof(float2) * 16 * (size_t)width > 200 * 1024)
        return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
    const int tr = std::max(16, std::min(DS_TR_MAX, (int)(DS_SMEM / (sizeof(float2) * width)) / 16 * 16));
    const size_t smem = sizeof(float2) * (size_t)tr * width;
    static const cudaError_t attr_status = []() {
        cudaError_t e = cudaFuncSetAttribute(crossprod_split_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(crossprod_split_kernel<DS_PPT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     200 * 1024);
        return e;
    }();
    if (attr_status != cudaSuccess) return set_cuda_error(attr_status, "split crossprod attr");
    int* bad = nullptr;
    FEGB_TRY(scr.alloc(&bad, 1, "split range flag"));
    FEGB_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), s), "split flag reset");
    const long long total_pairs = gram ? (long long)a * (a + 1) / 2 : (long long)a * b;
    if (gram && A.cs == 1 && A.rs >= a && a >= 2 && a <= DS_ROWS_MAX_A) {
        const long long rows_pb = 32LL * DS_ROWS_GROUPS * DS_ROWS_PER_THREAD;
        const long long nb = (n + rows_pb - 1) / rows_pb;
        if (nb > 0x7fffffffLL) return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
        double* partials = nullptr;
        FEGB_TRY(scr.alloc(&partials, (size_t)nb * total_pairs, "split crossprod partials"));
        FEGB_TRY(split_rows_dispatch(a, A.ptr, A.rs, n, partials, bad, (int)nb, s));
        crossprod_reduce_kernel<<<reduce_blocks(total_pairs), 256, 0, s>>>(
            partials, (int)nb, (int)total_pairs, 0, 1, upper_only, a, alpha, beta, out, ldo);
        FEGB_LAUNCH_CHECK("split crossprod reduce");
        int hbad = 0;
        FEGB_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s), "split flag copy");
        FEGB_CUDA(cudaStreamSynchronize(s), "split flag sync");
        if (hbad) return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
        return 0;
    }
    if (gram && a > DS_ROWS_MAX_A && a <= DSB_MAX_A) {
        const int a4 = (a + 3) / 4 * 4;
        const int nbp = (a4 / 4) * (a4 / 4 + 1) / 2;
        const int gy = (nbp + CP_THREADS - 1) / CP_THREADS;
        const size_t bsmem = sizeof(double) * 16 * CP_THREADS + sizeof(float2) * (size_t)DSB_TR * a4;
        static const cudaError_t battr = cudaFuncSetAttribute(
            crossprod_split_blocked_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        if (battr != cudaSuccess) return set_cuda_error(battr, "split crossprod (blocked) attr");
        long long nbr = std::min<long long>((n + DSB_TR - 1) / DSB_TR, std::max(1LL, (long long)num_sms() * 6 / gy));
        long long rpb = (n + nbr - 1) / nbr;
        rpb = ((rpb + DSB_TR - 1) / DSB_TR) * DSB_TR;
        nbr = (n + rpb - 1) / rpb;
        double* partials = nullptr;
        FEGB_TRY(scr.alloc(&partials, (size_t)nbr * total_pairs, "split crossprod partials"));
        crossprod_split_blocked_kernel<<<dim3((unsigned)nbr, (unsigned)gy), CP_THREADS, bsmem, s>>>(
            A.ptr, A.rs, A.cs, a, n, rpb, partials, bad);
        FEGB_LAUNCH_CHECK("split crossprod (blocked)");
        crossprod_reduce_kernel<<<reduce_blocks(total_pairs), 256, 0, s>>>(
            partials, (int)nbr, (int)total_pairs, 0, 1, upper_only, a, alpha, beta, out, ldo);
        FEGB_LAUNCH_CHECK("split crossprod reduce");
        int hbad = 0;
        FEGB_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s), "split flag copy");
        FEGB_CUDA(cudaStreamSynchronize(s), "split flag sync");
        if (hbad) return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
        return 0;
    }
    long long nb = std::min<long long>((n + tr - 1) / tr, (long long)num_sms() * 8);
    long long rpb = (n + nb - 1) / nb;
    rpb = ((rpb + tr - 1) / tr) * tr;
    nb = (n + rpb - 1) / rpb;
    for (long long p0 = 0; p0 < total_pairs; p0 += CP_MAXPAIRS_LAUNCH) {
        const int np = (int)std::min<long long>(CP_MAXPAIRS_LAUNCH, total_pairs - p0);
        double* partials = nullptr;
        FEGB_TRY(scr.alloc(&partials, (size_t)nb * np, "split crossprod partials"));
        DSParams p;
        p.A = A.ptr;
        p.ars = A.rs;
        p.acs = A.cs;
        p.a = a;
        p.B = gram ? A.ptr : B.ptr;
        p.brs = gram ? A.rs : B.rs;
        p.bcs = gram ? A.cs : B.cs;
        p.b = b;
        p.n = n;
        p.gram = gram ? 1 : 0;
        p.p0 = p0;
        p.npairs = np;
        p.phases = np <= 128 ? CP_THREADS / np : 1;
        p.rows_per_block = rpb;
        p.tr = tr;
        p.partials = partials;
        p.bad = bad;
        if (np <= 128) {
            crossprod_split_kernel<1><<<(unsigned)nb, CP_THREADS, smem, s>>>(p);
        } else {
            dim3 grid((unsigned)nb, (unsigned)((np + DS_PAIRS_PER_BLOCK - 1) / DS_PAIRS_PER_BLOCK));
            crossprod_split_kernel<DS_PPT><<<grid, CP_THREADS, smem, s>>>(p);
        }
        FEGB_LAUNCH_CHECK("split crossprod");
        crossprod_reduce_kernel<<<reduce_blocks(np), 256, 0, s>>>(partials, (int)nb, np, p0, gram, upper_only, a, alpha,
                                                                  beta, out, ldo);
        FEGB_LAUNCH_CHECK("split crossprod reduce");
    }
    int hbad = 0;
    FEGB_CUDA(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s), "split flag copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "split flag sync");
    // a value outside the split range: the whole product again in FP64
    if (hbad) return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
    return 0;
}

int crossprod_auto(const MatView& A, const MatView& B, long long n, bool gram, bool upper_only, double alpha,
                   double beta, double* out, int ldo, cudaStream_t s, Scratch& scr) {
    const long long pairs = gram ? (long long)A.cols * (A.cols + 1) / 2 : (long long)A.cols * B.cols;
    const long long cols = gram ? A.cols : (long long)A.cols + B.cols;
    if (pairs >= (long long)tuning(TUNE_SPLIT_GRAM) * cols && n >= 4096)
        return crossprod_split(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
    return crossprod(A, B, n, gram, upper_only, alpha, beta, out, ldo, s, scr);
}

int residual_scores(const double* X, int C, long long n, const double* beta, int k, const int* score_cols_dev,
                    int n_score, double* S, double* resid, double* rss_dev, cudaStream_t s, Scratch& scr) {
    int nb = (int)std::min<long long>((long long)num_sms() * 8, std::max(1LL, (n + RS_THREADS - 1) / RS_THREADS));
    double* partials = nullptr;
    FEGB_TRY(scr.alloc(&partials, (size_t)nb, "rss partials"));
    if (C >= 32)
        residual_scores_wide_kernel<<<nb, RS_THREADS, 0, s>>>(X, C, n, beta, k, score_cols_dev, n_score, S, resid,
                                                              partials);
    else
        residual_scores_kernel<<<nb, RS_THREADS, 0, s>>>(X, C, n, beta, k, score_cols_dev, n_score, S, resid,
                                                         partials);
    FEGB_LAUNCH_CHECK("residual/scores");
    sum_partials_kernel<<<1, 32, 0, s>>>(partials, nb, rss_dev);
    FEGB_LAUNCH_CHECK("rss sum");
    return 0;
}

int dense_chol_solve_inv(int k, const double* Q, int ldq, const int* idx_dev, const double* b, double* beta_out,
                         double* Qinv, int* info_dev, double* work, cudaStream_t s) {
    if (k <= 0) return 0;
    chol_solve_inv_kernel<<<1, DN_THREADS, 0, s>>>(k, Q, ldq, idx_dev, b, beta_out, Qinv, info_dev, work);
    FEGB_LAUNCH_CHECK("cholesky");
    return 0;
}

int dense_gemm(bool ta, bool tb, int m, int n, int k, double alpha, const double* A, int lda, const double* B, int ldb,
               double beta, double* C, int ldc, cudaStream_t s) {
    long long tot = (long long)m * n;
    if (tot <= 0) return 0;
    gemm_small_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, s>>>(ta, tb, m, n, k, alpha, A, lda, B, ldb, beta, C,
                                                                     ldc);
    FEGB_LAUNCH_CHECK("small gemm");
    return 0;
}

int dense_sandwich_acc(int k, const double* Qinv, const double* M, int ldm, const int* idx_dev, double w, double* acc,
                       double* work, cudaStream_t s) {
    if (k <= 0) return 0;
    double* Ms = work;
    double* T = work + (size_t)k * k;
    select_kernel<<<(k * k + 255) / 256, 256, 0, s>>>(k, M, ldm, idx_dev, Ms);
    FEGB_LAUNCH_CHECK("meat select");
    FEGB_TRY(dense_gemm(false, false, k, k, k, 1.0, Ms, k, Qinv, k, 0.0, T, k, s));
    FEGB_TRY(dense_gemm(false, false, k, k, k, w, Qinv, k, T, k, 1.0, acc, k, s));
    return 0;
}

int dense_finalize_cov(int k, double* acc, double scalar, int do_psd, double* se_out, int* psd_applied, double* work,
                       cudaStream_t s) {
    if (k <= 0) return 0;
    finalize_cov_kernel<<<1, DN_THREADS, 0, s>>>(k, acc, scalar, do_psd, se_out, psd_applied, work);
    FEGB_LAUNCH_CHECK("covariance finalize");
    return 0;
}

}  // namespace fegb

// ---------------------------------------------------------------------------
// Allocation-free cross product (fe_gpu_syrk_noalloc, include/fe_gpu_runtime.h).
//
// fe_gpu_syrk takes the per-block partial sums of its reduction from the
// stream-ordered memory pool. Some callers cannot let a library allocate
// device memory while they run: a host that owns every device buffer through
// its own allocator and budget, or code that must not touch the allocator
// at all in a latency-critical section. For them this variant keeps the
// partials in a fixed file-scope device array of
// NOALLOC_BLOCKS x NOALLOC_MAX_PAIRS doubles (152 x 528 x 8 B = 642 KB, held
// by every GPU that loads the library until the process exits), which bounds
// the input to at most NOALLOC_MAX_COLS = 32 columns.
//
// The device address of the array is looked up with cudaGetSymbolAddress by
// the first call made while a device is current, and cached with the identity
// of that device's CUDA context (cuCtxGetId). A later call in a new context
// (after cudaDeviceReset, or a primary context that was released and created
// again) finds a different identity and looks the address up again. Make the
// first call on each device, and the first after a reset, before capturing
// any stream. Every call shares the one array: calls whose kernels overlap on
// the GPU (other host threads, or other streams) race on it. Each launch
// overwrites every partial it later reads, so nothing has to be cleared
// between calls.
// ---------------------------------------------------------------------------
namespace fegb {

namespace {

constexpr int NOALLOC_BLOCKS = 152;
constexpr int NOALLOC_MAX_COLS = 32;
constexpr int NOALLOC_MAX_PAIRS = NOALLOC_MAX_COLS * (NOALLOC_MAX_COLS + 1) / 2;

__device__ __align__(256) double g_syrk_noalloc_partials[NOALLOC_BLOCKS * NOALLOC_MAX_PAIRS];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
double* g_noalloc_partials[NOALLOC_MAX_DEVICES] = {};
unsigned long long g_noalloc_ctx_id[NOALLOC_MAX_DEVICES] = {};

// Driver entry points for the current context's identity, fetched through the
// runtime so the library needs no link against libcuda.
typedef int (*ctx_get_current_fn)(void** ctx);
typedef int (*ctx_get_id_fn)(void* ctx, unsigned long long* id);

// Identity of the calling thread's current context; *have = false when no
// context is current or its identity cannot be read (a context destroyed by a
// reset), so that the caller runs the set-up again.
int current_context_id(unsigned long long* id, bool* have) {
    static ctx_get_current_fn get_current = nullptr;
    static ctx_get_id_fn get_id = nullptr;
    *have = false;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1{}, q2{};
        FEGB_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1),
                  "cudaGetDriverEntryPointByVersion (cuCtxGetCurrent)");
        FEGB_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2),
                  "cudaGetDriverEntryPointByVersion (cuCtxGetId)");
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return set_error("fe_gpu_syrk_noalloc: the driver does not provide cuCtxGetCurrent/cuCtxGetId");
        get_current = reinterpret_cast<ctx_get_current_fn>(f1);
        get_id = reinterpret_cast<ctx_get_id_fn>(f2);
    }
    void* ctx = nullptr;
    if (get_current(&ctx) != 0 || !ctx) return 0;
    if (get_id(ctx, id) != 0) return 0;
    *have = true;
    return 0;
}

// Device address of the partials array in the current device's context
// (looked up on the first call per device and again whenever the context
// changed since).
int noalloc_partials(double** out) {
    int dev = 0;
    FEGB_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return set_error("fe_gpu_syrk_noalloc: device %d out of range", dev);
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    unsigned long long ctx_id = 0;
    bool have = false;
    FEGB_TRY(current_context_id(&ctx_id, &have));
    if (!have || !g_noalloc_partials[dev] || g_noalloc_ctx_id[dev] != ctx_id) {
        // set-up: the lookup also makes the device's primary context current
        void* p = nullptr;
        FEGB_CUDA(cudaGetSymbolAddress(&p, g_syrk_noalloc_partials), "cudaGetSymbolAddress (syrk scratch)");
        FEGB_TRY(current_context_id(&ctx_id, &have));
        if (!have) return set_error("fe_gpu_syrk_noalloc: no current CUDA context after set-up");
        g_noalloc_partials[dev] = static_cast<double*>(p);
        g_noalloc_ctx_id[dev] = ctx_id;
    }
    *out = g_noalloc_partials[dev];
    return 0;
}

}  // namespace

}  // namespace fegb

extern "C" int fe_gpu_syrk_noalloc(int n_rows, int n_cols, double alpha, const double* W, int ldW, double beta,
                                   double* Q) {
    using namespace fegb;
    if (n_cols == 0) return set_ok();
    if (n_cols < 0 || n_rows < 0) return set_error("fe_gpu_syrk_noalloc: negative dimension");
    if (n_cols > NOALLOC_MAX_COLS)
        return set_error("fe_gpu_syrk_noalloc: n_cols=%d exceeds the %d-column limit of its fixed scratch", n_cols,
                         NOALLOC_MAX_COLS);
    if (ldW < std::max(1, n_rows))
        return set_error("fe_gpu_syrk_noalloc: ldW=%d is below max(1, n_rows=%d)", ldW, n_rows);
    double* partials = nullptr;
    FEGB_TRY(noalloc_partials(&partials));
    const cudaStream_t s = 0;  // legacy default stream, as the rest of the kernel-level ABI
    const int npairs = n_cols * (n_cols + 1) / 2;
    int nb = 0;
    if (n_rows > 0) {
        long long blocks = std::min<long long>(((long long)n_rows + CP_TR - 1) / CP_TR, NOALLOC_BLOCKS);
        long long rpb = ((long long)n_rows + blocks - 1) / blocks;
        rpb = ((rpb + CP_TR - 1) / CP_TR) * CP_TR;
        nb = (int)(((long long)n_rows + rpb - 1) / rpb);
        CPParams p;
        p.A = W;
        p.ars = 1;
        p.acs = ldW;
        p.a = n_cols;
        p.B = W;
        p.brs = 1;
        p.bcs = ldW;
        p.b = n_cols;
        p.n = n_rows;
        p.gram = 1;
        p.p0 = 0;
        p.npairs = npairs;
        p.phases = npairs <= 128 ? CP_THREADS / npairs : 1;
        p.rows_per_block = rpb;
        p.partials = partials;
        const size_t smem = sizeof(double) * CP_TR * n_cols;
        if (npairs <= 128)
            crossprod_kernel<1><<<nb, CP_THREADS, smem, s>>>(p);
        else
            crossprod_kernel<4><<<nb, CP_THREADS, smem, s>>>(p);
        FEGB_LAUNCH_CHECK("syrk noalloc");
    }
    // nb = 0 (no rows) leaves Q = beta Q on the upper triangle
    crossprod_reduce_kernel<<<reduce_blocks(npairs), 256, 0, s>>>(partials, nb, npairs, 0, 1, 1, n_cols, alpha, beta, Q,
                                                                  n_cols);
    FEGB_LAUNCH_CHECK("syrk noalloc reduce");
    FEGB_CUDA(cudaStreamSynchronize(s), "syrk noalloc sync");
    return set_ok();
}
