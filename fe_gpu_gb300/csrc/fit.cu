// Whole-fit estimator: device preparation, within-transform (plain FP64 and
// FP32-correction refinement), normal equations / 2SLS, clustered SEs.
//
// Host-side control mirrors the reference estimation driver
// (src/core/fe_pipeline.f90:516-1896) and within-transform
// (src/gpu/fe_gpu_demean.f90:63-311); all per-row work runs in this library's
// kernels on one stream.
#include "fegb.h"
#include "common.cuh"
#include "linalg.cuh"
#include "prep.cuh"
#include "sweep.cuh"
#include "batch_est.cuh"

#include <algorithm>
#include <thread>
#include <string>
#include <mutex>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <cfloat>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>
#include <vector>

namespace fegb {

namespace {

using Clock = std::chrono::steady_clock;
inline double seconds_since(Clock::time_point t0) {
    return std::chrono::duration<double>(Clock::now() - t0).count();
}

constexpr int MODE_CONTIG = 0;
constexpr int MODE_GATHER = 1;
// FEGB_TRACE in the environment: 1 = one stderr line per CG outer round,
// 2 = also every 10th inner iteration of a host-driven (profiled) solve
inline int trace_level() {
    static const int lvl = [] {
        const char* v = std::getenv("FEGB_TRACE");
        return v && v[0] ? std::atoi(v) : 0;
    }();
    return lvl;
}
inline bool trace_enabled() { return trace_level() > 0; }

// FEGB_TRACE >= 2: the stream drained and the time since t0 printed at a
// point of the preparation. The sync is taken only when tracing; it holds
// back the work issued after it, so a traced fit overlaps less.
inline void trace_phase(cudaStream_t s, Clock::time_point t0, const char* what) {
    if (trace_level() < 2) return;
    cudaStreamSynchronize(s);
    std::fprintf(stderr, "fegb prep: %-28s %8.2f ms\n", what,
                 1e3 * std::chrono::duration<double>(Clock::now() - t0).count());
}

constexpr int MODE_SMALLG = 2;
constexpr int CHUNK_R = 256;
constexpr int MAX_CLUSTER_DIMS = 3;  // src/core/fe_pipeline.f90:20

struct Dim {
    int G = 0;
    int mode = MODE_GATHER;
    int32_t* gid = nullptr;   // storage order, 0-based
    int32_t* perm = nullptr;  // traversal position -> storage row (gather mode)
    int32_t* gseq = nullptr;  // group id at traversal position (contig: = gid)
    int32_t* off = nullptr;   // G + 1 (contig / gather)
    int32_t* counts = nullptr;
    std::vector<int32_t*> gid_at_perm;  // [e] gid of dim e at traversal positions (gather)
    int32_t* long_list = nullptr;       // groups spanning more than SEG_LONG_SPAN chunks
    int n_long = 0;
    int32_t* long_list_cg = nullptr;    // the same for the CG operator's chunk size
    int n_long_cg = 0;
    int32_t* multi_list_cg = nullptr;   // groups crossing 1..SEG_LONG_SPAN CG chunk boundaries
    int n_multi_cg = 0;
    double* prev = nullptr;
    double* pend64 = nullptr;
    float* pend32 = nullptr;
    double* alpha = nullptr;
    double* mu = nullptr;
};

struct Problem {
    cudaStream_t s = nullptr;
    Scratch* scr = nullptr;
    long long n = 0;
    int k = 0, l = 0, C = 0, n_fe = 0;
    double* X = nullptr;  // n x C FP64, storage order
    float* Xc = nullptr;  // n x C FP32 correction (mixed form)
    int32_t* row_of = nullptr;
    int primary = -1;
    std::vector<Dim> dims;
    std::vector<int> order;
    double* relax = nullptr;
    double* prev_change = nullptr;
    unsigned long long* change_bits = nullptr;  // n_fe
    unsigned long long* max_bits = nullptr;     // [0] iteration max, [1] mu max
    double* max_partials = nullptr;              // per-block maxima of a finalize launch
    double* sums = nullptr;
    double* head = nullptr;
    double* tail = nullptr;
    double* partials = nullptr;
    // concatenated G-space storage of all dimensions (element (g, c) of dim d at (goff[d] + g) * C + c)
    long long Gt = 0;
    std::vector<long long> goff;
    int32_t* counts_all = nullptr;
    double* inv_counts_all = nullptr;
    double* alpha_all = nullptr;
    double* mu_all = nullptr;
    int smallg_nb = 0;
    // the CG operator's row sort by distinct id tuples of its swept dimensions
    // (positions grouped by tuple), kept for the cluster subset over the same
    // dimensions: tuple t holds sorted positions tuple_off[t] .. tuple_off[t+1]
    std::vector<int> tuple_dims;            // FE dimensions of the key, ascending
    std::vector<const int32_t*> tuple_gid;  // their id arrays when the sort ran
    const int32_t* tuple_perm = nullptr;
    const int32_t* tuple_off = nullptr;
    const int32_t* tuple_gseq = nullptr;
    int tuple_m = 0;
    long long tuple_n = 0;
    // compressed operator streams: the tuple of each storage row and, per swept
    // dimension, the group of each tuple; the refinement passes subtract one
    // combined increment per tuple (inc_tab) instead of one per dimension
    int32_t* row_tuple = nullptr;
    std::vector<int> tuple_sw;                 // swept dimensions of the tuples
    std::vector<const int32_t*> tuple_ids;     // m ids per swept dimension
    // per FE dimension of the tuples: the tuples in its group order (order:
    // tuple at each position, null = identity), their group ids and offsets
    std::vector<const int32_t*> tuple_dim_order, tuple_dim_gseq, tuple_dim_off;
    double* inc_tab = nullptr;                 // m x C
    // long-group lists of persistent offset arrays (the tuple streams), found
    // once: offsets array, group count -> list, list length
    struct LongCache {
        const int32_t* off;
        int G;
        int32_t* list;
        int n;
        int32_t* multi = nullptr;  // groups crossing 1..SEG_LONG_SPAN chunk edges (null: not found yet)
        int n_multi = 0;
    };
    std::vector<LongCache> long_cache;
    // recorded after the host upload of y, W and Z (null: already resident);
    // the data block waits for it, the id preparation does not
    cudaEvent_t data_ready = nullptr;
    // largest row count of a (group of d, group of e) pair, from the CG's count
    // matrices (-1: not counted); at most 1 means the pairs are unique
    std::vector<std::vector<int>> pair_max;
    int projections = 0;
    double demean_bytes = 0.0;
    // optional per-launch CUDA-event timing of the sweep kernels
    bool profile = false;
    struct Timed {
        cudaEvent_t a, b;
        int kind;
        double bytes;
    };
    std::vector<Timed> timed;
    ~Problem() {
        for (auto& t : timed) {
            cudaEventDestroy(t.a);
            cudaEventDestroy(t.b);
        }
    }
};

// Sums the recorded sweep-launch durations into the result (kind 0..3).
int collect_profile(Problem& P, fegb_result* res) {
    if (!P.profile || P.timed.empty()) return 0;
    FEGB_CUDA(cudaStreamSynchronize(P.s), "profile sync");
    for (auto& t : P.timed) {
        float ms = 0.f;
        FEGB_CUDA(cudaEventElapsedTime(&ms, t.a, t.b), "profile elapsed");
        if (t.kind < 0 || t.kind >= 8) continue;
        res->prof_launches[t.kind] += 1;
        res->prof_seconds[t.kind] += ms * 1e-3;
        res->prof_bytes[t.kind] += t.bytes;
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    P.timed.clear();
    return 0;
}

// ----------------------------- small kernels ------------------------------

// Row-major working copy X (n x C: y, then W, then Z) from the column-major
// inputs, and back. A block moves XT rows x all C columns through shared
// memory (stride Cp = C rounded up to odd, so a warp reading down a column
// does not conflict on banks): it reads XT consecutive values of each column
// and writes (or reads) the XT rows as one contiguous run of XT x C values.
// Whole rows per block matter: split by column tiles, every 32-byte sector of
// a row was written by two blocks far apart in time and read back from DRAM
// to merge the halves (25 ms at 10M x 111).
inline int xt_rows(int C) {
    const int cp = C | 1;
    const int fit = (96 * 1024) / (8 * cp);
    return fit >= 8 ? std::min(128, fit) / 8 * 8 : std::max(1, fit);
}

// column c of the (y, W, Z) inputs, each column-major with leading dimension ld
template <typename P>
__device__ __forceinline__ P* x_column(P* y, P* W, P* Z, int k, long long ld, int c) {
    return c == 0 ? y : (c <= k ? W + (long long)(c - 1) * ld : Z + (long long)(c - 1 - k) * ld);
}

__global__ void build_x_kernel(const double* __restrict__ y, const double* __restrict__ W,
                               const double* __restrict__ Z, int k, long long ld, const int32_t* __restrict__ row_of,
                               long long n, int C, int XT, double* __restrict__ X) {
    extern __shared__ double tile[];
    const int cp = C | 1;
    const long long r0 = (long long)blockIdx.x * XT;
    const int rows = (int)min((long long)XT, n - r0);
    for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e % rows, c = e / rows;
        const long long src = row_of ? (long long)row_of[r0 + r] : r0 + r;
        tile[r * cp + c] = x_column(y, W, Z, k, ld, c)[src];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e / C, c = e - r * C;
        X[r0 * C + e] = tile[r * cp + c];
    }
}

// X[r] = T[row_of[r]] for whole rows of C values: one warp per row, lanes
// over the columns (contiguous runs on both sides)
__global__ void gather_rows_kernel(const double* __restrict__ T, const int32_t* __restrict__ row_of, long long n, int C,
                                   double* __restrict__ X) {
    const int lane = threadIdx.x & 31;
    long long r = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const long long st = ((long long)gridDim.x * blockDim.x) >> 5;
    for (; r < n; r += st) {
        const double* src = T + (long long)row_of[r] * C;
        double* dst = X + r * C;
        for (int c = lane; c < C; c += 32) dst[c] = src[c];
    }
}

__global__ void scatter_x_kernel(const double* __restrict__ X, const int32_t* __restrict__ row_of, long long n, int C,
                                 int k, long long ld, int XT, double* __restrict__ y, double* __restrict__ W,
                                 double* __restrict__ Z) {
    extern __shared__ double tile[];
    const int cp = C | 1;
    const long long r0 = (long long)blockIdx.x * XT;
    const int rows = (int)min((long long)XT, n - r0);
    for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e / C, c = e - r * C;
        tile[r * cp + c] = X[r0 * C + e];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < rows * C; e += blockDim.x) {
        const int r = e % rows, c = e / rows;
        const long long dst = row_of ? (long long)row_of[r0 + r] : r0 + r;
        x_column(y, W, Z, k, ld, c)[dst] = tile[r * cp + c];
    }
}

__global__ void gather_gid_kernel(const int32_t* __restrict__ ids, const int32_t* __restrict__ rows, long long n,
                                  int32_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) out[i] = ids[rows ? rows[i] : i] - 1;
}

// *flag = 1 when keys is not non-decreasing (every writer stores the same value)
__global__ void order_check_kernel(const uint32_t* __restrict__ keys, long long n, int* __restrict__ flag) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x + 1;
    const long long st = (long long)gridDim.x * blockDim.x;
    bool bad = false;
    for (; i < n; i += st) bad = bad || keys[i] < keys[i - 1];
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) *flag = 1;
}

__global__ void gather_keys_kernel(const int32_t* __restrict__ ids, const int32_t* __restrict__ rows, long long n,
                                   uint32_t* __restrict__ keys, int32_t* __restrict__ vals) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        long long r = rows ? rows[i] : i;
        keys[i] = (uint32_t)(ids[r] - 1);
        vals[i] = (int32_t)r;
    }
}

__global__ void gather_i32_kernel(const int32_t* __restrict__ src, const int32_t* __restrict__ idx, long long n,
                                  int32_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) out[i] = src[idx[i]];
}

// Distinct id tuples of the swept dimensions: tuple k covers the key-sorted
// rows [off[k], off[k + 1]); its weight is that row count and its ids are
// those of its first row.
__global__ void tuple_build_kernel(const int32_t* __restrict__ off, const int32_t* __restrict__ perm, long long m,
                                   int nd, const int32_t* const* __restrict__ gids, int32_t* const* __restrict__ tgid,
                                   float* __restrict__ weight) {
    long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; k < m; k += st) {
        const int r = perm[off[k]];
        weight[k] = (float)(off[k + 1] - off[k]);
        for (int j = 0; j < nd; ++j) tgid[j][k] = gids[j][r];
    }
}

__global__ void gather_f32_kernel(const float* __restrict__ src, const int32_t* __restrict__ idx, long long n,
                                  float* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) out[i] = src[idx[i]];
}

// Sets *hit when two rows share both their group of a and their group of b
// (b has at most 64 groups): one 64-bit mask of seen groups of b per group
// of a. The outcome does not depend on the order of the atomic updates.
__global__ void pair_collision_kernel(const int32_t* __restrict__ ga, const int32_t* __restrict__ gb, long long n,
                                      unsigned long long* __restrict__ seen, int* __restrict__ hit) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    bool h = false;
    for (; i < n; i += st) {
        const unsigned long long bit = 1ULL << gb[i];
        h |= (atomicOr(seen + ga[i], bit) & bit) != 0;
    }
    if (__any_sync(0xffffffffu, h) && (threadIdx.x & 31) == 0) atomicOr(hit, 1);
}

__global__ void counts_from_offsets_kernel(const int32_t* __restrict__ off, int G, int32_t* __restrict__ counts) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < G) counts[g] = off[g + 1] - off[g];
}

// Group sizes of a small-G dimension: a shared-memory histogram per block,
// then one global add per (block, group). Integer sums, so the result does not
// depend on the order of the adds.
__global__ void count_ids_kernel(const int32_t* __restrict__ gid, long long n, int G, int32_t* __restrict__ counts) {
    extern __shared__ int32_t hist[];
    for (int g = threadIdx.x; g < G; g += blockDim.x) hist[g] = 0;
    __syncthreads();
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) atomicAdd(&hist[gid[i]], 1);
    __syncthreads();
    for (int g = threadIdx.x; g < G; g += blockDim.x)
        if (hist[g]) atomicAdd(&counts[g], hist[g]);
}

__global__ void reset_relax_kernel(double* relax, double* prev_change, int n) {
    int d = threadIdx.x;
    if (d < n) {
        relax[d] = 1.5;
        prev_change[d] = DBL_MAX;
    }
}

__global__ void keep_flags_kernel(const uint8_t* __restrict__ keep, long long n, uint32_t* __restrict__ flags) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) flags[i] = keep[i] ? 1u : 0u;
}

__global__ void compact_rows_kernel(const uint8_t* __restrict__ keep, const uint32_t* __restrict__ excl, long long n,
                                    int32_t* __restrict__ rows) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st)
        if (keep[i]) rows[excl[i]] = (int32_t)i;
}

__global__ void deinterleave_ids_kernel(const int32_t* __restrict__ ids, int n_fe, long long n, int32_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n * n_fe; i += st) {
        long long row = i / n_fe;
        int d = (int)(i - row * n_fe);
        out[(long long)d * n + row] = ids[i];
    }
}

// ------------------------------ helpers -----------------------------------

template <typename T>
int dalloc(Scratch& scr, T** p, size_t count, const char* what) {
    return scr.alloc(p, count, what);
}

int d2h_sync(void* dst, const void* src, size_t bytes, cudaStream_t s, const char* what) {
    FEGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s), what);
    FEGB_CUDA(cudaStreamSynchronize(s), what);
    return 0;
}

int h2d_sync(void* dst, const void* src, size_t bytes, cudaStream_t s, const char* what) {
    FEGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s), what);
    FEGB_CUDA(cudaStreamSynchronize(s), what);
    return 0;
}

double bits_to_double(unsigned long long b) {
    double v;
    std::memcpy(&v, &b, sizeof(v));
    return v;
}

// ---------------------------- preparation ---------------------------------

// Builds the storage-order problem from device inputs in the reference layout.
// Dimensions the CG operator handles through dense count matrices: at most
// DENSE_SMALL_MAX_G groups, C <= 32, and all matrices together within 8 GB at
// uint32 counts. Such a dimension needs no row sort of its own.
std::vector<char> cg_dense_plan(const std::vector<int>& G, int C, long long n) {
    std::vector<char> dense(G.size(), 0);
    if (C > 32 || n <= 0) return dense;
    double bytes = 0.0;  // worst case: uint32 counts
    for (size_t d = 0; d < G.size(); ++d)
        if (G[d] > 0 && G[d] <= DENSE_SMALL_MAX_G)
            for (size_t e = 0; e < G.size(); ++e)
                if (e != d) bytes += 4.0 * std::max(1, G[e]) * G[d];
    if (bytes > 8e9) return dense;
    for (size_t d = 0; d < G.size(); ++d) dense[d] = G[d] > 0 && G[d] <= DENSE_SMALL_MAX_G;
    return dense;
}

int build_problem(Problem& P, long long n_in, int k, int l, int n_fe, const double* y, const double* W, const double* Z,
                  const int32_t* const* ids, const int* G_in, bool drop_singletons, bool mixed, long long* n_single,
                  bool sorted_all = false) {
    cudaStream_t s = P.s;
    Scratch& scr = *P.scr;
    const auto t_bp = Clock::now();
    P.k = k;
    P.l = l;
    P.C = 1 + k + l;
    P.n_fe = n_fe;
    if (n_fe > SWEEP_MAXP) return set_error("at most %d FE dimensions are supported (got %d)", SWEEP_MAXP, n_fe);
    *n_single = 0;
    std::vector<int> G(n_fe, 0);
    for (int d = 0; d < n_fe; ++d) {
        int mn = 0, mx = 0;
        FEGB_TRY(ids_min_max(ids[d], n_in, &mn, &mx, s, scr));
        if (n_in > 0 && mn < 1)
            return set_error("FE indices must be positive and contiguous (dimension %d)", d + 1);
        G[d] = n_in > 0 ? mx : 0;
        if (G_in && G_in[d] > 0) {
            if (G_in[d] < G[d]) return set_error("group size %d below max id %d (dimension %d)", G_in[d], G[d], d + 1);
            G[d] = G_in[d];
        }
    }
    trace_phase(s, t_bp, "id ranges");
    // rows kept (singleton removal) in original order
    const int32_t* rows = nullptr;
    long long n = n_in;
    if (drop_singletons && n_fe > 0 && n_in > 0) {
        std::vector<int32_t*> g0(n_fe);
        for (int d = 0; d < n_fe; ++d) {
            FEGB_TRY(dalloc(scr, &g0[d], (size_t)n_in, "singleton gid"));
            gather_gid_kernel<<<grid_stride_blocks(n_in, 256), 256, 0, s>>>(ids[d], nullptr, n_in, g0[d]);
            FEGB_LAUNCH_CHECK("singleton gid");
        }
        uint8_t* keep = nullptr;
        FEGB_TRY(dalloc(scr, &keep, (size_t)n_in, "keep mask"));
        long long dropped = 0;
        FEGB_TRY(fegb::drop_singletons(g0.data(), G.data(), n_fe, n_in, keep, &dropped, s, scr));
        *n_single = dropped;
        if (dropped > 0) {
            uint32_t *flags = nullptr, *excl = nullptr;
            int32_t* kept = nullptr;
            FEGB_TRY(dalloc(scr, &flags, (size_t)n_in, "keep flags"));
            FEGB_TRY(dalloc(scr, &excl, (size_t)n_in, "keep scan"));
            FEGB_TRY(dalloc(scr, &kept, (size_t)n_in, "kept rows"));
            keep_flags_kernel<<<grid_stride_blocks(n_in, 256), 256, 0, s>>>(keep, n_in, flags);
            FEGB_TRY(scan_exclusive_u32(flags, excl, n_in, nullptr, s, scr));
            compact_rows_kernel<<<grid_stride_blocks(n_in, 256), 256, 0, s>>>(keep, excl, n_in, kept);
            FEGB_LAUNCH_CHECK("compact rows");
            rows = kept;
            n = n_in - dropped;
        }
    }
    P.n = n;
    const int C = P.C;
    // primary dimension: the one with most groups (first on ties)
    P.primary = -1;
    for (int d = 0; d < n_fe; ++d)
        if (P.primary < 0 || G[d] > G[P.primary]) P.primary = d;
    P.dims.assign(n_fe, Dim());
    for (int d = 0; d < n_fe; ++d) P.dims[d].G = G[d];
    // storage order: stable sort by the primary id
    int32_t* row_of = nullptr;
    if (P.primary >= 0 && n > 0) {
        uint32_t *keys = nullptr, *sorted = nullptr;
        int32_t* vals = nullptr;
        FEGB_TRY(dalloc(scr, &keys, (size_t)n, "primary keys"));
        FEGB_TRY(dalloc(scr, &vals, (size_t)n, "primary rows"));
        FEGB_TRY(dalloc(scr, &sorted, (size_t)n, "primary sorted"));
        FEGB_TRY(dalloc(scr, &row_of, (size_t)n, "row_of"));
        gather_keys_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(ids[P.primary], rows, n, keys, vals);
        FEGB_LAUNCH_CHECK("primary keys");
        // rows already in primary order (a panel stored id by id) keep their order: no sort
        int* unsorted = nullptr;
        FEGB_TRY(dalloc(scr, &unsorted, 1, "order flag"));
        FEGB_CUDA(cudaMemsetAsync(unsorted, 0, sizeof(int), s), "order flag");
        order_check_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(keys, n, unsorted);
        FEGB_LAUNCH_CHECK("primary order check");
        int h_unsorted = 1;
        FEGB_TRY(d2h_sync(&h_unsorted, unsorted, sizeof(int), s, "order flag copy"));
        if (!h_unsorted) {
            row_of = rows ? vals : nullptr;
            P.dims[P.primary].gid = reinterpret_cast<int32_t*>(keys);
        } else {
            FEGB_TRY(radix_sort_u32(keys, vals, sorted, row_of, n, bits_for((unsigned long long)G[P.primary]), s,
                                    scr));
            P.dims[P.primary].gid = reinterpret_cast<int32_t*>(sorted);
        }
    } else if (rows) {
        row_of = const_cast<int32_t*>(rows);
    }
    P.row_of = row_of;
    // the AoS data block is built last: everything before it reads only the ids,
    // so it overlaps an upload of y, W and Z still in flight (P.data_ready)
    FEGB_TRY(dalloc(scr, &P.X, (size_t)n * C, "data block"));
    if (mixed) FEGB_TRY(dalloc(scr, &P.Xc, (size_t)n * C, "correction block"));
    // per-dimension structures; group-indexed tables are slices of concatenated arrays
    P.goff.assign(n_fe + 1, 0);
    for (int d = 0; d < n_fe; ++d) P.goff[d + 1] = P.goff[d] + std::max(1, G[d]);
    P.Gt = P.goff[n_fe];
    FEGB_TRY(dalloc(scr, &P.counts_all, (size_t)std::max(1LL, P.Gt), "counts"));
    FEGB_TRY(dalloc(scr, &P.alpha_all, (size_t)std::max(1LL, P.Gt) * C, "fe coefficients"));
    FEGB_TRY(dalloc(scr, &P.mu_all, (size_t)std::max(1LL, P.Gt) * C, "fp64 group means"));
    FEGB_CUDA(cudaMemsetAsync(P.counts_all, 0, sizeof(int32_t) * (size_t)std::max(1LL, P.Gt), s), "counts zero");
    FEGB_CUDA(cudaMemsetAsync(P.alpha_all, 0, sizeof(double) * (size_t)std::max(1LL, P.Gt) * C, s), "alpha zero");
    int gmax = 1, gmax_small = 0;
    // the CG operator sweeps every dimension it does not handle densely
    std::vector<char> cg_sorted(n_fe, 0);
    if (sorted_all) {
        const std::vector<char> dense = cg_dense_plan(G, C, n);
        for (int d = 0; d < n_fe; ++d) cg_sorted[d] = d != P.primary && !dense[d];
    }
    for (int d = 0; d < n_fe; ++d) {
        Dim& D = P.dims[d];
        D.counts = P.counts_all + P.goff[d];
        D.alpha = P.alpha_all + P.goff[d] * C;
        D.mu = P.mu_all + P.goff[d] * C;
        if (d != P.primary) {
            FEGB_TRY(dalloc(scr, &D.gid, (size_t)n, "gid"));
            if (n > 0) {
                gather_gid_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(ids[d], row_of, n, D.gid);
                FEGB_LAUNCH_CHECK("gid gather");
            }
        }
        if (d == P.primary) {
            D.mode = MODE_CONTIG;
            D.gseq = D.gid;
        } else if (smallg_eligible(D.G, C)) {
            D.mode = MODE_SMALLG;
        } else {
            D.mode = MODE_GATHER;
        }
        const bool need_sorted = D.mode == MODE_GATHER || cg_sorted[d];
        if (need_sorted && n > 0) {
            uint32_t* sorted = nullptr;
            FEGB_TRY(dalloc(scr, &sorted, (size_t)n, "gather gseq"));
            FEGB_TRY(dalloc(scr, &D.perm, (size_t)n, "gather perm"));
            FEGB_TRY(radix_sort_u32(reinterpret_cast<const uint32_t*>(D.gid), nullptr, sorted, D.perm, n,
                                    bits_for((unsigned long long)D.G), s, scr));
            D.gseq = reinterpret_cast<int32_t*>(sorted);
        }
        if (D.mode != MODE_SMALLG || need_sorted) {
            FEGB_TRY(dalloc(scr, &D.off, (size_t)D.G + 1, "offsets"));
            if (n > 0) {
                FEGB_TRY(segment_offsets(reinterpret_cast<const uint32_t*>(D.gseq), n, D.G, D.off, s));
            } else {
                FEGB_CUDA(cudaMemsetAsync(D.off, 0, sizeof(int32_t) * ((size_t)D.G + 1), s), "offsets zero");
            }
            if (D.G > 0) {
                counts_from_offsets_kernel<<<(D.G + 255) / 256, 256, 0, s>>>(D.off, D.G, D.counts);
                FEGB_LAUNCH_CHECK("counts");
                FEGB_TRY(dalloc(scr, &D.long_list, (size_t)D.G, "long groups"));
                FEGB_TRY(find_long_groups(D.off, D.G, CHUNK_R, D.long_list, &D.n_long, s));
                if (sorted_all && (cg_sorted[d] || d == P.primary)) {  // the dimensions the CG operator sweeps
                    FEGB_TRY(dalloc(scr, &D.long_list_cg, (size_t)D.G, "long groups (cg)"));
                    FEGB_TRY(find_long_groups(D.off, D.G, CG_CHUNK, D.long_list_cg, &D.n_long_cg, s));
                    FEGB_TRY(dalloc(scr, &D.multi_list_cg, (size_t)D.G, "multi-chunk groups (cg)"));
                    FEGB_TRY(find_multi_groups(D.off, D.G, CG_CHUNK, D.multi_list_cg, &D.n_multi_cg, s));
                }
            }
        }
        if (D.mode == MODE_SMALLG) {
            if (!need_sorted) {  // sorted dimensions already have counts from their offsets
                FEGB_CUDA(cudaMemsetAsync(D.counts, 0, sizeof(int32_t) * (size_t)D.G, s), "counts zero");
                if (n > 0 && D.G > 0) {
                    count_ids_kernel<<<std::min<unsigned>(grid_stride_blocks(n, 256), 4u * (unsigned)num_sms()), 256,
                                       sizeof(int32_t) * (size_t)D.G, s>>>(D.gid, n, D.G, D.counts);
                    FEGB_LAUNCH_CHECK("count ids");
                }
            }
            gmax_small = std::max(gmax_small, D.G);
        }
        gmax = std::max(gmax, D.G);
        size_t gc = (size_t)std::max(1, D.G) * C;
        FEGB_TRY(dalloc(scr, &D.prev, gc, "prev means"));
        FEGB_TRY(dalloc(scr, &D.pend64, gc, "pending means"));
        if (mixed) FEGB_TRY(dalloc(scr, &D.pend32, gc, "pending means fp32"));
    }
    FEGB_TRY(dalloc(scr, &P.inv_counts_all, (size_t)std::max(1LL, P.Gt), "inverse counts"));
    FEGB_TRY(launch_inv_counts(P.counts_all, P.Gt, P.inv_counts_all, s));
    for (int d = 0; d < n_fe; ++d) {
        Dim& D = P.dims[d];
        D.gid_at_perm.assign(n_fe, nullptr);
        if (!(D.mode == MODE_GATHER || cg_sorted[d]) || n == 0) continue;
        for (int e = 0; e < n_fe; ++e) {
            if (e == d) continue;
            FEGB_TRY(dalloc(scr, &D.gid_at_perm[e], (size_t)n, "gid at perm"));
            gather_i32_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(P.dims[e].gid, D.perm, n, D.gid_at_perm[e]);
            FEGB_LAUNCH_CHECK("gid at perm");
        }
    }
    long long nchunks = std::max(1LL, seg_nchunks(n, CHUNK_R));
    FEGB_TRY(dalloc(scr, &P.sums, (size_t)gmax * C, "group sums"));
    FEGB_TRY(dalloc(scr, &P.head, (size_t)nchunks * C, "chunk heads"));
    FEGB_TRY(dalloc(scr, &P.tail, (size_t)nchunks * C, "chunk tails"));
    P.smallg_nb = smallg_nblocks(std::max(1LL, n));
    if (gmax_small > 0) FEGB_TRY(dalloc(scr, &P.partials, (size_t)P.smallg_nb * gmax_small * C, "small-G partials"));
    FEGB_TRY(dalloc(scr, &P.relax, (size_t)std::max(1, n_fe), "relaxation"));
    FEGB_TRY(dalloc(scr, &P.prev_change, (size_t)std::max(1, n_fe), "prev change"));
    FEGB_TRY(dalloc(scr, &P.change_bits, (size_t)std::max(1, n_fe), "change"));
    FEGB_TRY(dalloc(scr, &P.max_bits, 2, "max update"));
    FEGB_TRY(dalloc(scr, &P.max_partials, (size_t)finalize_blocks((long long)gmax * C) + 1, "max partials"));
    // sweep order: ascending group count, exchange sort of fe_gpu_demean.f90:104-114
    P.order.resize(n_fe);
    for (int d = 0; d < n_fe; ++d) P.order[d] = d;
    for (int a = 0; a < n_fe - 1; ++a)
        for (int b = a + 1; b < n_fe; ++b)
            if (G[P.order[b]] < G[P.order[a]]) std::swap(P.order[a], P.order[b]);
    trace_phase(s, t_bp, "id preparation");
    if (P.data_ready) FEGB_CUDA(cudaStreamWaitEvent(s, P.data_ready, 0), "data upload wait");
    trace_phase(s, t_bp, "data upload");
    if (n > 0) {
        const int xt = xt_rows(C);
        const size_t smem = sizeof(double) * (size_t)xt * (C | 1);
        static const cudaError_t attr =
            cudaFuncSetAttribute(build_x_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
        if (attr != cudaSuccess) return set_cuda_error(attr, "build data block attr");
        // Rows in a new order: transpose the inputs in their own order first,
        // then gather whole rows (C x 8 contiguous bytes each). Gathering each
        // value from its column directly reads one 32-byte sector per 8 bytes
        // at random (0.7 TB/s at 10M x 111). Only when the extra copy fits
        // with room to spare.
        size_t free_b = 0, total_b = 0;
        const size_t tmp_bytes = sizeof(double) * (size_t)n_in * C;
        bool two_pass = row_of && C >= 2 && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
                        free_b > 2 * tmp_bytes + (1ull << 30);
        if (two_pass) {
            Scratch tmp(s);
            double* T = nullptr;
            if (tmp.alloc(&T, (size_t)n_in * C, "transposed inputs") != 0) {
                cudaGetLastError();
                set_ok();
                two_pass = false;
            } else {
                build_x_kernel<<<(unsigned)((n_in + xt - 1) / xt), 256, smem, s>>>(y, W, Z, k, n_in, nullptr, n_in,
                                                                                   C, xt, T);
                FEGB_LAUNCH_CHECK("transpose inputs");
                gather_rows_kernel<<<grid_stride_blocks(n * 32, 256), 256, 0, s>>>(T, row_of, n, C, P.X);
                FEGB_LAUNCH_CHECK("gather rows");
                // tmp is released on the stream after the gather
            }
        }
        if (!two_pass) {
            build_x_kernel<<<(unsigned)((n + xt - 1) / xt), 256, smem, s>>>(y, W, Z, k, n_in, row_of, n, C, xt, P.X);
            FEGB_LAUNCH_CHECK("build data block");
        }
        trace_phase(s, t_bp, two_pass ? "data block (two passes)" : "data block (one pass)");
    }
    return 0;
}

// ------------------------------- sweeps -----------------------------------

struct PendingList {
    std::vector<int> dims;
    bool has(int d) const { return std::find(dims.begin(), dims.end(), d) != dims.end(); }
};

template <typename T>
const T* pend_table(const Dim& D);
template <>
const double* pend_table<double>(const Dim& D) {
    return D.pend64;
}
template <>
const float* pend_table<float>(const Dim& D) {
    return D.pend32;
}

template <typename T>
PendingSet<T> make_pending(const Problem& P, int d, const PendingList& pl) {
    PendingSet<T> ps{};
    ps.n = 0;
    const Dim& D = P.dims[d];
    for (int e : pl.dims) {
        const int32_t* g;
        if (D.mode == MODE_GATHER)
            g = (e == d) ? D.gseq : D.gid_at_perm[e];
        else
            g = P.dims[e].gid;
        ps.gid[ps.n] = g;
        ps.tab[ps.n] = pend_table<T>(P.dims[e]);
        ++ps.n;
    }
    return ps;
}

struct ProjectionOpts {
    const double* bias = nullptr;
    bool alpha = false;
    bool mixing = true;
};

// Group sums of dimension d over the current residual of `data`, with all
// pending tables applied; then the finalize epilogue.
template <typename T>
int sweep_sums_impl(Problem& P, int d, T* data, const PendingSet<T>& ps, bool writeback);

// One sweep launch (segment or small-G), timed with CUDA events on the fit's
// stream when profiling is on. Algorithmic bytes per launch: n (4 + C s) for
// the group ids and the rows read, n C s more when the rows are written back,
// 4 n for the traversal permutation of a gathered sweep and 4 n per pending
// table's ids.
template <typename T>
int sweep_sums(Problem& P, int d, T* data, const PendingSet<T>& ps, bool writeback) {
    if (!P.profile) return sweep_sums_impl<T>(P, d, data, ps, writeback);
    Problem::Timed t;
    t.kind = (P.dims[d].mode == MODE_SMALLG ? 2 : 0) + (sizeof(T) == 4 ? 1 : 0);
    const Dim& D = P.dims[d];
    const bool wb = writeback && D.mode != MODE_GATHER;
    t.bytes = (double)P.n * (4.0 + (wb ? 2.0 : 1.0) * P.C * sizeof(T) + (D.mode == MODE_GATHER ? 4.0 : 0.0) +
                             4.0 * ps.n);
    FEGB_CUDA(cudaEventCreate(&t.a), "profile event");
    FEGB_CUDA(cudaEventCreate(&t.b), "profile event");
    FEGB_CUDA(cudaEventRecord(t.a, P.s), "profile record");
    int st = sweep_sums_impl<T>(P, d, data, ps, writeback);
    FEGB_CUDA(cudaEventRecord(t.b, P.s), "profile record");
    P.timed.push_back(t);
    return st;
}

template <typename T>
int sweep_sums_impl(Problem& P, int d, T* data, const PendingSet<T>& ps, bool writeback) {
    Dim& D = P.dims[d];
    if (D.mode == MODE_SMALLG) {
        SmallGParams<T> sp{};
        sp.X = data;
        sp.C = P.C;
        sp.n = P.n;
        sp.gid = D.gid;
        sp.G = D.G;
        sp.pend = ps;
        sp.writeback = writeback ? 1 : 0;
        sp.rows_per_block = (P.n + P.smallg_nb - 1) / P.smallg_nb;
        sp.partials = P.partials;
        FEGB_TRY(launch_smallg_sweep<T>(sp, P.smallg_nb, P.s));
        return launch_fold_smallg(P.partials, P.smallg_nb, D.G, P.C, P.sums, P.s);
    }
    SegSweepParams<T> sp{};
    sp.X = data;
    sp.rs = P.C;
    sp.cs = 1;
    sp.C = P.C;
    sp.n = P.n;
    sp.perm = D.mode == MODE_GATHER ? D.perm : nullptr;
    sp.gseq = D.gseq;
    sp.pend = ps;
    sp.writeback = (writeback && D.mode == MODE_CONTIG) ? 1 : 0;
    sp.R = CHUNK_R;
    sp.sums = P.sums;
    sp.head = P.head;
    sp.tail = P.tail;
    FEGB_TRY(launch_seg_sweep<T>(sp, P.s));
    return launch_long_sums(D.off, P.head, P.tail, CHUNK_R, P.C, D.long_list, D.n_long, P.sums, P.s);
}

FinalizeParams finalize_base(const Problem& P, int d) {
    const Dim& D = P.dims[d];
    FinalizeParams f{};
    f.G = D.G;
    f.C = P.C;
    if (D.mode == MODE_SMALLG) {
        f.sums = P.sums;  // folded by launch_fold_smallg
    } else {
        f.off = D.off;
        f.sums = P.sums;
        f.head = P.head;
        f.tail = P.tail;
        f.R = CHUNK_R;
    }
    f.counts = D.counts;
    f.inv_counts = P.inv_counts_all + P.goff[d];
    return f;
}

// One AP projection of dimension d (symmetric relaxed scheme).
template <typename T>
int project(Problem& P, int d, T* data, PendingList& pl, const ProjectionOpts& o) {
    if (P.n == 0 || P.dims[d].G <= 0) return 0;
    Dim& D = P.dims[d];
    PendingSet<T> ps = make_pending<T>(P, d, pl);
    const bool wb = D.mode != MODE_GATHER;
    FEGB_TRY(sweep_sums<T>(P, d, data, ps, wb));
    bool accumulate = false;
    if (wb) {
        pl.dims.clear();
        pl.dims.push_back(d);
    } else {
        accumulate = pl.has(d);
        if (!accumulate) pl.dims.push_back(d);
    }
    FinalizeParams f = finalize_base(P, d);
    f.bias = o.bias;
    if (o.mixing) {
        f.prev = D.prev;
        f.relax = P.relax + d;
    }
    f.pend64 = D.pend64;
    f.pend32 = D.pend32;
    f.pend_accumulate = accumulate ? 1 : 0;
    f.alpha = o.alpha ? D.alpha : nullptr;
    f.max_partials = P.max_partials;
    f.do_relax_update = 1;
    f.relax_rw = P.relax + d;
    f.prev_change = P.prev_change + d;
    f.max_update_bits = P.max_bits;
    FEGB_TRY(launch_finalize(f, P.s));
    P.projections += 1;
    P.demean_bytes += (double)P.n * (4.0 + 2.0 * P.C * sizeof(T));
    return 0;
}

template <typename T>
int apply_all_pending(Problem& P, T* data, PendingList& pl) {
    if (pl.dims.empty() || P.n == 0) return 0;
    PendingSet<T> ps{};
    ps.n = 0;
    for (int e : pl.dims) {
        ps.gid[ps.n] = P.dims[e].gid;
        ps.tab[ps.n] = pend_table<T>(P.dims[e]);
        ++ps.n;
    }
    FEGB_TRY(launch_apply_pending<T>(data, P.C, P.n, ps, P.s));
    pl.dims.clear();
    return 0;
}

int reset_ap_state(Problem& P, bool alpha) {
    for (int d = 0; d < P.n_fe; ++d) {
        size_t gc = (size_t)std::max(1, P.dims[d].G) * P.C;
        FEGB_CUDA(cudaMemsetAsync(P.dims[d].prev, 0, gc * sizeof(double), P.s), "reset prev");
        if (alpha && P.dims[d].alpha)
            FEGB_CUDA(cudaMemsetAsync(P.dims[d].alpha, 0, gc * sizeof(double), P.s), "reset alpha");
    }
    if (P.n_fe > 0) {
        reset_relax_kernel<<<1, 32 * ((P.n_fe + 31) / 32), 0, P.s>>>(P.relax, P.prev_change, P.n_fe);
        FEGB_LAUNCH_CHECK("reset relaxation");
    }
    return 0;
}

// One iteration = two symmetric sweeps (forward then backward over the dims),
// as in fe_gpu_demean.f90:144-292. Returns the max |mixed mean| on the host.
template <typename T>
int ap_iteration(Problem& P, T* data, PendingList& pl, const ProjectionOpts& o, double* max_update) {
    FEGB_CUDA(cudaMemsetAsync(P.max_bits, 0, sizeof(unsigned long long), P.s), "reset max");
    for (int sweep = 0; sweep < 2; ++sweep) {
        for (int sidx = 0; sidx < P.n_fe; ++sidx) FEGB_TRY(project<T>(P, P.order[sidx], data, pl, o));
        for (int sidx = P.n_fe - 1; sidx >= 0; --sidx) FEGB_TRY(project<T>(P, P.order[sidx], data, pl, o));
    }
    unsigned long long b = 0;
    FEGB_TRY(d2h_sync(&b, P.max_bits, sizeof(b), P.s, "max update copy"));
    *max_update = bits_to_double(b);
    return 0;
}

int demean_plain(Problem& P, double tol, int max_iter, int* iterations, int* converged, double* max_update) {
    *iterations = 0;
    *converged = 1;
    *max_update = 0.0;
    if (P.n_fe == 0 || P.n == 0) return 0;
    FEGB_TRY(reset_ap_state(P, false));
    PendingList pl;
    ProjectionOpts o;
    int hit = 0;
    double mu = 0.0;
    for (int iter = 1; iter <= max_iter; ++iter) {
        FEGB_TRY(ap_iteration<double>(P, P.X, pl, o, &mu));
        *iterations = iter;
        if (mu < tol) {
            hit = 1;
            break;
        }
    }
    FEGB_TRY(apply_all_pending<double>(P, P.X, pl));
    *converged = hit;
    *max_update = mu;
    return 0;
}

// inc[t][c] = sum over the swept dimensions j of alpha_j[ids_j[t]][c], in
// dimension order (FP64)
struct TupleInc {
    int nd;
    const int32_t* ids[SWEEP_MAXP];
    const double* alpha[SWEEP_MAXP];
};
// (one element per thread, 32-bit index arithmetic when m C < 2^31)
__global__ void tuple_increments_kernel(TupleInc ti, long long m, int C, double* __restrict__ inc) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    const long long total = m * C;
    const bool narrow = total < 0x7fffffffLL;
    for (; i < total; i += st) {
        const long long t = narrow ? (long long)((unsigned)i / (unsigned)C) : i / C;
        const int c = (int)(i - t * C);
        double v = ti.alpha[0][(long long)ti.ids[0][t] * C + c];
        for (int j = 1; j < ti.nd; ++j) v += ti.alpha[j][(long long)ti.ids[j][t] * C + c];
        inc[i] = v;
    }
}

// Sums of the ns columns of S (row-major, stride ns) over the clusters of a
// traversal (perm: storage row at each position, null = storage order; gseq:
// cluster at each position; off: n_cl + 1 offsets) into Sc (n_cl x ns), over
// npos positions (-1: all rows). timed_kind >= 0 records the sweep launch in
// that profile family.
int cluster_score_sums(Problem& P, const double* S, int ns, const int32_t* perm, const int32_t* gseq,
                       const int32_t* off, int n_cl, double* Sc, Scratch& scr, long long npos = -1,
                       int timed_kind = -1, bool persistent_off = false, const FinalizeParams* outputs = nullptr);

int tuple_row_sums(Problem& P, const double* X, int C, double* out, Scratch& scr, int timed_kind);

// FP64 group means of the current FP64 residual for every dimension, after
// subtracting the FE increments of the previous refinement round from the rows
// (apply_alpha; one element pass, then read-only sweeps). With compressed CG
// streams the swept dimensions' sums come from one row sweep into per-tuple
// sums and short sweeps of those (n C + sum_d m C additions instead of
// n C per dimension). Returns max |mean|.
int fp64_mean_pass(Problem& P, bool apply_alpha, double* mu_max) {
    if (apply_alpha && P.n > 0) {
        PendingSet<double> ps{};
        std::vector<char> in_tuple(P.n_fe, 0);
        if (P.row_tuple && P.tuple_n == P.n && P.tuple_sw.size() > 1) {
            // one combined increment per tuple of the swept dimensions: two FP64
            // subtractions per element at 20M (tuple, period) instead of three
            TupleInc ti{};
            ti.nd = (int)P.tuple_sw.size();
            for (int j = 0; j < ti.nd; ++j) {
                ti.ids[j] = P.tuple_ids[j];
                ti.alpha[j] = P.dims[P.tuple_sw[j]].alpha;
                in_tuple[P.tuple_sw[j]] = 1;
            }
            tuple_increments_kernel<<<grid_stride_blocks((long long)P.tuple_m * P.C, 256), 256, 0, P.s>>>(
                ti, P.tuple_m, P.C, P.inc_tab);
            FEGB_LAUNCH_CHECK("tuple increments");
            ps.gid[ps.n] = P.row_tuple;
            ps.tab[ps.n] = P.inc_tab;
            ++ps.n;
        }
        for (int e = 0; e < P.n_fe; ++e) {
            if (in_tuple[e]) continue;
            ps.gid[ps.n] = P.dims[e].gid;
            ps.tab[ps.n] = P.dims[e].alpha;
            ++ps.n;
        }
        FEGB_TRY(launch_apply_pending<double>(P.X, P.C, P.n, ps, P.s));
        P.demean_bytes += (double)P.n * (4.0 * ps.n + 16.0 * P.C);
    }
    FEGB_CUDA(cudaMemsetAsync(P.max_bits + 1, 0, sizeof(unsigned long long), P.s), "reset mu max");
    std::vector<char> via_tuples(P.n_fe, 0);
    Scratch ts(P.s);
    if (P.n > 0 && P.tuple_m > 0 && P.tuple_n == P.n && P.tuple_sw.size() > 1 &&
        (double)P.tuple_m <= 0.75 * (double)P.n) {
        bool all = true;
        for (int d : P.tuple_sw) all = all && P.tuple_dim_gseq.size() > (size_t)d && P.tuple_dim_gseq[d];
        if (all) {
            double* tsum = nullptr;
            FEGB_TRY(ts.alloc(&tsum, (size_t)P.tuple_m * P.C, "tuple sums"));
            FEGB_TRY(tuple_row_sums(P, P.X, P.C, tsum, ts, 0));
            P.demean_bytes += (double)P.n * (8.0 + 8.0 * P.C);
            for (int d : P.tuple_sw) {
                Dim& D = P.dims[d];
                FinalizeParams f{};
                f.counts = D.counts;
                f.inv_counts = P.inv_counts_all + P.goff[d];
                f.mean_out = D.mu;
                f.max_partials = P.max_partials;
                f.change_bits = P.max_bits + 1;
                FEGB_TRY(cluster_score_sums(P, tsum, P.C, P.tuple_dim_order[d], P.tuple_dim_gseq[d],
                                            P.tuple_dim_off[d], D.G, nullptr, ts, P.tuple_m, -1, true, &f));
                P.demean_bytes += (double)P.tuple_m * ((P.tuple_dim_order[d] ? 8.0 : 4.0) + 8.0 * P.C);
                via_tuples[d] = 1;
            }
        }
    }
    for (int d = 0; d < P.n_fe; ++d) {
        Dim& D = P.dims[d];
        if (D.G <= 0 || P.n <= 0 || via_tuples[d]) continue;
        FEGB_TRY(sweep_sums<double>(P, d, P.X, PendingSet<double>{}, false));
        FinalizeParams f = finalize_base(P, d);
        f.mean_out = D.mu;
        f.max_partials = P.max_partials;
        f.change_bits = P.max_bits + 1;
        FEGB_TRY(launch_finalize(f, P.s));
        P.demean_bytes += (double)P.n * (4.0 + 8.0 * P.C);
    }
    unsigned long long b = 0;
    FEGB_TRY(d2h_sync(&b, P.max_bits + 1, sizeof(b), P.s, "mu max copy"));
    *mu_max = bits_to_double(b);
    return 0;
}

// Mixed form: FP64 residual r (P.X) and FP64 FE increments alpha; the inner
// alternating projections run on an FP32 correction block c with the FP64 group
// means of r as a per-group bias (group means of r + c = mu + means of c).
int demean_mixed(Problem& P, double tol, int max_iter, int* iterations, int* converged, double* max_update,
                 int* outer) {
    *iterations = 0;
    *converged = 1;
    *max_update = 0.0;
    *outer = 0;
    if (P.n_fe == 0 || P.n == 0) return 0;
    const int max_outer = 12;
    double mu = 0.0, mu_prev = DBL_MAX;
    int total_iter = 0;
    bool apply_alpha = false;
    int hit = 0;
    for (int round = 0; round < max_outer; ++round) {
        FEGB_TRY(fp64_mean_pass(P, apply_alpha, &mu));
        *outer = round + 1;
        if (mu < tol) {
            hit = 1;
            break;
        }
        if (total_iter >= max_iter) break;
        if (round > 2 && mu > 0.5 * mu_prev) break;  // refinement stalled
        mu_prev = mu;
        // inner FP32 correction sweeps
        FEGB_CUDA(cudaMemsetAsync(P.Xc, 0, sizeof(float) * (size_t)P.n * P.C, P.s), "zero correction");
        FEGB_TRY(reset_ap_state(P, true));
        PendingList pl;
        double inner_tol = std::max(0.25 * tol, 1e-5 * mu);
        double upd = 0.0;
        for (int it = 0; it < max_iter - total_iter; ++it) {
            // per-dimension bias = FP64 means of r
            ProjectionOpts o;
            o.alpha = true;
            // the bias differs per dimension: run the iteration projection by projection
            FEGB_CUDA(cudaMemsetAsync(P.max_bits, 0, sizeof(unsigned long long), P.s), "reset max");
            for (int sweep = 0; sweep < 2; ++sweep) {
                for (int pass = 0; pass < 2; ++pass) {
                    for (int sidx = 0; sidx < P.n_fe; ++sidx) {
                        int d = pass == 0 ? P.order[sidx] : P.order[P.n_fe - 1 - sidx];
                        o.bias = P.dims[d].mu;
                        FEGB_TRY(project<float>(P, d, P.Xc, pl, o));
                    }
                }
            }
            unsigned long long b = 0;
            FEGB_TRY(d2h_sync(&b, P.max_bits, sizeof(b), P.s, "inner max copy"));
            upd = bits_to_double(b);
            ++total_iter;
            if (upd < inner_tol) break;
        }
        apply_alpha = true;
    }
    *iterations = total_iter;
    *converged = hit;
    *max_update = mu;
    return 0;
}


// ----------------------- conjugate gradients (alpha space) -----------------------

// Scratch of the CG solve in storage type T.
template <typename T>
struct CGBuffers {
    T *r = nullptr, *z = nullptr, *p = nullptr, *q = nullptr, *x = nullptr, *inv = nullptr;
    int ld = 0;  // padded row stride of the G-space vectors
    double *rz = nullptr, *rz_new = nullptr, *pq = nullptr;
    double *rz_part = nullptr, *pq_part = nullptr, *zmax_part = nullptr;
    T* sums = nullptr;  // operator sweep: complete-run group sums (G_max x C, storage type)
    double *head = nullptr, *tail = nullptr;  // and chunk head/tail partials (chunks x C)
    unsigned long long* zmax = nullptr;
    int rz_blocks = 0, pq_blocks = 0;
    std::vector<int> pq_block_off;
    // dimensions with few groups handled through dense count matrices:
    // dense[s] says whether s is one; N8[s][e] / N32[s][e] = G_e x G_s counts
    // of the rows of each (group of e, group of s) pair, e != s (uint8 when
    // every count is below 256)
    std::vector<char> dense;
    std::vector<std::vector<uint8_t*>> N8;
    std::vector<std::vector<uint32_t*>> N32;
    std::vector<long long> dpart_off, dsum_off;  // per dense s: its partial blocks, its sums
    double* dense_part = nullptr;
    double* dense_sums = nullptr;
    T* extra = nullptr;  // Gt x C: the dense dimensions' share of each swept dimension's q
    bool any_dense = false;
    // the operator sweep of each many-group dimension d: positions in d's group
    // order, either the rows or (compressed) the distinct id tuples of the
    // many-group dimensions, each weighted by its row count
    struct Stream {
        long long m = 0;
        const int32_t* gseq = nullptr;
        const int32_t* off = nullptr;  // G_d + 1 offsets over the positions
        int n_src = 0;
        const int32_t* src_gid[SWEEP_MAXP] = {};
        int src_dim[SWEEP_MAXP] = {};
        const float* weight = nullptr;
        const int32_t* long_list = nullptr;
        int n_long = 0;
        const int32_t* multi_list = nullptr;
        int n_multi = 0;
        bool short_groups = false;  // every group short: the one-thread-per-group sweep applies
    };
    std::vector<Stream> stream;
    bool compressed = false;
    // Schur-complement form: the primary (largest) dimension is eliminated, the
    // CG vectors span the other dimensions only (off[d]: their rows, Gv in all),
    // and the primary's slot of p (at off[primary]) holds -u = -(1/n) D_P'D_R x,
    // the primary's response to the other dimensions' x
    bool schur = false;
    int prim = -1;
    std::vector<long long> off;
    long long Gv = 0;
    int32_t* counts_v = nullptr;  // group sizes in the CG layout
    double* mu_v = nullptr;       // FP64 group means in the CG layout (Schur form)
};

// row_tuple[perm[i]] = rank[i]: the tuple of each storage row
__global__ void scatter_tuple_kernel(const int32_t* __restrict__ perm, const int32_t* __restrict__ rank, long long n,
                                     int32_t* __restrict__ row_tuple) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) row_tuple[perm[i]] = rank[i];
}

// flags[i] = 1 where the pair (ga, gb) changes along an ordered list of rows
__global__ void pair_flags_kernel(const int32_t* __restrict__ ga, const int32_t* __restrict__ gb, long long n,
                                  uint32_t* __restrict__ flags) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) flags[i] = (i == 0 || ga[i] != ga[i - 1] || gb[i] != gb[i - 1]) ? 1u : 0u;
}

// rank[i] = the run of position i; off[run] = its first position
__global__ void run_ranks_kernel(const uint32_t* __restrict__ flags, const uint32_t* __restrict__ excl, long long n,
                                 int32_t* __restrict__ off, int32_t* __restrict__ rank) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        const int32_t r = (int32_t)(excl[i] + flags[i]) - 1;
        rank[i] = r;
        if (flags[i]) off[r] = (int32_t)i;
    }
}

// Position streams of the CG operator sweeps (see CGBuffers::Stream). The
// rows are compressed into distinct id tuples of the many-group dimensions
// when that removes at least a quarter of the positions: the operator carries
// no row data, so rows with equal ids contribute equally (weight x one row).
template <typename T>
int cg_streams(Problem& P, CGBuffers<T>& B) {
    Scratch& scr = *P.scr;
    cudaStream_t s = P.s;
    const long long n = P.n;
    std::vector<int> sw;  // swept dimensions, the primary last (most significant key part)
    for (int d = 0; d < P.n_fe; ++d)
        if (P.dims[d].G > 0 && !B.dense[d] && d != P.primary) sw.push_back(d);
    if (P.primary >= 0 && P.dims[P.primary].G > 0 && !B.dense[P.primary]) sw.push_back(P.primary);
    B.stream.assign(P.n_fe, typename CGBuffers<T>::Stream());
    // rows, in each dimension's group order
    for (int d : sw) {
        Dim& D = P.dims[d];
        auto& st = B.stream[d];
        st.m = n;
        st.gseq = D.gseq;
        st.off = D.off;
        for (int e : sw) {
            if (e == d) continue;
            st.src_dim[st.n_src] = e;
            st.src_gid[st.n_src++] = d == P.primary ? P.dims[e].gid : D.gid_at_perm[e];
        }
        st.long_list = D.long_list_cg;
        st.n_long = D.n_long_cg;
        st.multi_list = D.multi_list_cg;
        st.n_multi = D.n_multi_cg;
    }
    if (sw.size() < 2 || n < 4096) return 0;
    std::vector<const int32_t*> ptrs;
    std::vector<unsigned long long> strides;
    unsigned long long stride = 1;
    for (int d : sw) {
        const unsigned long long Gd = (unsigned long long)P.dims[d].G;
        if (stride > (1ULL << 62) / Gd) return 0;  // key does not fit: keep the rows
        ptrs.push_back(P.dims[d].gid);
        strides.push_back(stride);
        stride *= Gd;
    }
    int m = 0;
    int32_t *perm = nullptr, *toff = nullptr, *tseq = nullptr;
    // the swept dimension whose group order the tuples come in: the primary (the
    // most significant key part) after a key sort; with one other swept
    // dimension e, e itself: its own row sort is stable over the storage order,
    // which is the primary's, so it already lists the rows in (group of e,
    // primary group) order and the tuples are its runs of equal pairs
    int in_order = P.primary;
    const int32_t n32 = (int32_t)n;
    {
        Scratch tmp(s);  // the sort's work arrays, released once the tuples are built
        // the row permutation, offsets and tuple ranks outlive the operator: the
        // cluster subset over the same dimensions reuses them
        FEGB_TRY(dalloc(scr, &toff, (size_t)n + 1, "tuple offsets"));
        FEGB_TRY(dalloc(scr, &tseq, (size_t)n, "tuple ranks"));
        const Dim* E = (sw.size() == 2 && sw[1] == P.primary) ? &P.dims[sw[0]] : nullptr;
        if (E && E->perm && E->gseq && E->gid_at_perm.size() > (size_t)P.primary && E->gid_at_perm[P.primary]) {
            in_order = sw[0];
            perm = E->perm;
            uint32_t *flags = nullptr, *excl = nullptr, *total = nullptr;
            FEGB_TRY(tmp.alloc(&flags, (size_t)n, "pair run flags"));
            FEGB_TRY(tmp.alloc(&excl, (size_t)n, "pair run scan"));
            FEGB_TRY(tmp.alloc(&total, 1, "pair run count"));
            pair_flags_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(E->gseq, E->gid_at_perm[P.primary], n, flags);
            FEGB_LAUNCH_CHECK("pair run flags");
            FEGB_TRY(scan_exclusive_u32(flags, excl, n, total, s, tmp));
            run_ranks_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(flags, excl, n, toff, tseq);
            FEGB_LAUNCH_CHECK("pair run ranks");
            uint32_t hm = 0;
            FEGB_TRY(d2h_sync(&hm, total, sizeof(hm), s, "pair run count copy"));
            m = (int)hm;
            FEGB_TRY(h2d_sync(toff + m, &n32, sizeof(int32_t), s, "pair run end"));
        } else {
            FEGB_TRY(dalloc(scr, &perm, (size_t)n, "tuple perm"));
            FEGB_TRY(cluster_ids_by_key(ptrs.data(), strides.data(), (int)sw.size(), n, bits_for(stride), nullptr,
                                        &m, perm, toff, s, tmp, true, tseq));
        }
        if (m > 0) {
            P.tuple_dims.assign(sw.begin(), sw.end());
            std::sort(P.tuple_dims.begin(), P.tuple_dims.end());
            P.tuple_gid.clear();
            for (int d : P.tuple_dims) P.tuple_gid.push_back(P.dims[d].gid);
            P.tuple_perm = perm;
            P.tuple_off = toff;
            P.tuple_gseq = tseq;
            P.tuple_m = m;
            P.tuple_n = n;
        }
        if (m <= 0 || (double)m > 0.75 * (double)n) return 0;
        std::vector<int32_t*> tg(sw.size());
        for (size_t j = 0; j < sw.size(); ++j) FEGB_TRY(dalloc(scr, &tg[j], (size_t)m, "tuple ids"));
        float* w = nullptr;
        FEGB_TRY(dalloc(scr, &w, (size_t)m, "tuple weights"));
        int32_t** dg = nullptr;
        const int32_t** dsrc = nullptr;
        FEGB_TRY(tmp.alloc(&dg, sw.size(), "tuple id table"));
        FEGB_TRY(tmp.alloc(&dsrc, sw.size(), "tuple source table"));
        FEGB_CUDA(cudaMemcpyAsync(dg, tg.data(), sizeof(int32_t*) * sw.size(), cudaMemcpyHostToDevice, s),
                  "tuple id table");
        FEGB_CUDA(cudaMemcpyAsync(dsrc, ptrs.data(), sizeof(int32_t*) * sw.size(), cudaMemcpyHostToDevice, s),
                  "tuple source table");
        tuple_build_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(toff, perm, m, (int)sw.size(), dsrc, dg, w);
        FEGB_LAUNCH_CHECK("tuple build");
        FEGB_TRY(dalloc(scr, &P.row_tuple, (size_t)n, "tuple of each row"));
        FEGB_TRY(dalloc(scr, &P.inc_tab, (size_t)m * P.C, "combined increments"));
        scatter_tuple_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(perm, tseq, n, P.row_tuple);
        FEGB_LAUNCH_CHECK("tuple of each row");
        P.tuple_sw.assign(sw.begin(), sw.end());
        P.tuple_ids.assign(tg.begin(), tg.end());
        P.tuple_dim_order.assign(P.n_fe, nullptr);
        P.tuple_dim_gseq.assign(P.n_fe, nullptr);
        P.tuple_dim_off.assign(P.n_fe, nullptr);
        FEGB_CUDA(cudaStreamSynchronize(s), "tuple build sync");  // host tables above are stack arrays
        // per swept dimension: the tuples in its group order
        for (size_t jd = 0; jd < sw.size(); ++jd) {
            const int d = sw[jd];
            const int G = P.dims[d].G;
            auto& st = B.stream[d];
            st = typename CGBuffers<T>::Stream();
            st.m = m;
            int32_t* order = nullptr;  // tuple index at each position (null: identity)
            if (d == in_order) {
                st.gseq = tg[jd];  // the tuples are already in this dimension's group order
                st.weight = w;
            } else {
                uint32_t* sorted = nullptr;
                float* wd = nullptr;
                FEGB_TRY(dalloc(scr, &sorted, (size_t)m, "tuple gseq"));
                FEGB_TRY(dalloc(scr, &order, (size_t)m, "tuple order"));
                FEGB_TRY(radix_sort_u32(reinterpret_cast<const uint32_t*>(tg[jd]), nullptr, sorted, order, m,
                                        bits_for((unsigned long long)G), s, tmp));
                FEGB_TRY(dalloc(scr, &wd, (size_t)m, "tuple weights (sorted)"));
                gather_f32_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(w, order, m, wd);
                FEGB_LAUNCH_CHECK("tuple weight gather");
                st.gseq = reinterpret_cast<int32_t*>(sorted);
                st.weight = wd;
            }
            for (size_t je = 0; je < sw.size(); ++je) {
                if (je == jd) continue;
                if (!order) {
                    st.src_gid[st.n_src] = tg[je];
                } else {
                    int32_t* gj = nullptr;
                    FEGB_TRY(dalloc(scr, &gj, (size_t)m, "tuple source ids"));
                    gather_i32_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(tg[je], order, m, gj);
                    FEGB_LAUNCH_CHECK("tuple id gather");
                    st.src_gid[st.n_src] = gj;
                }
                st.src_dim[st.n_src++] = sw[je];
            }
            int32_t *off = nullptr, *ll = nullptr, *ml = nullptr;
            FEGB_TRY(dalloc(scr, &off, (size_t)G + 1, "tuple group offsets"));
            FEGB_TRY(segment_offsets(reinterpret_cast<const uint32_t*>(st.gseq), m, G, off, s));
            FEGB_TRY(dalloc(scr, &ll, (size_t)G, "tuple long groups"));
            FEGB_TRY(find_long_groups(off, G, CG_CHUNK, ll, &st.n_long, s));
            FEGB_TRY(dalloc(scr, &ml, (size_t)G, "tuple multi-chunk groups"));
            FEGB_TRY(find_multi_groups(off, G, CG_CHUNK, ml, &st.n_multi, s));
            st.off = off;
            st.long_list = ll;
            st.multi_list = ml;
            // the SEs sum the scores of this dimension's clusters from the tuples' sums
            P.tuple_dim_order[d] = order;
            P.tuple_dim_gseq[d] = st.gseq;
            P.tuple_dim_off[d] = off;
        }
        FEGB_CUDA(cudaStreamSynchronize(s), "tuple streams sync");
    }
    B.compressed = true;
    return 0;
}

// Schur form: Jacobi preconditioner from the diagonal of
// S = D_R'(I - P_P)D_R, S_gg = n_g - sum_w n_{w,g}^2 / n_w over the (group,
// primary group) pairs, instead of the group counts n_g (which overstate S_gg
// by up to n_g / S_gg: the inner solve's max |z| stop would then end it early).
// The pairs come from the dimension's compressed stream when its positions are
// exactly those pairs (one other swept dimension), from a sort of the rows by
// pair otherwise, and from the count matrices for the small dimensions.
template <typename T>
int cg_schur_precond(Problem& P, CGBuffers<T>& B) {
    const int pd = B.prim;
    std::vector<int> swept;
    for (int d = 0; d < P.n_fe; ++d)
        if (d != pd && P.dims[d].G > 0 && !B.dense[d]) swept.push_back(d);
    Scratch tmp(P.s);
    unsigned long long* acc = nullptr;
    FEGB_TRY(tmp.alloc(&acc, (size_t)std::max(1LL, B.Gv), "schur diagonal"));
    FEGB_CUDA(cudaMemsetAsync(acc, 0, sizeof(unsigned long long) * std::max(1LL, B.Gv), P.s), "schur diagonal zero");
    const bool stream_pairs = swept.size() == 1 && B.compressed;
    std::vector<int> by_counts;  // dimensions whose pair key does not fit 62 bits keep 1 / n_g
    for (int e : swept) {
        const auto& st = B.stream[e];
        const int32_t* pid = nullptr;
        for (int i = 0; i < st.n_src; ++i)
            if (st.src_dim[i] == pd) pid = st.src_gid[i];
        if (stream_pairs && pid) {
            FEGB_TRY(launch_schur_diag_stream(st.gseq, st.m, st.weight, pid, P.dims[pd].counts, acc + B.off[e], P.s));
            continue;
        }
        // the rows sorted by (group of e, primary group): one segment per pair
        const int32_t* ptrs[2] = {P.dims[pd].gid, P.dims[e].gid};
        const unsigned long long Gp = (unsigned long long)std::max(1, P.dims[pd].G);
        const unsigned long long strides[2] = {1ULL, Gp};
        if (Gp > (1ULL << 62) / (unsigned long long)P.dims[e].G) {
            by_counts.push_back(e);
            continue;
        }
        Scratch sub(P.s);
        int32_t *perm = nullptr, *off = nullptr;
        int npairs = 0;
        FEGB_TRY(sub.alloc(&perm, (size_t)P.n, "pair perm"));
        FEGB_TRY(sub.alloc(&off, (size_t)P.n + 1, "pair offsets"));
        FEGB_TRY(cluster_ids_by_key(ptrs, strides, 2, P.n, bits_for(Gp * (unsigned long long)P.dims[e].G), nullptr,
                                    &npairs, perm, off, P.s, sub, true, nullptr));
        FEGB_TRY(launch_schur_diag_pairs(perm, off, npairs, P.dims[e].gid, P.dims[pd].gid, P.dims[pd].counts,
                                         acc + B.off[e], P.s));
        FEGB_CUDA(cudaStreamSynchronize(P.s), "schur pairs sync");  // sub is released here
    }
    for (int sd = 0; sd < P.n_fe; ++sd) {
        if (!B.dense[sd] || sd == pd || P.dims[sd].G <= 0) continue;
        const int Gs = P.dims[sd].G;
        if (B.N8[sd][pd])
            FEGB_TRY(launch_schur_diag_dense<uint8_t>(B.N8[sd][pd], P.dims[pd].G, Gs, P.dims[pd].counts,
                                                      acc + B.off[sd], P.s));
        else
            FEGB_TRY(launch_schur_diag_dense<uint32_t>(B.N32[sd][pd], P.dims[pd].G, Gs, P.dims[pd].counts,
                                                       acc + B.off[sd], P.s));
    }
    FEGB_TRY(launch_inv_diag<T>(acc, B.counts_v, B.Gv, B.inv, P.s));
    for (int e : by_counts)
        FEGB_TRY(launch_inv_counts_t<T>(B.counts_v + B.off[e], P.dims[e].G, B.inv + B.off[e], P.s));
    FEGB_CUDA(cudaStreamSynchronize(P.s), "schur diagonal sync");
    return 0;
}

template <typename T>
int cg_alloc(Problem& P, CGBuffers<T>& B) {
    Scratch& scr = *P.scr;
    // r, z, q, x: compact rows of C; p (gathered by the operator sweep): rows padded to B.ld
    B.ld = cg_row_stride(P.C, (int)sizeof(T));
    const int C = P.C;
    // layout: the Schur form when the primary is swept (more than DENSE_SMALL_MAX_G
    // groups, or too many columns for the dense path) and another dimension exists
    B.prim = P.primary;
    {
        int others = 0;
        for (int d = 0; d < P.n_fe; ++d)
            if (d != P.primary && P.dims[d].G > 0) ++others;
        const bool prim_dense = P.primary < 0 || (P.dims[P.primary].G <= DENSE_SMALL_MAX_G && C <= 32);
        B.schur = !prim_dense && others > 0 && P.dims[P.primary].G > 0;
    }
    B.off.assign(P.n_fe, 0);
    long long prows = 0;  // rows of p
    if (B.schur) {
        long long o = 0;
        for (int d = 0; d < P.n_fe; ++d) {
            if (d == B.prim) continue;
            B.off[d] = o;
            o += std::max(1, P.dims[d].G);
        }
        B.Gv = o;
        B.off[B.prim] = o;
        prows = o + std::max(1, P.dims[B.prim].G);
    } else {
        for (int d = 0; d < P.n_fe; ++d) B.off[d] = P.goff[d];
        B.Gv = P.Gt;
        prows = P.Gt;
    }
    const size_t nc = (size_t)std::max(1LL, B.Gv) * C;
    const size_t np = (size_t)std::max(1LL, prows) * B.ld;
    FEGB_TRY(dalloc(scr, &B.r, nc, "cg r"));
    FEGB_TRY(dalloc(scr, &B.z, nc, "cg z"));
    FEGB_TRY(dalloc(scr, &B.p, np, "cg p"));
    FEGB_CUDA(cudaMemsetAsync(B.p, 0, sizeof(T) * np, P.s), "cg p padding zero");
    FEGB_TRY(dalloc(scr, &B.q, nc, "cg q"));
    FEGB_TRY(dalloc(scr, &B.x, nc, "cg solution"));
    if (B.schur) {
        FEGB_TRY(dalloc(scr, &B.counts_v, (size_t)std::max(1LL, B.Gv), "cg counts"));
        FEGB_TRY(dalloc(scr, &B.mu_v, nc, "cg group means"));
        FEGB_CUDA(cudaMemsetAsync(B.counts_v, 0, sizeof(int32_t) * (size_t)std::max(1LL, B.Gv), P.s), "cg counts");
        for (int d = 0; d < P.n_fe; ++d)
            if (d != B.prim && P.dims[d].G > 0)
                FEGB_CUDA(cudaMemcpyAsync(B.counts_v + B.off[d], P.counts_all + P.goff[d],
                                          sizeof(int32_t) * P.dims[d].G, cudaMemcpyDeviceToDevice, P.s),
                          "cg counts copy");
    } else {
        B.counts_v = P.counts_all;
    }
    FEGB_TRY(dalloc(scr, &B.inv, (size_t)std::max(1LL, B.Gv), "cg inverse counts"));
    FEGB_TRY(launch_inv_counts_t<T>(B.counts_v, B.Gv, B.inv, P.s));
    const int L = B.ld;
    FEGB_TRY(dalloc(scr, &B.rz, (size_t)C, "cg rz"));
    FEGB_TRY(dalloc(scr, &B.rz_new, (size_t)C, "cg rz new"));
    FEGB_TRY(dalloc(scr, &B.pq, (size_t)C, "cg pq"));
    FEGB_TRY(dalloc(scr, &B.zmax, 1, "cg zmax"));
    B.rz_blocks = cg_partial_blocks(B.Gv, C);
    B.pq_block_off.assign(P.n_fe + 1, 0);
    for (int d = 0; d < P.n_fe; ++d)
        B.pq_block_off[d + 1] =
            B.pq_block_off[d] + (B.schur && d == B.prim ? 0 : cg_partial_blocks(std::max(1, P.dims[d].G), C));
    B.pq_blocks = B.pq_block_off[P.n_fe];
    FEGB_TRY(dalloc(scr, &B.rz_part, (size_t)B.rz_blocks * C, "cg rz partials"));
    FEGB_TRY(dalloc(scr, &B.zmax_part, (size_t)B.rz_blocks, "cg zmax partials"));
    FEGB_TRY(dalloc(scr, &B.pq_part, (size_t)std::max(1, B.pq_blocks) * C, "cg pq partials"));
    FEGB_CUDA(cudaMemsetAsync(B.pq_part, 0, sizeof(double) * (size_t)std::max(1, B.pq_blocks) * C, P.s),
              "cg pq partials zero");
    // dense count matrices for dimensions with few groups (see CGBuffers)
    B.dense.assign(P.n_fe, 0);
    B.N8.assign(P.n_fe, std::vector<uint8_t*>(P.n_fe, nullptr));
    B.N32.assign(P.n_fe, std::vector<uint32_t*>(P.n_fe, nullptr));
    B.dpart_off.assign(P.n_fe, 0);
    B.dsum_off.assign(P.n_fe, 0);
    std::vector<int> Gd(P.n_fe);
    for (int d = 0; d < P.n_fe; ++d) Gd[d] = P.dims[d].G;
    const std::vector<char> plan = cg_dense_plan(Gd, C, P.n);
    if (std::find(plan.begin(), plan.end(), 1) != plan.end()) {
        {
            long long parts = 0, sums = 0;
            unsigned* mx = nullptr;
            FEGB_TRY(dalloc(scr, &mx, 1, "count max"));
            for (int d = 0; d < P.n_fe; ++d) {
                if (!plan[d]) continue;
                B.dense[d] = 1;
                B.any_dense = true;
                B.dpart_off[d] = parts;
                B.dsum_off[d] = sums;
                sums += (long long)P.dims[d].G * C;
                for (int e = 0; e < P.n_fe; ++e) {
                    if (e == d || P.dims[e].G <= 0) continue;
                    const size_t cnt = (size_t)P.dims[e].G * P.dims[d].G;
                    Scratch tmp(P.s);  // the uint32 counts, released once narrowed or copied
                    uint32_t* N = nullptr;
                    FEGB_TRY(tmp.alloc(&N, cnt, "count matrix"));
                    FEGB_CUDA(cudaMemsetAsync(N, 0, sizeof(uint32_t) * cnt, P.s), "count matrix zero");
                    FEGB_TRY(launch_count_pairs(P.dims[e].gid, P.dims[d].gid, P.n, P.dims[d].G, N, P.s));
                    FEGB_TRY(launch_count_max(N, (long long)cnt, mx, P.s));
                    unsigned hmx = 0;
                    FEGB_TRY(d2h_sync(&hmx, mx, sizeof(hmx), P.s, "count max copy"));
                    if (P.pair_max.size() != (size_t)P.n_fe) P.pair_max.assign(P.n_fe, std::vector<int>(P.n_fe, -1));
                    P.pair_max[d][e] = P.pair_max[e][d] = (int)std::min<unsigned>(hmx, 0x7fffffffu);
                    if (hmx < 256) {
                        FEGB_TRY(dalloc(scr, &B.N8[d][e], cnt, "count matrix (uint8)"));
                        FEGB_TRY(launch_narrow_counts(N, (long long)cnt, B.N8[d][e], P.s));
                    } else {
                        FEGB_TRY(dalloc(scr, &B.N32[d][e], cnt, "count matrix (uint32)"));
                        FEGB_CUDA(cudaMemcpyAsync(B.N32[d][e], N, sizeof(uint32_t) * cnt, cudaMemcpyDeviceToDevice,
                                                  P.s),
                                  "count matrix copy");
                    }
                    parts += (long long)dense_chunks(P.dims[e].G) * P.dims[d].G * C;
                }
            }
            if (B.any_dense) {
                FEGB_TRY(dalloc(scr, &B.dense_part, (size_t)std::max(1LL, parts), "dense partials"));
                FEGB_TRY(dalloc(scr, &B.dense_sums, (size_t)std::max(1LL, sums), "dense sums"));
                FEGB_TRY(dalloc(scr, &B.extra, (size_t)std::max(1LL, prows) * C, "dense extra"));
            }
        }
    }
    FEGB_TRY(cg_streams(P, B));
    // streams whose groups are all short (a worker's few firms) take the
    // one-thread-per-group sweep
    for (int d = 0; d < P.n_fe; ++d) {
        auto& st = B.stream[d];
        st.short_groups = false;
        if (st.n_src < 1 || st.n_src > 3 || !st.off || P.dims[d].G <= 0) continue;
        if ((long long)P.dims[d].G * CG_SHORT_MEAN < st.m) continue;
        int longest = 0;
        FEGB_TRY(max_group_length(st.off, P.dims[d].G, &longest, P.s));
        st.short_groups = longest <= CG_SHORT_MAX;
    }
    if (B.schur) FEGB_TRY(cg_schur_precond(P, B));
    // the operator sweep's sums / head / tail, compact rows of C
    {
        const long long nchunks = std::max(1LL, seg_nchunks(P.n, CG_CHUNK));
        int gmax = 1;
        for (int d = 0; d < P.n_fe; ++d) gmax = std::max(gmax, P.dims[d].G);
        FEGB_TRY(dalloc(scr, &B.sums, (size_t)gmax * C, "cg sums"));
        FEGB_TRY(dalloc(scr, &B.head, (size_t)nchunks * C, "cg heads"));
        FEGB_TRY(dalloc(scr, &B.tail, (size_t)nchunks * C, "cg tails"));
    }
    return 0;
}

// Profile events around a group of launches (no-ops unless P.profile).
struct CGTimer {
    Problem& P;
    Problem::Timed tm{};
    bool on = false;
    explicit CGTimer(Problem& p) : P(p) {}
    int begin(int kind, double bytes) {
        if (!P.profile) return 0;
        tm.kind = kind;
        tm.bytes = bytes;
        FEGB_CUDA(cudaEventCreate(&tm.a), "profile event");
        FEGB_CUDA(cudaEventCreate(&tm.b), "profile event");
        FEGB_CUDA(cudaEventRecord(tm.a, P.s), "profile record");
        on = true;
        return 0;
    }
    int end() {
        if (!on) return 0;
        FEGB_CUDA(cudaEventRecord(tm.b, P.s), "profile record");
        P.timed.push_back(tm);
        on = false;
        return 0;
    }
};

// The operator sweep of swept dimension d over its stream: complete group sums
// of -(sum of the sources' rows, weighted) into B.sums (storage type, stride C).
// Returns the number of swept sources (0: no sweep, B.sums untouched).
template <typename T>
int cg_sweep(Problem& P, CGBuffers<T>& B, int d, int* n_src) {
    const int C = P.C;
    const int L = B.ld;
    const auto& st = B.stream[d];
    *n_src = st.n_src;
    if (st.n_src == 0) return 0;
    CGRowsParams<T> rp{};
    rp.n = st.m;
    rp.C = C;
    rp.ld = L;
    rp.gseq = st.gseq;
    rp.n_src = st.n_src;
    for (int i = 0; i < st.n_src; ++i) {
        rp.src_gid[i] = st.src_gid[i];
        rp.src_tab[i] = B.p + B.off[st.src_dim[i]] * L;
    }
    rp.weight = st.weight;
    rp.sums = B.sums;
    rp.head = B.head;
    rp.tail = B.tail;
    // per position: destination id, source ids, weight, gathered source rows
    const double bytes =
        (double)st.m * (4.0 * (1 + rp.n_src) + (st.weight ? 4.0 : 0.0) + (double)rp.n_src * C * sizeof(T));
    CGTimer tm(P);
    FEGB_TRY(tm.begin(4 + (sizeof(T) == 4 ? 1 : 0), bytes));
    if (st.short_groups && tuning(TUNE_CG_SHORT)) {
        FEGB_TRY(launch_cg_short<T>(rp, st.off, P.dims[d].G, P.s));
    } else {
        FEGB_TRY(launch_cg_rows<T>(rp, P.s));
        FEGB_TRY(launch_group_sums<T>(st.off, B.head, B.tail, CG_CHUNK, C, st.long_list, st.n_long, st.multi_list,
                                      st.n_multi, B.sums, P.s));
    }
    FEGB_TRY(tm.end());
    P.demean_bytes += bytes;
    return 0;
}

// Schur form, step 1: the primary's slot of p = -u with
// u = (1/n_P) (D_P'D_R x), x = the other dimensions' rows of p: the primary's
// stream sweep gives -(sum over its rows of the swept dimensions' x), the dense
// count matrices the small dimensions' share.
// With exactly one small dimension s, one pass over the primary's count matrix
// both forms -u and the small side of s for the primary (*prim_small_done).
template <typename T>
int cg_schur_u(Problem& P, CGBuffers<T>& B, bool* prim_small_done = nullptr) {
    const int C = P.C;
    const int L = B.ld;
    const int pd = B.prim;
    const Dim& D = P.dims[pd];
    if (prim_small_done) *prim_small_done = false;
    int n_src = 0;
    FEGB_TRY(cg_sweep<T>(P, B, pd, &n_src));
    if (n_src == 0) FEGB_CUDA(cudaMemsetAsync(B.sums, 0, sizeof(T) * (size_t)D.G * C, P.s), "schur sums zero");
    int n_dense = 0, sd1 = -1;
    for (int d = 0; d < P.n_fe; ++d)
        if (B.dense[d]) {
            ++n_dense;
            sd1 = d;
        }
    if (n_dense == 1 && prim_small_done) {
        const int Gs = P.dims[sd1].G;
        long long part = 0;  // the primary's block of sd1's partials (cg_apply_rest's order)
        for (int e = 0; e < pd; ++e)
            if (e != sd1 && P.dims[e].G > 0) part += dense_chunks(P.dims[e].G);
        DenseSchur<T> sch;
        sch.sums = B.sums;
        sch.counts = D.counts;
        sch.table = B.p + B.off[pd] * L;
        double* pb = B.dense_part + B.dpart_off[sd1] + part * Gs * C;
        const T* ps = B.p + B.off[sd1] * L;
        const double bytes = (double)D.G * ((B.N8[sd1][pd] ? 1.0 : 4.0) * Gs + 2.0 * C * sizeof(T) + 4.0);
        CGTimer tm(P);
        FEGB_TRY(tm.begin(6 + (sizeof(T) == 4 ? 1 : 0), bytes));
        if (B.N8[sd1][pd])
            FEGB_TRY((launch_dense_pair<T, uint8_t>(B.N8[sd1][pd], D.G, Gs, nullptr, ps, L, C, pb, nullptr, 0, P.s,
                                                    sch)));
        else
            FEGB_TRY((launch_dense_pair<T, uint32_t>(B.N32[sd1][pd], D.G, Gs, nullptr, ps, L, C, pb, nullptr, 0,
                                                     P.s, sch)));
        FEGB_TRY(tm.end());
        P.demean_bytes += bytes;
        *prim_small_done = true;
        return 0;
    }
    T* ex = nullptr;
    if (B.any_dense) {
        CGTimer tm(P);
        double bytes = 0.0;
        bool first = true;
        FEGB_TRY(tm.begin(6 + (sizeof(T) == 4 ? 1 : 0), 0.0));
        for (int sd = 0; sd < P.n_fe; ++sd) {
            if (!B.dense[sd]) continue;
            ex = B.extra + B.off[pd] * C;
            const T* ps = B.p + B.off[sd] * L;
            if (B.N8[sd][pd])
                FEGB_TRY((launch_dense_pair<T, uint8_t>(B.N8[sd][pd], D.G, P.dims[sd].G, nullptr, ps, L, C, nullptr,
                                                        ex, first ? 0 : 1, P.s)));
            else
                FEGB_TRY((launch_dense_pair<T, uint32_t>(B.N32[sd][pd], D.G, P.dims[sd].G, nullptr, ps, L, C,
                                                         nullptr, ex, first ? 0 : 1, P.s)));
            bytes += (double)D.G * ((B.N8[sd][pd] ? 1.0 : 4.0) * P.dims[sd].G + (double)C * sizeof(T) * (first ? 1 : 2));
            first = false;
        }
        tm.tm.bytes = bytes;
        FEGB_TRY(tm.end());
        P.demean_bytes += bytes;
    }
    return launch_schur_u<T>(B.sums, ex, D.counts, D.G, C, B.p + B.off[pd] * L, L, P.s);
}

// q = D'D p over the CG dimensions, given p (and, in the Schur form, the
// primary's slot of p): (1) one pass over each count matrix of a small
// dimension, (2) the operator sweep of each many-group dimension, (3) q of
// the small dimensions from their complete sums. In the Schur form the primary
// is a source of the sweeps and of the count-matrix passes but has no q.
template <typename T>
int cg_apply_rest(Problem& P, CGBuffers<T>& B, bool prim_small_done = false) {
    const int C = P.C;
    const int L = B.ld;
    const int fp32 = sizeof(T) == 4 ? 1 : 0;
    auto in_cg = [&](int d) { return P.dims[d].G > 0 && !(B.schur && d == B.prim); };
    if (B.any_dense) {
        CGTimer tm(P);
        double bytes = 0.0;
        for (int sd = 0; sd < P.n_fe; ++sd) {
            if (!B.dense[sd]) continue;
            for (int e = 0; e < P.n_fe; ++e) {
                if (e == sd || P.dims[e].G <= 0 || (prim_small_done && e == B.prim)) continue;
                const double cb = B.N8[sd][e] ? 1.0 : 4.0;
                const bool ext = !B.dense[e] && in_cg(e);
                bytes += (double)P.dims[e].G * (cb * P.dims[sd].G + (double)C * sizeof(T) * (ext ? 2.0 : 1.0));
            }
        }
        FEGB_TRY(tm.begin(6 + fp32, bytes));
        std::vector<char> written(P.n_fe, 0);
        for (int sd = 0; sd < P.n_fe; ++sd) {
            if (!B.dense[sd]) continue;
            const int Gs = P.dims[sd].G;
            long long part = 0;
            double* pbase = B.dense_part + B.dpart_off[sd];
            for (int e = 0; e < P.n_fe; ++e) {
                if (e == sd || P.dims[e].G <= 0) continue;
                if (prim_small_done && e == B.prim) {  // done with the primary's response
                    part += dense_chunks(P.dims[e].G);
                    continue;
                }
                // the small side always; the other side only for a swept CG dimension
                T* ex = (B.dense[e] || !in_cg(e)) ? nullptr : B.extra + B.off[e] * C;
                const int acc = ex && written[e] ? 1 : 0;
                const T* pe = B.p + B.off[e] * L;
                const T* ps = B.p + B.off[sd] * L;
                if (B.N8[sd][e])
                    FEGB_TRY((launch_dense_pair<T, uint8_t>(B.N8[sd][e], P.dims[e].G, Gs, pe, ps, L, C,
                                                            pbase + part * Gs * C, ex, acc, P.s)));
                else
                    FEGB_TRY((launch_dense_pair<T, uint32_t>(B.N32[sd][e], P.dims[e].G, Gs, pe, ps, L, C,
                                                             pbase + part * Gs * C, ex, acc, P.s)));
                if (ex) written[e] = 1;
                part += dense_chunks(P.dims[e].G);
            }
            FEGB_TRY(launch_fold_dense(pbase, (int)part, Gs, C, B.dense_sums + B.dsum_off[sd], P.s));
        }
        FEGB_TRY(tm.end());
        P.demean_bytes += bytes;
    }
    for (int d = 0; d < P.n_fe; ++d) {
        Dim& D = P.dims[d];
        if (!in_cg(d) || B.dense[d]) continue;
        int n_src = 0;
        FEGB_TRY(cg_sweep<T>(P, B, d, &n_src));
        FinalizeParams src{};
        src.G = D.G;
        src.counts = D.counts;
        src.C = C;  // complete sums, compact rows (none without a swept source)
        if (n_src > 0) {
            if constexpr (sizeof(T) == 4)
                src.sums32 = reinterpret_cast<const float*>(B.sums);
            else
                src.sums = reinterpret_cast<const double*>(B.sums);
        }
        FEGB_TRY(launch_cg_q<T>(src, C, B.p + B.off[d] * L, L, B.q + B.off[d] * C,
                                B.pq_part + (size_t)B.pq_block_off[d] * C, P.s,
                                B.any_dense ? B.extra + B.off[d] * C : nullptr));
        P.projections += 1;
    }
    for (int sd = 0; sd < P.n_fe; ++sd) {
        if (!B.dense[sd] || !in_cg(sd)) continue;
        FinalizeParams src{};
        src.G = P.dims[sd].G;
        src.C = C;
        src.sums = B.dense_sums + B.dsum_off[sd];  // complete sums of -p, compact rows
        src.counts = P.dims[sd].counts;
        FEGB_TRY(launch_cg_q<T>(src, C, B.p + B.off[sd] * L, L, B.q + B.off[sd] * C,
                                B.pq_part + (size_t)B.pq_block_off[sd] * C, P.s));
        P.projections += 1;
    }
    return 0;
}

// One operator application q = A p with the p.q partials folded into B.pq:
// A = D'D, or in the Schur form A = D_R'(I - P_P) D_R over the non-primary
// dimensions R (P_P: projection on the primary's group means).
template <typename T>
int cg_apply(Problem& P, CGBuffers<T>& B) {
    bool prim_small_done = false;
    if (B.schur) FEGB_TRY(cg_schur_u<T>(P, B, &prim_small_done));
    FEGB_TRY(cg_apply_rest<T>(P, B, prim_small_done));
    return launch_fold_partials(B.pq_part, B.pq_blocks, P.C, B.pq, P.s);
}

// Start of an inner solve from the current FP64 group means (mu_all):
// standard form r = D'r_data = counts * mu; Schur form
// r = D_R'(I - P_P) r_data = counts_R * mu_R - D_R'D_P mu_P, obtained from the
// operator with x = 0 and the primary's slot of p = -mu_P.
template <typename T>
int cg_start(Problem& P, CGBuffers<T>& B) {
    const int C = P.C;
    const int L = B.ld;
    if (!B.schur)
        return launch_cg_init<T>(P.Gt, C, P.counts_all, P.mu_all, B.r, B.z, B.p, L, B.x, B.rz_part, B.zmax_part,
                                 B.zmax, P.s);
    const int pd = B.prim;
    FEGB_CUDA(cudaMemsetAsync(B.p, 0, sizeof(T) * (size_t)B.Gv * L, P.s), "cg p zero");
    FEGB_TRY(launch_table_from_f64<T>(P.mu_all + P.goff[pd] * C, P.dims[pd].G, C, -1.0, B.p + B.off[pd] * L, L,
                                      P.s));
    FEGB_TRY(cg_apply_rest<T>(P, B));
    for (int d = 0; d < P.n_fe; ++d)
        if (d != pd && P.dims[d].G > 0)
            FEGB_CUDA(cudaMemcpyAsync(B.mu_v + B.off[d] * C, P.mu_all + P.goff[d] * C,
                                      sizeof(double) * (size_t)P.dims[d].G * C, cudaMemcpyDeviceToDevice, P.s),
                      "cg means copy");
    return launch_cg_init_rhs<T>(B.Gv, C, B.counts_v, B.mu_v, B.q, B.inv, B.r, B.z, B.p, L, B.x, B.rz_part,
                                 B.zmax_part, B.zmax, P.s);
}

// End of an inner solve: the FE increments of x become the FP64 table applied
// by the next FP64 pass; in the Schur form the primary's increment is
// mu_P - u(x) (the group means of the residual after the others' increments).
template <typename T>
int cg_finish(Problem& P, CGBuffers<T>& B) {
    const int C = P.C;
    const int L = B.ld;
    if (!B.schur) return launch_to_f64<T>(B.x, C, P.alpha_all, C, P.Gt, P.s);
    const int pd = B.prim;
    for (int d = 0; d < P.n_fe; ++d)
        if (d != pd && P.dims[d].G > 0)
            FEGB_TRY(launch_to_f64<T>(B.x + B.off[d] * C, C, P.alpha_all + P.goff[d] * C, C, P.dims[d].G, P.s));
    FEGB_TRY(launch_table_from_compact<T>(B.x, B.Gv, C, B.p, L, P.s));
    FEGB_TRY(cg_schur_u<T>(P, B));
    return launch_alpha_primary<T>(P.mu_all + P.goff[pd] * C, B.p + B.off[pd] * L, P.dims[pd].G, C, L,
                                   P.alpha_all + P.goff[pd] * C, P.s);
}

// ---- graph-driven CG loop ----
// One CG iteration (operator, update, fold, convergence test, direction) is
// captured once per fit as the body of a conditional while-node; a one-thread
// kernel applies the host loop's stopping rules on the device and clears the
// node's condition, so the solve runs without a host round trip per
// iteration. Used whenever kernel timing (profile) is off.
struct CGLoopCtl {
    double tol;
    double best;
    double best_rz;
    double zm;
    int max_it;
    int it;
    int since_best;
    int stop;
};

__global__ void cg_loop_reset_kernel(CGLoopCtl* c, double tol, int max_it) {
    c->tol = tol;
    c->best = DBL_MAX;
    c->best_rz = DBL_MAX;
    c->zm = 0.0;
    c->max_it = max_it;
    c->it = 0;
    c->since_best = 0;
    c->stop = 0;
}

// Stopping rules of an inner solve (host and device loops alike): the largest
// preconditioned residual |z| below the tolerance ends it. Past the attainable
// accuracy of the storage type the recursive residual stops falling and then
// grows again (the iterate drifts away from its best); the solve ends there:
// when r.z (summed over the columns) rises above CG_DIVERGE times its best
// value, or after CG_STALL_ITERS iterations in which neither max |z| nor r.z
// fell below 0.9 of its best. max |z| alone can sit on a plateau for many
// iterations while r.z still falls.
constexpr int CG_STALL_ITERS = 60;
constexpr double CG_DIVERGE = 10.0;

__host__ __device__ inline bool cg_stop_rule(double zm, double rz, double tol, double* best, double* best_rz,
                                             int* since_best) {
    if (zm < tol) return true;
    if (rz > CG_DIVERGE * *best_rz) return true;
    bool progress = false;
    if (zm < 0.9 * *best) {
        *best = zm;
        progress = true;
    }
    if (rz < 0.9 * *best_rz) {
        *best_rz = rz;
        progress = true;
    }
    if (progress) {
        *since_best = 0;
        return false;
    }
    return ++*since_best > CG_STALL_ITERS;
}

__host__ __device__ inline double cg_rz_total(const double* rz, int C) {
    double t = 0.0;
    for (int c = 0; c < C; ++c) t += rz[c];
    return t;
}

__global__ void cg_loop_check_kernel(const unsigned long long* __restrict__ zmax_bits,
                                     const double* __restrict__ rz_new, int C, CGLoopCtl* c,
                                     cudaGraphConditionalHandle h) {
    const double zm = __longlong_as_double((long long)*zmax_bits);
    c->zm = zm;
    const int it = c->it + 1;
    c->it = it;
    bool stop = cg_stop_rule(zm, cg_rz_total(rz_new, C), c->tol, &c->best, &c->best_rz, &c->since_best);
    if (it >= c->max_it) stop = true;
    c->stop = stop ? 1 : 0;
    cudaGraphSetConditional(h, stop ? 0u : 1u);
}

template <typename T>
struct CGGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CGLoopCtl* ctl = nullptr;  // device
    ~CGGraph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

// Builds the loop graph; returns nonzero (and leaves G empty) when the driver
// refuses any step, in which case the caller keeps the host loop.
template <typename T>
int cg_build_graph(Problem& P, CGBuffers<T>& B, CGGraph<T>& G) {
    if (cudaGraphCreate(&G.graph, 0) != cudaSuccess) return 1;
    cudaGraphConditionalHandle h;
    if (cudaGraphConditionalHandleCreate(&h, G.graph, 1, cudaGraphCondAssignDefault) != cudaSuccess) return 1;
    // the parameter struct has no default constructor: zeroed storage, as the API requires
    alignas(cudaGraphNodeParams) unsigned char npbuf[sizeof(cudaGraphNodeParams)];
    std::memset(npbuf, 0, sizeof(npbuf));
    cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(npbuf);
    np.type = cudaGraphNodeTypeConditional;
    np.conditional.handle = h;
    np.conditional.type = cudaGraphCondTypeWhile;
    np.conditional.size = 1;
    cudaGraphNode_t node;
    if (cudaGraphAddNode(&node, G.graph, nullptr, nullptr, 0, &np) != cudaSuccess) return 1;
    cudaGraph_t body = np.conditional.phGraph_out[0];
    cudaStream_t cs = nullptr;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return 1;
    if (cudaStreamBeginCaptureToGraph(cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
        cudaStreamDestroy(cs);
        return 1;
    }
    cudaStream_t saved = P.s;
    P.s = cs;
    const int C = P.C;
    int st = cg_apply<T>(P, B);
    if (!st)
        st = launch_cg_update<T>(B.Gv, C, B.inv, B.rz, B.pq, B.p, B.ld, B.q, B.x, B.r, B.z, B.rz_part, B.zmax_part,
                                 B.zmax, cs);
    if (!st) st = launch_fold_partials(B.rz_part, B.rz_blocks, C, B.rz_new, cs);
    if (!st) {
        cg_loop_check_kernel<<<1, 1, 0, cs>>>(B.zmax, B.rz_new, C, G.ctl, h);
        count_launch();
        if (cudaPeekAtLastError() != cudaSuccess) st = 1;
    }
    if (!st) st = launch_cg_direction<T>(B.Gv, C, B.rz, B.rz_new, B.z, B.p, B.ld, cs, &G.ctl->stop);
    P.s = saved;
    cudaGraph_t captured = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(cs, &captured);
    cudaStreamDestroy(cs);
    if (st || ec != cudaSuccess) return 1;
    if (cudaGraphInstantiate(&G.exec, G.graph, 0) != cudaSuccess) return 1;
    return 0;
}

template <typename T>
int cg_solve_host(Problem& P, CGBuffers<T>& B, double inner_tol, int max_it, int* iters, double* zmax_out);

// Preconditioned (group-count) CG on D'D delta = D'r, r = current FP64
// residual whose group means are in mu_all; delta accumulates into alpha_all.
// With a loop graph the iterations run on the device (same stopping rules).
template <typename T>
int cg_solve(Problem& P, CGBuffers<T>& B, double inner_tol, int max_it, int* iters, double* zmax_out,
             CGGraph<T>* G = nullptr) {
    if (G && G->exec && max_it > 0) {
        const int C = P.C;
        FEGB_TRY(cg_start<T>(P, B));
        FEGB_TRY(launch_fold_partials(B.rz_part, B.rz_blocks, C, B.rz, P.s));
        cg_loop_reset_kernel<<<1, 1, 0, P.s>>>(G->ctl, inner_tol, max_it);
        FEGB_LAUNCH_CHECK("cg loop reset");
        FEGB_CUDA(cudaGraphLaunch(G->exec, P.s), "cg loop graph launch");
        CGLoopCtl h;
        FEGB_TRY(d2h_sync(&h, G->ctl, sizeof(h), P.s, "cg loop state copy"));
        *iters = h.it;
        *zmax_out = h.zm;
        return cg_finish<T>(P, B);
    }
    return cg_solve_host<T>(P, B, inner_tol, max_it, iters, zmax_out);
}

template <typename T>
int cg_solve_host(Problem& P, CGBuffers<T>& B, double inner_tol, int max_it, int* iters, double* zmax_out) {
    const int C = P.C;  // vector ops run over compact rows; p keeps the padded stride B.ld
    FEGB_TRY(cg_start<T>(P, B));
    FEGB_TRY(launch_fold_partials(B.rz_part, B.rz_blocks, C, B.rz, P.s));
    double best = DBL_MAX, best_rz = DBL_MAX;
    int since_best = 0;
    int it = 0;
    double zm = 0.0;
    std::vector<double> rz_host((size_t)C);
    for (; it < max_it; ++it) {
        FEGB_TRY(cg_apply<T>(P, B));
        FEGB_TRY(launch_cg_update<T>(B.Gv, C, B.inv, B.rz, B.pq, B.p, B.ld, B.q, B.x, B.r, B.z, B.rz_part,
                                     B.zmax_part, B.zmax, P.s));
        FEGB_TRY(launch_fold_partials(B.rz_part, B.rz_blocks, C, B.rz_new, P.s));
        FEGB_CUDA(cudaMemcpyAsync(rz_host.data(), B.rz_new, sizeof(double) * C, cudaMemcpyDeviceToHost, P.s),
                  "cg r.z copy");
        unsigned long long bits = 0;
        FEGB_TRY(d2h_sync(&bits, B.zmax, sizeof(bits), P.s, "cg zmax copy"));
        zm = bits_to_double(bits);
        if (trace_level() >= 2 && it % 10 == 0)
            std::fprintf(stderr, "fegb cg:   iteration %d max |z| %.3e r.z %.3e\n", it, zm,
                         cg_rz_total(rz_host.data(), C));
        if (cg_stop_rule(zm, cg_rz_total(rz_host.data(), C), inner_tol, &best, &best_rz, &since_best)) {
            ++it;
            break;
        }
        FEGB_TRY(launch_cg_direction<T>(B.Gv, C, B.rz, B.rz_new, B.z, B.p, B.ld, P.s));
    }
    *iters = it;
    *zmax_out = zm;
    return cg_finish<T>(P, B);
}

// FP64 refinement loop around a CG inner solve in storage type T.
template <typename T>
int demean_cg(Problem& P, double tol, int max_iter, int* iterations, int* converged, double* max_update, int* outer) {
    *iterations = 0;
    *converged = 1;
    *max_update = 0.0;
    *outer = 0;
    if (P.n_fe == 0 || P.n == 0) return 0;
    CGBuffers<T> B;
    FEGB_TRY(cg_alloc<T>(P, B));
    CGGraph<T> G;
    bool use_graph = false;
    if (!P.profile && tuning(TUNE_CG_GRAPH)) {
        FEGB_TRY(dalloc(*P.scr, &G.ctl, 1, "cg loop state"));
        use_graph = cg_build_graph<T>(P, B, G) == 0;
        if (!use_graph) {
            cudaGetLastError();  // the host loop takes over
            set_ok();
        }
    }
    const int max_outer = 12;
    double mu = 0.0, mu_prev = DBL_MAX;
    int total = 0, hit = 0;
    bool apply_alpha = false;
    for (int round = 0; round < max_outer; ++round) {
        FEGB_TRY(fp64_mean_pass(P, apply_alpha, &mu));
        *outer = round + 1;
        if (trace_enabled() && (mu < tol || round + 1 == max_outer))
            std::fprintf(stderr, "fegb cg: outer %d max group mean %.3e (tolerance %.1e)\n", round + 1, mu, tol);
        if (mu < tol) {
            hit = 1;
            break;
        }
        if (total >= max_iter) break;
        if (round > 2 && mu > 0.5 * mu_prev) break;
        mu_prev = mu;
        const double inner_tol =
            sizeof(T) == 4 ? std::max(0.5 * tol, 2e-6 * mu) : std::max(0.5 * tol, 1e-12 * mu);
        int it = 0;
        double zm = 0.0;
        FEGB_TRY(cg_solve<T>(P, B, inner_tol, max_iter - total, &it, &zm, use_graph ? &G : nullptr));
        if (trace_enabled())
            std::fprintf(stderr, "fegb cg: outer %d max group mean %.3e inner tol %.3e: %d iterations, max |z| %.3e\n",
                         round + 1, mu, inner_tol, it, zm);
        total += it;
        apply_alpha = true;
    }
    if (sizeof(T) == 4 && B.any_dense) {
        // the tensor-core count-matrix passes record a wait that ran out of time
        int umma_err = 0;
        FEGB_TRY(dense_umma_error(&umma_err, true, P.s));
        if (umma_err) return set_error("CG operator: a tensor-core count-matrix pass timed out waiting on its copies");
    }
    *iterations = total;
    *converged = hit;
    *max_update = mu;
    return 0;
}

// ------------------------------ estimator ---------------------------------

struct Stats {
    double rss = 0, tss_total = 0, tss_within = 0;
};

// fe_pipeline.f90:1963-2008
void finalize_stats(fegb_result* r, long long n_obs) {
    const double EPS = 1e-12;
    double n = (double)std::max(1LL, n_obs);
    double df_model = (double)std::max(0, r->dof_model);
    double df_resid = (double)std::max(1LL, r->dof_resid);
    double dev = r->rss;
    double dev0 = std::max(EPS, r->tss_total);
    if (dev0 > EPS) {
        r->r2 = std::max(0.0, std::min(1.0, 1.0 - dev / dev0));
    } else {
        r->r2 = 0.0;
    }
    if (r->tss_within > EPS)
        r->r2_within = std::max(0.0, std::min(1.0, 1.0 - dev / r->tss_within));
    else
        r->r2_within = r->r2;
    double k_total = (double)(r->dof_model + r->dof_fes + 1);
    double denom = std::max(n - k_total, 1.0);
    if (n > 1.0 && dev0 > EPS)
        r->r2_adj = std::max(0.0, std::min(1.0, 1.0 - (dev * (n - 1.0)) / (dev0 * denom)));
    else
        r->r2_adj = r->r2;
    double ssr = std::max(0.0, dev0 - dev);
    if (df_model > 0.0 && df_resid > 0.0 && dev > EPS)
        r->f_stat = (ssr / df_model) / (dev / df_resid);
    else
        r->f_stat = 0.0;
}

__global__ void tss_partials_kernel(const double* __restrict__ y, long long n, double mean, double* partials,
                                    double* sums) {
    __shared__ double red[256 / 32];
    double a = 0.0;
    long long i = (long long)blockIdx.x * 256 + threadIdx.x;
    const long long st = (long long)gridDim.x * 256;
    for (; i < n; i += st) a += sums ? y[i] : (y[i] - mean) * (y[i] - mean);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double v = 0.0;
        for (int w = 0; w < 8; ++w) v += red[w];
        (sums ? sums : partials)[blockIdx.x] = v;
    }
}

// Total sum of squares around the mean of the raw y (compute_tss,
// fe_pipeline.f90:1935-1955), with a fixed reduction order.
int compute_tss_dev(const double* y, long long n, double* out, cudaStream_t s, Scratch& scr) {
    *out = 0.0;
    if (n <= 0) return 0;
    int nb = (int)std::min<long long>((long long)num_sms() * 4, (n + 255) / 256);
    double* part = nullptr;
    FEGB_TRY(scr.alloc(&part, (size_t)nb, "tss partials"));
    std::vector<double> h(nb);
    tss_partials_kernel<<<nb, 256, 0, s>>>(y, n, 0.0, nullptr, part);
    FEGB_LAUNCH_CHECK("tss sum");
    FEGB_TRY(d2h_sync(h.data(), part, sizeof(double) * nb, s, "tss sum copy"));
    double sum = 0.0;
    for (double v : h) sum += v;
    double mean = sum / (double)n;
    tss_partials_kernel<<<nb, 256, 0, s>>>(y, n, mean, part, nullptr);
    FEGB_LAUNCH_CHECK("tss");
    FEGB_TRY(d2h_sync(h.data(), part, sizeof(double) * nb, s, "tss copy"));
    double t = 0.0;
    for (double v : h) t += v;
    *out = t;
    return 0;
}

// Cluster-score sums of S (n x ns AoS, storage order) over the groups of one
// cluster subset; writes Sc (n_cl x ns).
// bit of FE dimension d (0-based) in a cluster-subset mask over cdims (1-based dims)
inline int ia_mask_bit(const std::vector<int>& cdims, int d) {
    for (size_t j = 0; j < cdims.size(); ++j)
        if (cdims[j] - 1 == d) return (int)j;
    return 0;
}

int cluster_score_sums(Problem& P, const double* S, int ns, const int32_t* perm, const int32_t* gseq,
                       const int32_t* off, int n_cl, double* Sc, Scratch& scr, long long npos, int timed_kind,
                       bool persistent_off, const FinalizeParams* outputs) {
    SegSweepParams<double> sp{};
    sp.X = const_cast<double*>(S);
    sp.rs = ns;
    sp.cs = 1;
    sp.C = ns;
    sp.n = npos >= 0 ? npos : P.n;
    sp.perm = perm;
    sp.gseq = gseq;
    sp.pend.n = 0;
    sp.writeback = 0;
    sp.R = CHUNK_R;
    long long nchunks = std::max(1LL, seg_nchunks(sp.n, CHUNK_R));
    double *sums = nullptr, *head = nullptr, *tail = nullptr;
    FEGB_TRY(scr.alloc(&sums, (size_t)std::max(1, n_cl) * ns, "score sums"));
    FEGB_TRY(scr.alloc(&head, (size_t)nchunks * ns, "score heads"));
    FEGB_TRY(scr.alloc(&tail, (size_t)nchunks * ns, "score tails"));
    sp.sums = sums;
    sp.head = head;
    sp.tail = tail;
    int32_t* long_list = nullptr;
    int n_long = 0;
    bool cached = false;
    if (persistent_off)
        for (const auto& c : P.long_cache)
            if (c.off == off && c.G == n_cl) {
                long_list = c.list;
                n_long = c.n;
                cached = true;
            }
    if (!cached) {
        Scratch& where = persistent_off ? *P.scr : scr;
        FEGB_TRY(where.alloc(&long_list, (size_t)std::max(1, n_cl), "score long groups"));
        FEGB_TRY(find_long_groups(off, n_cl, CHUNK_R, long_list, &n_long, P.s));
        if (persistent_off) P.long_cache.push_back({off, n_cl, long_list, n_long});
    }
    // outputs: the finalize's other outputs (means, maxima), its sources set here
    FinalizeParams f = outputs ? *outputs : FinalizeParams{};
    f.G = n_cl;
    f.C = ns;
    f.off = off;
    f.sums = sums;
    f.head = head;
    f.tail = tail;
    f.R = CHUNK_R;
    f.partials = nullptr;
    f.sum_out = Sc;
    CGTimer tm(P);
    if (timed_kind >= 0)
        FEGB_TRY(tm.begin(timed_kind, (double)sp.n * (4.0 + (perm ? 4.0 : 0.0) + 8.0 * ns)));
    FEGB_TRY(launch_seg_sweep<double>(sp, P.s));
    FEGB_TRY(tm.end());
    FEGB_TRY(launch_long_sums(off, head, tail, CHUNK_R, ns, long_list, n_long, sums, P.s));
    return launch_finalize(f, P.s);
}

// Complete per-tuple sums of the rows (m x C) written in place: runs inside a
// chunk come straight from the sweep, the chunk-crossing ones are completed by
// the group-sum pass (no finalize copy). The tuples' offsets are persistent,
// so their group lists are found once.
int tuple_row_sums(Problem& P, const double* X, int C, double* out, Scratch& scr, int timed_kind) {
    const int G = P.tuple_m;
    const int32_t* off = P.tuple_off;
    Problem::LongCache* c = nullptr;
    for (auto& e : P.long_cache)
        if (e.off == off && e.G == G) c = &e;
    if (!c) {
        Problem::LongCache e{off, G, nullptr, 0};
        FEGB_TRY(P.scr->alloc(&e.list, (size_t)std::max(1, G), "tuple long groups"));
        FEGB_TRY(find_long_groups(off, G, CHUNK_R, e.list, &e.n, P.s));
        P.long_cache.push_back(e);
        c = &P.long_cache.back();
    }
    if (!c->multi) {
        FEGB_TRY(P.scr->alloc(&c->multi, (size_t)std::max(1, G), "tuple multi-chunk groups"));
        FEGB_TRY(find_multi_groups(off, G, CHUNK_R, c->multi, &c->n_multi, P.s));
    }
    SegSweepParams<double> sp{};
    sp.X = const_cast<double*>(X);
    sp.rs = C;
    sp.cs = 1;
    sp.C = C;
    sp.n = P.n;
    sp.perm = P.tuple_perm;
    sp.gseq = P.tuple_gseq;
    sp.R = CHUNK_R;
    const long long nchunks = std::max(1LL, seg_nchunks(P.n, CHUNK_R));
    FEGB_TRY(scr.alloc(&sp.head, (size_t)nchunks * C, "tuple heads"));
    FEGB_TRY(scr.alloc(&sp.tail, (size_t)nchunks * C, "tuple tails"));
    sp.sums = out;
    CGTimer tm(P);
    if (timed_kind >= 0) FEGB_TRY(tm.begin(timed_kind, (double)P.n * (8.0 + 8.0 * C)));
    FEGB_TRY(launch_seg_sweep<double>(sp, P.s));
    FEGB_TRY(tm.end());
    return launch_group_sums<double>(off, sp.head, sp.tail, CHUNK_R, C, c->list, c->n, c->multi, c->n_multi, out,
                                     P.s);
}

struct FitTimes {
    double prep = 0, demean = 0, regression = 0, se = 0;
};

// Within-transform done outside the fit (the batched path demeans many
// specifications together and estimates each on its own rows).
struct PreDemeaned {
    int iterations = 0;
    int converged = 1;
    int outer = 0;
    double max_update = 0.0;
    double seconds = 0.0;
    int projections = 0;
    double demean_bytes = 0.0;
    fegb_result prof{};  // sweep-family timings of the shared within-transform (when profiling)
    bool carry_profile = false;  // copy them into the result of the fit that uses this state
};

int estimate_on_problem(Problem& P, const fegb_config& cfg, const int* G_all, long long n_raw, double tss_total,
                        double* beta_out, double* se_out, fegb_result* res, FitTimes& tm,
                        const PreDemeaned* pre = nullptr) {
    cudaStream_t s = P.s;
    Scratch& scr = *P.scr;
    const int k = P.k, l = P.l, C = P.C, n_fe = P.n_fe;
    const long long n = P.n;
    const bool cpu_conv = cfg.se_convention == FEGB_SE_CPU;
    for (int j = 0; j < k; ++j) {
        beta_out[j] = 0.0;
        se_out[j] = 0.0;
    }
    res->tss_total = tss_total;
    int dof_fes = 0;
    for (int d = 0; d < n_fe; ++d) dof_fes += std::max(0, G_all[d] - 1);
    res->dof_fes = dof_fes;
    // cluster dims: valid, unique, first three (fe_pipeline.f90:1553-1599, 305-346)
    std::vector<int> cdims;
    for (int i = 0; i < cfg.n_cluster_dims; ++i) {
        int v = cfg.cluster_dims[i];
        if (v < 1 || v > n_fe) continue;
        if (std::find(cdims.begin(), cdims.end(), v) != cdims.end()) continue;
        if ((int)cdims.size() == MAX_CLUSTER_DIMS) break;
        cdims.push_back(v);
    }
    int nested = 0;
    for (int v : cdims) nested += std::max(0, G_all[v - 1] - 1);

    // ---------------- within-transform ----------------
    auto t0 = Clock::now();
    int iters = 0, conv = 1, outer = 0;
    double mu = 0.0;
    if (pre) {
        iters = pre->iterations;
        conv = pre->converged;
        outer = pre->outer;
        mu = pre->max_update;
    } else if (cfg.demean_method == FEGB_DEMEAN_CG) {
        if (cfg.precision == FEGB_PREC_MIXED)
            FEGB_TRY(demean_cg<float>(P, cfg.fe_tol, cfg.fe_max_iter, &iters, &conv, &mu, &outer));
        else
            FEGB_TRY(demean_cg<double>(P, cfg.fe_tol, cfg.fe_max_iter, &iters, &conv, &mu, &outer));
    } else if (cfg.precision == FEGB_PREC_MIXED) {
        FEGB_TRY(demean_mixed(P, cfg.fe_tol, cfg.fe_max_iter, &iters, &conv, &mu, &outer));
    } else {
        FEGB_TRY(demean_plain(P, cfg.fe_tol, cfg.fe_max_iter, &iters, &conv, &mu));
    }
    FEGB_CUDA(cudaStreamSynchronize(s), "demean sync");
    tm.demean = pre ? pre->seconds : seconds_since(t0);
    FEGB_TRY(collect_profile(P, res));
    res->converged = conv;
    res->fe_iterations = iters;
    res->max_update = mu;
    res->outer_iterations = outer;
    res->projections = P.projections;
    res->demean_bytes = P.demean_bytes;
    if (pre) {
        res->projections = pre->projections;
        res->demean_bytes = pre->demean_bytes;
        if (pre->carry_profile) {
            for (int f = 0; f < 8; ++f) {
                res->prof_launches[f] = pre->prof.prof_launches[f];
                res->prof_seconds[f] = pre->prof.prof_seconds[f];
                res->prof_bytes[f] = pre->prof.prof_bytes[f];
            }
        }
    }
    if (k <= 0) return 0;

    // ---------------- normal equations ----------------
    t0 = Clock::now();
    double* gram = nullptr;
    FEGB_TRY(scr.alloc(&gram, (size_t)C * C, "gram"));
    MatView xv{P.X, C, 1, C};
    FEGB_TRY(crossprod_auto(xv, xv, n, true, false, 1.0, 0.0, gram, C, s, scr));
    std::vector<double> hg((size_t)C * C);
    FEGB_TRY(d2h_sync(hg.data(), gram, sizeof(double) * C * C, s, "gram copy"));
    auto Gm = [&](int i, int j) { return hg[(size_t)i + (size_t)j * C]; };
    res->tss_within = Gm(0, 0);
    std::vector<double> vdiag(k);
    for (int j = 0; j < k; ++j) vdiag[j] = Gm(1 + j, 1 + j);

    // endogenous / instruments (fe_pipeline.f90:672-746)
    std::vector<int> is_endog(k, 0);
    if (!cpu_conv)
        for (int i = 0; i < cfg.n_iv_regressors; ++i) {
            int v = cfg.iv_regressors[i];
            if (v >= 1 && v <= k) is_endog[v - 1] = 1;
        }
    int n_endog = 0;
    for (int v : is_endog) n_endog += v;
    std::vector<int> sel;
    if (l > 0 && !cpu_conv) {
        for (int i = 0; i < cfg.n_iv_instruments; ++i) {
            int v = cfg.iv_instruments[i];
            if (v >= 1 && v <= l) sel.push_back(v);
        }
        if (sel.empty())
            for (int i = 1; i <= l; ++i) sel.push_back(i);
    }
    bool use_iv = n_endog > 0 && (int)sel.size() >= n_endog;
    std::vector<int> za;  // X columns of Z_aug = [exogenous W, selected Z]
    if (use_iv) {
        for (int j = 0; j < k; ++j)
            if (!is_endog[j]) za.push_back(1 + j);
        for (int v : sel) za.push_back(1 + k + (v - 1));
    }
    const int na = (int)za.size();
    res->is_iv = use_iv ? 1 : 0;
    res->n_instruments = use_iv ? na : 0;

    int kmax = std::max(k, std::max(na, 1));
    double *Q = nullptr, *b = nullptr, *work = nullptr, *Pi = nullptr;
    int* info_dev = nullptr;
    FEGB_TRY(scr.alloc(&Q, (size_t)k * k, "Q"));
    FEGB_TRY(scr.alloc(&b, (size_t)k, "b"));
    FEGB_TRY(scr.alloc(&work, (size_t)4 * kmax * kmax, "dense work"));
    FEGB_TRY(scr.alloc(&info_dev, 4, "info"));
    // Q = W'W, b = W'y from the Gram block
    {
        std::vector<double> hQ((size_t)k * k), hb(k);
        for (int i = 0; i < k; ++i) {
            hb[i] = Gm(1 + i, 0);
            for (int j = 0; j < k; ++j) hQ[(size_t)i + (size_t)j * k] = Gm(1 + i, 1 + j);
        }
        FEGB_TRY(h2d_sync(Q, hQ.data(), sizeof(double) * k * k, s, "Q upload"));
        FEGB_TRY(h2d_sync(b, hb.data(), sizeof(double) * k, s, "b upload"));
    }
    if (use_iv) {
        // build_iv_normal_equations (fe_pipeline.f90:947-1032)
        double *Qzz = nullptr, *Qzy = nullptr, *Qzx = nullptr, *rhs = nullptr, *Qinv_zz = nullptr;
        FEGB_TRY(scr.alloc(&Qzz, (size_t)na * na, "Qzz"));
        FEGB_TRY(scr.alloc(&Qzy, (size_t)na, "Qzy"));
        FEGB_TRY(scr.alloc(&Qzx, (size_t)na * k, "Qzx"));
        FEGB_TRY(scr.alloc(&rhs, (size_t)na, "iv rhs"));
        FEGB_TRY(scr.alloc(&Qinv_zz, (size_t)na * na, "Qzz inverse"));
        FEGB_TRY(scr.alloc(&Pi, (size_t)na * k, "projection"));
        std::vector<double> hzz((size_t)na * na), hzy(na), hzx((size_t)na * k);
        for (int i = 0; i < na; ++i) {
            hzy[i] = Gm(za[i], 0);
            for (int j = 0; j < na; ++j) hzz[(size_t)i + (size_t)j * na] = Gm(za[i], za[j]);
            for (int j = 0; j < k; ++j) hzx[(size_t)i + (size_t)j * na] = Gm(za[i], 1 + j);
        }
        FEGB_TRY(h2d_sync(Qzz, hzz.data(), sizeof(double) * na * na, s, "Qzz upload"));
        FEGB_TRY(h2d_sync(Qzy, hzy.data(), sizeof(double) * na, s, "Qzy upload"));
        FEGB_TRY(h2d_sync(Qzx, hzx.data(), sizeof(double) * na * k, s, "Qzx upload"));
        FEGB_TRY(dense_chol_solve_inv(na, Qzz, na, nullptr, Qzy, rhs, Qinv_zz, info_dev, work, s));
        int info = 0;
        FEGB_TRY(d2h_sync(&info, info_dev, sizeof(int), s, "iv info"));
        if (info != 0) {
            res->solver_info = info;
            return 0;
        }
        FEGB_TRY(dense_gemm(false, false, na, k, na, 1.0, Qinv_zz, na, Qzx, na, 0.0, Pi, na, s));
        // Q = 0.5 (T + T^T)
        FEGB_TRY(dense_gemm(true, false, k, k, na, 0.5, Qzx, na, Pi, na, 0.0, Q, k, s));
        FEGB_TRY(dense_gemm(true, false, k, k, na, 0.5, Pi, na, Qzx, na, 1.0, Q, k, s));
        FEGB_TRY(dense_gemm(true, false, k, 1, na, 1.0, Qzx, na, rhs, na, 0.0, b, k, s));
    }
    // column filter (fe_pipeline.f90:1034-1107); the CPU path keeps every column
    std::vector<int> kept;
    {
        double dmax = 0.0;
        for (int j = 0; j < k; ++j) dmax = std::max(dmax, std::fabs(vdiag[j]));
        dmax = std::max(dmax, 1.0);
        double tol = 1.0e-10 * dmax;
        for (int j = 0; j < k; ++j)
            if (cpu_conv || !(std::fabs(vdiag[j]) <= tol)) kept.push_back(j);
    }
    const int kk = (int)kept.size();
    res->dof_model = kk;
    if (kk == 0) {
        res->solver_info = -1;
        return 0;
    }
    int* idx_dev = nullptr;
    double *beta_sel = nullptr, *Qinv = nullptr, *beta_full = nullptr;
    FEGB_TRY(scr.alloc(&idx_dev, (size_t)kk, "kept idx"));
    FEGB_TRY(scr.alloc(&beta_sel, (size_t)kk, "beta sel"));
    FEGB_TRY(scr.alloc(&Qinv, (size_t)kk * kk, "Qinv"));
    FEGB_TRY(scr.alloc(&beta_full, (size_t)k, "beta"));
    FEGB_TRY(h2d_sync(idx_dev, kept.data(), sizeof(int) * kk, s, "idx upload"));
    FEGB_TRY(dense_chol_solve_inv(kk, Q, k, idx_dev, b, beta_sel, Qinv, info_dev, work, s));
    int info = 0;
    FEGB_TRY(d2h_sync(&info, info_dev, sizeof(int), s, "solve info"));
    res->solver_info = info;
    if (info != 0) return 0;
    std::vector<double> hbeta(kk);
    FEGB_TRY(d2h_sync(hbeta.data(), beta_sel, sizeof(double) * kk, s, "beta copy"));
    for (int t = 0; t < kk; ++t) beta_out[kept[t]] = hbeta[t];
    res->rank = kk;
    FEGB_TRY(h2d_sync(beta_full, beta_out, sizeof(double) * k, s, "beta upload"));
    tm.regression = seconds_since(t0);

    // ---------------- residual, scores and SEs ----------------
    t0 = Clock::now();
    const bool clusters = !cdims.empty();
    std::vector<int> score_cols;
    if (use_iv)
        score_cols = za;
    else
        for (int j = 0; j < k; ++j) score_cols.push_back(1 + j);
    const int ns = (int)score_cols.size();
    int* score_cols_dev = nullptr;
    double *S = nullptr, *rss_dev = nullptr;
    FEGB_TRY(scr.alloc(&score_cols_dev, (size_t)ns, "score cols"));
    FEGB_TRY(scr.alloc(&rss_dev, 1, "rss"));
    FEGB_TRY(h2d_sync(score_cols_dev, score_cols.data(), sizeof(int) * ns, s, "score cols upload"));
    if (clusters) FEGB_TRY(scr.alloc(&S, (size_t)n * ns, "score rows"));
    FEGB_TRY(residual_scores(P.X, C, n, beta_full, k, score_cols_dev, ns, S, nullptr, rss_dev, s, scr));
    double rss = 0.0;
    FEGB_TRY(d2h_sync(&rss, rss_dev, sizeof(double), s, "rss copy"));
    res->rss = rss;
    long long df;
    if (cpu_conv) {
        df = n - k;  // fe_pipeline.f90:187
    } else {
        long long pc = (long long)std::max(0, res->dof_model) + std::max(0, res->dof_fes) + 1;
        df = std::max(1LL, n - pc);  // fe_pipeline.f90:1171-1176
    }
    res->dof_resid = df;
    double sigma2 = cpu_conv ? rss / std::max(1.0, (double)(n - k)) : rss / (double)df;
    bool cluster_ok = false;
    if (clusters) {
        cluster_ok = true;
        double* acc = nullptr;
        double* meat = nullptr;
        double* meat_k = nullptr;
        double* se_sel = nullptr;
        int* psd_dev = nullptr;
        FEGB_TRY(scr.alloc(&acc, (size_t)kk * kk, "cov acc"));
        FEGB_TRY(scr.alloc(&meat, (size_t)ns * ns, "meat"));
        FEGB_TRY(scr.alloc(&meat_k, (size_t)k * k, "meat k"));
        FEGB_TRY(scr.alloc(&se_sel, (size_t)kk, "se sel"));
        FEGB_TRY(scr.alloc(&psd_dev, 1, "psd"));
        FEGB_CUDA(cudaMemsetAsync(acc, 0, sizeof(double) * kk * kk, s), "acc zero");
        const int ncd = (int)cdims.size();
        long long min_single = LLONG_MAX;
        // subsets whose clusters are single rows, and the meat S'S they all share
        std::vector<int> row_masks;
        double* meat_rows = nullptr;
        // score sums per CG tuple (m x ns), formed once when a subset needs them
        double* tuple_scores = nullptr;
        auto tuple_sums = [&]() -> int {
            if (tuple_scores) return 0;
            FEGB_TRY(scr.alloc(&tuple_scores, (size_t)P.tuple_m * ns, "tuple scores"));
            Scratch ts(s);
            FEGB_TRY(tuple_row_sums(P, S, ns, tuple_scores, ts, -1));
            FEGB_CUDA(cudaStreamSynchronize(s), "tuple scores sync");
            return 0;
        };
        for (int mask = 1; mask < (1 << ncd) && cluster_ok; ++mask) {
            std::vector<int> sd;
            for (int j = 0; j < ncd; ++j)
                if (mask & (1 << j)) sd.push_back(cdims[j] - 1);
            const int m = (int)sd.size();
            Scratch sub(s);
            const int32_t *perm = nullptr, *gseq = nullptr, *off = nullptr;
            int n_cl = 0;
            bool rows = false;  // every cluster of this subset is one row
            for (int u : row_masks) rows = rows || (mask & u) == u;
            if (!rows && m > 1) {
                // a pair with a dimension of at most 64 groups: one pass tells whether its pairs are unique
                for (int ia = 0; ia < m && !rows; ++ia)
                    for (int ib = 0; ib < m && !rows; ++ib) {
                        const int a = sd[ia], b = sd[ib];
                        if (a == b || P.dims[b].G > 64 || P.dims[a].G <= 0) continue;
                        if (!P.pair_max.empty() && P.pair_max[a][b] >= 0) {
                            // the CG's count matrix of this pair already tells
                            if (P.pair_max[a][b] <= 1) {
                                rows = true;
                                row_masks.push_back((1 << ia_mask_bit(cdims, a)) | (1 << ia_mask_bit(cdims, b)));
                            }
                            continue;
                        }
                        unsigned long long* seen = nullptr;
                        int* hit = nullptr;
                        FEGB_TRY(sub.alloc(&seen, (size_t)P.dims[a].G, "pair masks"));
                        FEGB_TRY(sub.alloc(&hit, 1, "pair hit"));
                        FEGB_CUDA(cudaMemsetAsync(seen, 0, sizeof(unsigned long long) * P.dims[a].G, s), "pair masks");
                        FEGB_CUDA(cudaMemsetAsync(hit, 0, sizeof(int), s), "pair hit");
                        pair_collision_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(P.dims[a].gid, P.dims[b].gid,
                                                                                         n, seen, hit);
                        FEGB_LAUNCH_CHECK("pair uniqueness");
                        int h = 1;
                        FEGB_TRY(d2h_sync(&h, hit, sizeof(int), s, "pair hit copy"));
                        if (!h) {
                            rows = true;
                            row_masks.push_back((1 << ia_mask_bit(cdims, a)) | (1 << ia_mask_bit(cdims, b)));
                        }
                    }
            }
            const bool smallg_single = m == 1 && !rows && P.dims[sd[0]].mode == MODE_SMALLG &&
                                       smallg_eligible(P.dims[sd[0]].G, ns);
            bool tuples = m > 1 && P.tuple_m > 0 && P.tuple_n == n && P.tuple_dims.size() == sd.size();
            if (tuples) {
                std::vector<int> sds(sd);
                std::sort(sds.begin(), sds.end());
                for (size_t j = 0; j < sds.size() && tuples; ++j)
                    tuples = sds[j] == P.tuple_dims[j] && P.dims[sds[j]].gid == P.tuple_gid[j];
            }
            // a single dimension of the tuples: its clusters' sums from the tuples' sums
            const bool tuple_single = m == 1 && !rows && !smallg_single && P.tuple_m > 0 && P.tuple_n == n &&
                                      (size_t)sd[0] < P.tuple_dim_gseq.size() && P.tuple_dim_gseq[sd[0]] &&
                                      P.tuple_dim_off[sd[0]];
            if (rows && m > 1) {
                n_cl = (int)n;  // a refinement of single-row clusters: no sort needed
            } else if (tuple_single) {
                n_cl = P.dims[sd[0]].G;
            } else if (tuples) {
                // the clusters are the CG operator's id tuples: its row sort serves
                perm = P.tuple_perm;
                gseq = P.tuple_gseq;
                off = P.tuple_off;
                n_cl = P.tuple_m;
            } else if (smallg_single) {
                n_cl = P.dims[sd[0]].G;  // sums from per-block tables in storage order, no sort
            } else if (m == 1 && P.dims[sd[0]].mode != MODE_SMALLG) {
                const Dim& D = P.dims[sd[0]];
                perm = D.mode == MODE_GATHER ? D.perm : nullptr;
                gseq = D.gseq;
                off = D.off;
                n_cl = D.G;
            } else {
                // intersection (or small-G single) clusters: sort rows by key
                std::vector<const int32_t*> ptrs;
                std::vector<unsigned long long> strides;
                unsigned long long stride = 1;
                bool fits = true;
                for (int d : sd) {
                    ptrs.push_back(P.dims[d].gid);
                    strides.push_back(stride);
                    unsigned long long Gd = (unsigned long long)std::max(1, P.dims[d].G);
                    if (stride > (1ULL << 62) / Gd) fits = false;
                    stride *= Gd;
                }
                if (!fits) {
                    set_error("cluster key span exceeds 2^62 for a %d-way subset", m);
                    cluster_ok = false;
                    break;
                }
                int32_t *pm = nullptr, *gs = nullptr, *of = nullptr;
                FEGB_TRY(sub.alloc(&pm, (size_t)n, "cluster perm"));
                FEGB_TRY(sub.alloc(&gs, (size_t)n, "cluster gseq"));
                FEGB_TRY(sub.alloc(&of, (size_t)n + 1, "cluster offsets"));
                FEGB_TRY(cluster_ids_by_key(ptrs.data(), strides.data(), m, n, bits_for(stride), nullptr, &n_cl, pm,
                                            of, s, sub, true, gs));
                perm = pm;
                gseq = gs;
                off = of;
                if (m == 1 && !cpu_conv) n_cl = P.dims[sd[0]].G;  // ids equal FE ids; empty groups add nothing
                if (m == 1 && !cpu_conv) {
                    // offsets must cover G groups: rebuild from the FE counts when groups are empty
                    int32_t* of2 = nullptr;
                    FEGB_TRY(sub.alloc(&of2, (size_t)n_cl + 1, "cluster offsets G"));
                    uint32_t* gsu = reinterpret_cast<uint32_t*>(gs);
                    // gseq holds ranks; for a single dim the FE id order equals rank order, so
                    // recompute the sorted FE ids and offsets over all G groups
                    gather_i32_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(P.dims[sd[0]].gid, pm, n, gs);
                    FEGB_LAUNCH_CHECK("single cluster ids");
                    FEGB_TRY(segment_offsets(gsu, n, n_cl, of2, s));
                    off = of2;
                }
            }
            if (n_cl <= 0) {
                cluster_ok = false;
                break;
            }
            if (m == 1) {
                long long nc1 = n_cl;
                if (cpu_conv && (P.dims[sd[0]].mode != MODE_SMALLG || smallg_single)) {
                    // the CPU path counts distinct ids (cluster_id_builder ranks)
                    std::vector<int32_t> hc(P.dims[sd[0]].G);
                    FEGB_TRY(d2h_sync(hc.data(), P.dims[sd[0]].counts, sizeof(int32_t) * hc.size(), s, "counts copy"));
                    nc1 = 0;
                    for (int32_t c : hc) nc1 += c > 0;
                }
                min_single = std::min(min_single, nc1);
            }
            if (m > 1 && !rows && n_cl == n) {
                rows = true;
                row_masks.push_back(mask);
            }
            if (rows) {
                // cluster sums of single-row clusters are the score rows: meat = S'S
                if (!meat_rows) {
                    FEGB_TRY(scr.alloc(&meat_rows, (size_t)ns * ns, "meat of single-row clusters"));
                    MatView sv{S, ns, 1, ns};
                    FEGB_TRY(crossprod_auto(sv, sv, n, true, false, 1.0, 0.0, meat_rows, ns, s, sub));
                }
                FEGB_CUDA(cudaMemcpyAsync(meat, meat_rows, sizeof(double) * ns * ns, cudaMemcpyDeviceToDevice, s),
                          "meat copy");
            } else {
                double* Sc = nullptr;
                if (tuples || tuple_single) FEGB_TRY(tuple_sums());
                if (tuples)
                    Sc = tuple_scores;  // the clusters are the tuples
                else
                    FEGB_TRY(sub.alloc(&Sc, (size_t)n_cl * ns, "cluster scores"));
                if (tuples) {
                } else if (tuple_single) {
                    // n rows -> m tuple sums -> G cluster sums: the second pass reads m positions
                    FEGB_TRY(cluster_score_sums(P, tuple_scores, ns, P.tuple_dim_order[sd[0]],
                                                P.tuple_dim_gseq[sd[0]], P.tuple_dim_off[sd[0]], n_cl, Sc, sub,
                                                P.tuple_m, -1, true));
                } else if (smallg_single) {
                    const Dim& D = P.dims[sd[0]];
                    SmallGParams<double> sp{};
                    sp.X = S;
                    sp.C = ns;
                    sp.n = n;
                    sp.gid = D.gid;
                    sp.G = D.G;
                    sp.pend.n = 0;
                    sp.rows_per_block = (n + P.smallg_nb - 1) / P.smallg_nb;
                    FEGB_TRY(sub.alloc(&sp.partials, (size_t)P.smallg_nb * D.G * ns, "cluster score partials"));
                    FEGB_TRY(launch_smallg_sweep<double>(sp, P.smallg_nb, s));
                    FEGB_TRY(launch_fold_smallg(sp.partials, P.smallg_nb, D.G, ns, Sc, s));
                } else {
                    FEGB_TRY(cluster_score_sums(P, S, ns, perm, gseq, off, n_cl, Sc, sub));
                }
                MatView sv{Sc, ns, 1, ns};
                FEGB_TRY(crossprod_auto(sv, sv, n_cl, true, false, 1.0, 0.0, meat, ns, s, sub));
            }
            const double* Mk = meat;
            int ldm = ns;
            if (use_iv) {
                // meat of the projected regressors: Pi^T meat_Z Pi
                FEGB_TRY(dense_gemm(false, false, ns, k, ns, 1.0, meat, ns, Pi, na, 0.0, work, ns, s));
                FEGB_TRY(dense_gemm(true, false, k, k, ns, 1.0, Pi, na, work, ns, 0.0, meat_k, k, s));
                Mk = meat_k;
                ldm = k;
            }
            double w = (m % 2 == 1) ? 1.0 : -1.0;
            FEGB_TRY(dense_sandwich_acc(kk, Qinv, Mk, ldm, idx_dev, w, acc, work, s));
        }
        if (cluster_ok) {
            double scalar;
            long long ms = min_single == LLONG_MAX ? 0 : min_single;
            if (cpu_conv) {
                // fe_pipeline.f90:466-472
                double denom = (double)std::max(1LL, n - (long long)k);
                scalar = (double)std::max(1LL, n - 1) / denom;
                if (ms > 1) scalar *= (double)ms / (double)(ms - 1);
            } else {
                // fe_pipeline.f90:1348-1360
                int nested_adj = nested > 0 ? 1 : 0;
                long long pce = (long long)std::max(0, res->dof_model) + nested_adj;
                double denom = (double)std::max(1LL, n - pce);
                scalar = (double)std::max(1LL, n - 1) / denom;
                if (ms > 1) scalar *= (double)ms / (double)(ms - 1);
            }
            FEGB_TRY(dense_finalize_cov(kk, acc, scalar, cpu_conv ? 0 : 1, se_sel, psd_dev, work, s));
            std::vector<double> hse(kk);
            int psd = 0;
            FEGB_TRY(d2h_sync(hse.data(), se_sel, sizeof(double) * kk, s, "se copy"));
            FEGB_TRY(d2h_sync(&psd, psd_dev, sizeof(int), s, "psd copy"));
            for (int t = 0; t < kk; ++t) se_out[kept[t]] = hse[t];
            res->psd_fix_applied = psd;
            if (ms > 0) res->dof_resid = std::max(1LL, ms - 1);
            res->n_cluster_dims_used = ncd;
            res->min_single_cluster = (int)ms;
        }
    }
    if (!cluster_ok) {
        std::vector<double> hq((size_t)kk * kk);
        FEGB_TRY(d2h_sync(hq.data(), Qinv, sizeof(double) * kk * kk, s, "Qinv copy"));
        for (int t = 0; t < kk; ++t)
            se_out[kept[t]] = std::sqrt(std::max(0.0, sigma2 * hq[(size_t)t + (size_t)t * kk]));
    }
    tm.se = seconds_since(t0);
    finalize_stats(res, n);
    (void)n_raw;
    return 0;
}

class StreamHolder {
  public:
    explicit StreamHolder(void* user) {
        if (user) {
            s_ = static_cast<cudaStream_t>(user);
        } else {
            cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking);
            own_ = true;
        }
    }
    ~StreamHolder() {
        if (own_) cudaStreamDestroy(s_);
    }
    cudaStream_t get() const { return s_; }

  private:
    cudaStream_t s_ = nullptr;
    bool own_ = false;
};

int estimate_device_impl(const fegb_config* cfg_in, long long n, int k, int l, int n_fe, const double* y,
                         const double* W, const double* Z, const int32_t* const* ids, const int* group_sizes,
                         double* beta, double* se, fegb_result* result, double t_h2d, cudaStream_t s,
                         const PreDemeaned* pre = nullptr, const double* y_raw = nullptr,
                         cudaEvent_t data_ready = nullptr) {
    auto t_start = Clock::now();
    fegb_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        fegb_config_init(&cfg);
    fegb_result local{};
    fegb_result* res = result ? result : &local;
    std::memset(res, 0, sizeof(*res));
    if (n < 0 || k < 0 || l < 0 || n_fe < 0) return set_error("invalid sizes n=%lld k=%d l=%d n_fe=%d", n, k, l, n_fe);
    if (n > 0x7fffffffLL) return set_error("n=%lld exceeds the int32 row index range", n);
    if (k > 0 && (!beta || !se)) return set_error("beta/se output arrays are required");
    if (cfg.demean_method != FEGB_DEMEAN_AP && cfg.demean_method != FEGB_DEMEAN_CG)
        return set_error("unknown demean method %d", cfg.demean_method);
    configure_mem_pool();
    Scratch scr(s);
    Problem P;
    P.s = s;
    P.scr = &scr;
    P.profile = cfg.profile != 0;
    P.data_ready = data_ready;
    FitTimes tm;
    auto t0 = Clock::now();
    long long n_single = 0;
    FEGB_TRY(build_problem(P, n, k, l, n_fe, y, W, Z, ids, group_sizes, cfg.drop_singletons != 0,
                           !pre && cfg.precision == FEGB_PREC_MIXED && cfg.demean_method == FEGB_DEMEAN_AP, &n_single,
                           !pre && cfg.demean_method == FEGB_DEMEAN_CG));
    std::vector<int> G(n_fe);
    for (int d = 0; d < n_fe; ++d) G[d] = P.dims[d].G;
    // TSS of the raw y over the rows used
    double tss = 0.0;
    {
        double* ycol = nullptr;
        FEGB_TRY(scr.alloc(&ycol, (size_t)std::max(1LL, P.n), "y column"));
        // copy the strided column 0 of the data block into a contiguous vector
        // (or the raw y when the block was demeaned beforehand)
        if (y_raw && P.n > 0) {
            FEGB_CUDA(cudaMemcpyAsync(ycol, y_raw, sizeof(double) * P.n, cudaMemcpyDeviceToDevice, s), "raw y copy");
        } else if (P.n > 0) {
            FEGB_CUDA(cudaMemcpy2DAsync(ycol, sizeof(double), P.X, sizeof(double) * P.C, sizeof(double), (size_t)P.n,
                                        cudaMemcpyDeviceToDevice, s),
                      "y column copy");
        }
        FEGB_TRY(compute_tss_dev(ycol, P.n, &tss, s, scr));
    }
    trace_phase(s, t0, "problem and tss");
    FEGB_CUDA(cudaStreamSynchronize(s), "prep sync");
    tm.prep = seconds_since(t0);
    res->n_obs_used = P.n;
    res->n_singletons = n_single;
    int st = estimate_on_problem(P, cfg, G.data(), n, tss, beta, se, res, tm, pre);
    FEGB_CUDA(cudaStreamSynchronize(s), "fit sync");
    res->time_h2d = t_h2d;
    res->time_prep = tm.prep;
    res->time_demean = tm.demean;
    res->time_regression = tm.regression;
    res->time_se = tm.se;
    res->time_total = seconds_since(t_start) + t_h2d;
    if (st != 0) return st;
    return set_ok();
}

// ------------------------- FE reconstruction (--save-fe) -------------------------
//
// reconstruct_and_save_fixed_effects (src/core/fe_pipeline.f90:1619-1733):
// the residual r = y - W beta is swept dimension by dimension in index order
// (forward Gauss-Seidel, no relaxation); each dimension's group means, centred
// on their count-weighted mean, are added to its FE values and subtracted from
// r, until the largest update is below the tolerance. The weighted mean of
// the group means is the mean of r, which those subtractions keep constant, so
// the loop equals plain forward AP on r - mean(r) with the FE values as the
// accumulated updates: that is what runs here, on the sweep kernels.

__global__ void fe_resid_kernel(const double* __restrict__ y, const double* __restrict__ W, long long n, int k,
                                const double* __restrict__ beta, double* __restrict__ r) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        double v = y[i];
        for (int j = 0; j < k; ++j) v -= W[(long long)j * n + i] * beta[j];  // column by column, as the reference
        r[i] = v;
    }
}

__global__ void shift_kernel(double* __restrict__ r, long long n, double m) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) r[i] -= m;
}

int reconstruct_fe_impl(const fegb_config& cfg, long long n, int k, int n_fe, const double* y, const double* W,
                        const double* beta_host, const int32_t* const* ids, const int* group_sizes, double* values,
                        long long* counts, int* iterations, double* max_update, cudaStream_t s) {
    *iterations = 0;
    *max_update = 0.0;
    if (n <= 0 || n_fe <= 0) return 0;
    configure_mem_pool();
    Scratch scr(s);
    double *r = nullptr, *b = nullptr;
    FEGB_TRY(scr.alloc(&r, (size_t)n, "fe residual"));
    FEGB_TRY(scr.alloc(&b, (size_t)std::max(1, k), "fe beta"));
    if (k > 0) FEGB_TRY(h2d_sync(b, beta_host, sizeof(double) * k, s, "beta upload"));
    fe_resid_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(y, W, n, k, b, r);
    FEGB_LAUNCH_CHECK("fe residual");
    // mean of r (fixed-order partial sums)
    {
        int nb = (int)std::min<long long>((long long)num_sms() * 4, (n + 255) / 256);
        double* part = nullptr;
        FEGB_TRY(scr.alloc(&part, (size_t)nb, "fe mean partials"));
        tss_partials_kernel<<<nb, 256, 0, s>>>(r, n, 0.0, nullptr, part);
        FEGB_LAUNCH_CHECK("fe mean");
        std::vector<double> h(nb);
        FEGB_TRY(d2h_sync(h.data(), part, sizeof(double) * nb, s, "fe mean copy"));
        double sum = 0.0;
        for (double v : h) sum += v;
        shift_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(r, n, sum / (double)n);
        FEGB_LAUNCH_CHECK("fe centre");
    }
    Problem P;
    P.s = s;
    P.scr = &scr;
    long long n_single = 0;
    FEGB_TRY(build_problem(P, n, 0, 0, n_fe, r, nullptr, nullptr, ids, group_sizes, false, false, &n_single, false));
    FEGB_TRY(reset_ap_state(P, true));
    PendingList pl;
    ProjectionOpts o;
    o.alpha = true;
    o.mixing = false;
    double mu = 0.0;
    const int max_iter = std::max(1, cfg.fe_max_iter);
    int it = max_iter + 1;  // a DO loop that runs to completion leaves its index one past the end
    for (int iter = 1; iter <= max_iter; ++iter) {
        FEGB_CUDA(cudaMemsetAsync(P.max_bits, 0, sizeof(unsigned long long), s), "reset max");
        for (int d = 0; d < n_fe; ++d) FEGB_TRY(project<double>(P, d, P.X, pl, o));
        unsigned long long bits = 0;
        FEGB_TRY(d2h_sync(&bits, P.max_bits, sizeof(bits), s, "fe max copy"));
        mu = bits_to_double(bits);
        if (mu < cfg.fe_tol) {
            it = iter;
            break;
        }
    }
    *iterations = it;
    *max_update = mu;
    long long off = 0;
    for (int d = 0; d < n_fe; ++d) {
        const Dim& D = P.dims[d];
        if (D.G <= 0) continue;
        FEGB_TRY(d2h_sync(values + off, D.alpha, sizeof(double) * D.G, s, "fe values copy"));
        std::vector<int32_t> c(D.G);
        FEGB_TRY(d2h_sync(c.data(), D.counts, sizeof(int32_t) * D.G, s, "fe counts copy"));
        for (int g = 0; g < D.G; ++g) counts[off + g] = c[g];
        off += D.G;
    }
    return 0;
}

// In-place within-transform of device columns (column-major, ld n).
int within_impl(const fegb_config& cfg, long long n, int k, int l, int n_fe, double* d_y, double* d_W, double* d_Z,
                const int32_t* const* ids, const int* group_sizes, cudaStream_t s, PreDemeaned* out) {
    configure_mem_pool();
    auto t0 = Clock::now();
    Scratch scr(s);
    Problem P;
    P.s = s;
    P.scr = &scr;
    P.profile = cfg.profile != 0;
    long long n_single = 0;
    FEGB_TRY(build_problem(P, n, k, l, n_fe, d_y, d_W, d_Z, ids, group_sizes, false,
                           cfg.precision == FEGB_PREC_MIXED && cfg.demean_method == FEGB_DEMEAN_AP, &n_single,
                           cfg.demean_method == FEGB_DEMEAN_CG));
    int it = 0, conv = 1, outer = 0;
    double mu = 0.0;
    if (cfg.demean_method == FEGB_DEMEAN_CG) {
        if (cfg.precision == FEGB_PREC_MIXED)
            FEGB_TRY(demean_cg<float>(P, cfg.fe_tol, cfg.fe_max_iter, &it, &conv, &mu, &outer));
        else
            FEGB_TRY(demean_cg<double>(P, cfg.fe_tol, cfg.fe_max_iter, &it, &conv, &mu, &outer));
    } else if (cfg.precision == FEGB_PREC_MIXED) {
        FEGB_TRY(demean_mixed(P, cfg.fe_tol, cfg.fe_max_iter, &it, &conv, &mu, &outer));
    } else {
        FEGB_TRY(demean_plain(P, cfg.fe_tol, cfg.fe_max_iter, &it, &conv, &mu));
    }
    if (n > 0) {
        const int xt = xt_rows(P.C);
        const size_t smem = sizeof(double) * (size_t)xt * (P.C | 1);
        static const cudaError_t attr =
            cudaFuncSetAttribute(scatter_x_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024);
        if (attr != cudaSuccess) return set_cuda_error(attr, "scatter data block attr");
        scatter_x_kernel<<<(unsigned)((n + xt - 1) / xt), 256, smem, s>>>(P.X, P.row_of, n, P.C, k, n, xt, d_y, d_W,
                                                                          d_Z);
        FEGB_LAUNCH_CHECK("scatter data block");
    }
    FEGB_CUDA(cudaStreamSynchronize(s), "within sync");
    out->iterations = it;
    out->converged = conv;
    out->outer = outer;
    out->max_update = mu;
    out->seconds = seconds_since(t0);
    out->projections = P.projections;
    out->demean_bytes = P.demean_bytes;
    std::memset(&out->prof, 0, sizeof(out->prof));
    FEGB_TRY(collect_profile(P, &out->prof));
    return 0;
}

// ------------------------- batched specifications -------------------------
//
// Specifications are stacked into one problem per column-count class: rows
// one after the other, FE ids shifted so that every specification owns its
// own groups, missing FE dimensions filled with one group per specification
// (a group that every FE dimension already spans, so it changes no
// projection). The stacked system is block diagonal, so one within-transform
// gives every specification its own demeaned columns; each is then estimated
// on its own rows with the single-fit code, the within-transform skipped.

constexpr int BATCH_MAX_FE = SWEEP_MAXP;
constexpr int BATCH_FIT_THREADS = 8;  // host threads (one stream each) fitting specifications after the demean

struct BatchSpecDev {
    long long row0;
    long long n;
    int k, l, n_fe;
    const double* y;
    const double* W;
    const double* Z;
    const int32_t* ids[BATCH_MAX_FE];
    int goff[BATCH_MAX_FE];  // first stacked group (0-based) of each dimension
};

// Max over a block of 256 threads (result valid in thread 0).
__device__ int block_reduce_max_int(int v) {
    __shared__ int red[8];
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    __syncthreads();  // red[] may still be read by a previous call
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        v = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : INT_MIN;
        for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    }
    return v;
}

// Max and min id of every specification and dimension: one block per spec.
__global__ void batch_id_range_kernel(const BatchSpecDev* __restrict__ sp, int d, int* __restrict__ gmax,
                                      int* __restrict__ gmin) {
    const BatchSpecDev& S = sp[blockIdx.x];
    int mx = 0, mn = INT_MAX;
    if (d < S.n_fe)
        for (long long i = threadIdx.x; i < S.n; i += blockDim.x) {
            const int v = S.ids[d][i];
            mx = max(mx, v);
            mn = min(mn, v);
        }
    mx = block_reduce_max_int(mx);
    mn = -block_reduce_max_int(-mn);
    if (threadIdx.x == 0) {
        gmax[blockIdx.x] = mx;
        gmin[blockIdx.x] = mn;
    }
}

__device__ __forceinline__ int batch_spec_of(const BatchSpecDev* sp, int ns, long long i) {
    int lo = 0, hi = ns - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sp[mid].row0 <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Stacked columns (column-major, ld N): y, then W, then Z, then zeros up to kb
// columns; stacked 1-based ids with the per-spec group offsets.
__global__ void batch_stack_kernel(const BatchSpecDev* __restrict__ sp, int ns, long long N, int kb, int fe_b,
                                   double* __restrict__ yb, double* __restrict__ Wb, int32_t* __restrict__ idsb) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < N; i += st) {
        const int si = batch_spec_of(sp, ns, i);
        const BatchSpecDev& S = sp[si];
        const long long r = i - S.row0;
        yb[i] = S.y[r];
        for (int c = 0; c < kb; ++c) {
            double v = 0.0;
            if (c < S.k)
                v = S.W[(long long)c * S.n + r];
            else if (c < S.k + S.l)
                v = S.Z[(long long)(c - S.k) * S.n + r];
            Wb[(long long)c * N + i] = v;
        }
        for (int d = 0; d < fe_b; ++d)
            idsb[(long long)d * N + i] = S.goff[d] + (d < S.n_fe ? S.ids[d][r] : 1);
    }
}

// padded column count of a specification's class
int batch_class(int C) {
    if (C <= 4) return 4;
    if (C <= 8) return 8;
    if (C <= 12) return 12;
    if (C <= 16) return 16;
    if (C <= 24) return 24;
    if (C <= 32) return 32;
    return ((C + 15) / 16) * 16;
}

int estimate_batch_impl(const fegb_config& cfg, int n_specs, const fegb_spec* specs, double* beta, double* se,
                        fegb_result* results, cudaStream_t s) {
    if (n_specs < 0) return set_error("n_specs < 0");
    if (n_specs == 0) return set_ok();
    if (!specs || !results) return set_error("batch: null specs or results");
    if (cfg.drop_singletons) return set_error("batch: singleton dropping is not supported for batched specifications");
    configure_mem_pool();
    std::vector<long long> boff(n_specs + 1, 0);
    for (int i = 0; i < n_specs; ++i) {
        const fegb_spec& S = specs[i];
        if (S.n <= 0 || S.k < 0 || S.l < 0) return set_error("batch spec %d: invalid sizes", i);
        if (S.n > 0x7fffffffLL) return set_error("batch spec %d: n exceeds the int32 row range", i);
        if (S.n_fe < 1 || S.n_fe > BATCH_MAX_FE) return set_error("batch spec %d: n_fe must be 1..%d", i, BATCH_MAX_FE);
        if (!S.y || (S.k > 0 && !S.W) || (S.l > 0 && !S.Z) || !S.fe_ids)
            return set_error("batch spec %d: null array", i);
        boff[i + 1] = boff[i] + S.k;
    }
    if (boff[n_specs] > 0 && (!beta || !se)) return set_error("batch: beta/se output arrays are required");
    // specifications by column-count class, in spec order
    std::vector<std::pair<int, int>> order;
    for (int i = 0; i < n_specs; ++i) order.push_back({batch_class(1 + specs[i].k + specs[i].l), i});
    std::stable_sort(order.begin(), order.end(),
                     [](const std::pair<int, int>& a, const std::pair<int, int>& b) { return a.first < b.first; });
    size_t pos = 0;
    while (pos < order.size()) {
        size_t end = pos;
        while (end < order.size() && order[end].first == order[pos].first) ++end;
        const int cb = order[pos].first;
        const int kb = cb - 1;
        std::vector<int> idx;
        for (size_t t = pos; t < end; ++t) idx.push_back(order[t].second);
        pos = end;
        const int ns = (int)idx.size();
        Scratch scr(s);
        std::vector<BatchSpecDev> hs(ns);
        long long N = 0;
        int fe_b = 1;
        for (int t = 0; t < ns; ++t) {
            const fegb_spec& S = specs[idx[t]];
            BatchSpecDev& D = hs[t];
            std::memset(&D, 0, sizeof(D));
            D.row0 = N;
            D.n = S.n;
            D.k = S.k;
            D.l = S.l;
            D.n_fe = S.n_fe;
            D.y = S.y;
            D.W = S.W;
            D.Z = S.Z;
            for (int d = 0; d < S.n_fe; ++d) D.ids[d] = S.fe_ids[d];
            N += S.n;
            fe_b = std::max(fe_b, S.n_fe);
        }
        if (N > 0x7fffffffLL) return set_error("batch: %lld stacked rows exceed the int32 row range", N);
        BatchSpecDev* dsp = nullptr;
        FEGB_TRY(scr.alloc(&dsp, (size_t)ns, "batch specs"));
        FEGB_CUDA(cudaMemcpyAsync(dsp, hs.data(), sizeof(BatchSpecDev) * ns, cudaMemcpyHostToDevice, s),
                  "batch specs copy");
        // group sizes of every spec and dimension
        int *gmax = nullptr, *gmin = nullptr;
        FEGB_TRY(scr.alloc(&gmax, (size_t)ns * fe_b, "batch group max"));
        FEGB_TRY(scr.alloc(&gmin, (size_t)ns * fe_b, "batch group min"));
        for (int d = 0; d < fe_b; ++d) {
            batch_id_range_kernel<<<ns, 256, 0, s>>>(dsp, d, gmax + (size_t)d * ns, gmin + (size_t)d * ns);
            FEGB_LAUNCH_CHECK("batch id range");
        }
        std::vector<int> hmax((size_t)ns * fe_b), hmin((size_t)ns * fe_b);
        FEGB_CUDA(cudaMemcpyAsync(hmax.data(), gmax, sizeof(int) * hmax.size(), cudaMemcpyDeviceToHost, s), "gmax");
        FEGB_CUDA(cudaMemcpyAsync(hmin.data(), gmin, sizeof(int) * hmin.size(), cudaMemcpyDeviceToHost, s), "gmin");
        FEGB_CUDA(cudaStreamSynchronize(s), "batch sizes sync");
        std::vector<int> Gb(fe_b, 0);
        std::vector<std::vector<int>> Gs(ns, std::vector<int>(fe_b, 1));
        for (int d = 0; d < fe_b; ++d) {
            long long acc = 0;
            for (int t = 0; t < ns; ++t) {
                if (d < hs[t].n_fe) {
                    if (hmin[(size_t)d * ns + t] < 1)
                        return set_error("batch spec %d: FE dimension %d has an id < 1", idx[t], d + 1);
                    Gs[t][d] = hmax[(size_t)d * ns + t];
                }
                hs[t].goff[d] = (int)acc;
                acc += Gs[t][d];
            }
            if (acc > 0x7fffffffLL) return set_error("batch: stacked groups exceed the int32 range");
            Gb[d] = (int)acc;
        }
        FEGB_CUDA(cudaMemcpyAsync(dsp, hs.data(), sizeof(BatchSpecDev) * ns, cudaMemcpyHostToDevice, s),
                  "batch offsets copy");
        double *yb = nullptr, *Wb = nullptr;
        int32_t* idsb = nullptr;
        FEGB_TRY(scr.alloc(&yb, (size_t)N, "stacked y"));
        FEGB_TRY(scr.alloc(&Wb, (size_t)N * kb, "stacked columns"));
        FEGB_TRY(scr.alloc(&idsb, (size_t)N * fe_b, "stacked ids"));
        batch_stack_kernel<<<grid_stride_blocks(N, 256), 256, 0, s>>>(dsp, ns, N, kb, fe_b, yb, Wb, idsb);
        FEGB_LAUNCH_CHECK("batch stack");
        std::vector<const int32_t*> ids_b(fe_b);
        for (int d = 0; d < fe_b; ++d) ids_b[d] = idsb + (size_t)d * N;
        PreDemeaned pre;
        auto tc0 = Clock::now();
        FEGB_TRY(within_impl(cfg, N, kb, 0, fe_b, yb, Wb, nullptr, ids_b.data(), Gb.data(), s, &pre));
        FEGB_CUDA(cudaStreamSynchronize(s), "batch demean sync");
        const double t_within = seconds_since(tc0);
        tc0 = Clock::now();
        // the whole class at once (batch_est.cu) when the batched estimator takes it
        {
            std::vector<BeSpecHost> be(ns);
            for (int t = 0; t < ns; ++t) {
                const fegb_spec& S = specs[idx[t]];
                BeSpecHost& B = be[t];
                B.row0 = hs[t].row0;
                B.n = S.n;
                B.k = S.k;
                B.l = S.l;
                B.n_fe = S.n_fe;
                for (int d = 0; d < fe_b && d < BE_MAX_FE; ++d) {
                    B.G[d] = Gs[t][d];
                    B.goff[d] = hs[t].goff[d];
                }
                // cluster dimensions: valid, unique, the first three (fe_pipeline.f90:1553-1599)
                for (int i = 0; i < S.n_cluster_dims && B.n_cd < MAX_CLUSTER_DIMS; ++i) {
                    const int v = S.cluster_dims[i];
                    if (v < 1 || v > S.n_fe) continue;
                    bool dup = false;
                    for (int j = 0; j < B.n_cd; ++j) dup = dup || B.cd[j] == v - 1;
                    if (!dup) B.cd[B.n_cd++] = v - 1;
                }
                if (S.n_iv_regressors > 0) B.endog.assign(S.iv_regressors, S.iv_regressors + S.n_iv_regressors);
                if (S.n_iv_instruments > 0)
                    B.instr.assign(S.iv_instruments, S.iv_instruments + S.n_iv_instruments);
                B.y_raw = S.y;
            }
            if (fe_b <= BE_MAX_FE && batch_est_eligible(cfg, cb, be) && tuning(TUNE_BATCH_ESTIMATOR)) {
                std::vector<double*> bp(ns), sp(ns);
                std::vector<fegb_result*> rp(ns);
                for (int t = 0; t < ns; ++t) {
                    const int si = idx[t];
                    bp[t] = beta + boff[si];
                    sp[t] = se + boff[si];
                    rp[t] = &results[si];
                    fegb_result* r = rp[t];
                    std::memset(r, 0, sizeof(*r));
                    for (int j = 0; j < specs[si].k; ++j) bp[t][j] = sp[t][j] = 0.0;
                    r->converged = pre.converged;
                    r->fe_iterations = pre.iterations;
                    r->max_update = pre.max_update;
                    r->outer_iterations = pre.outer;
                    r->projections = pre.projections;
                    r->demean_bytes = pre.demean_bytes;
                    r->time_demean = pre.seconds;
                    if (t == 0)
                        for (int f = 0; f < 8; ++f) {
                            r->prof_launches[f] = pre.prof.prof_launches[f];
                            r->prof_seconds[f] = pre.prof.prof_seconds[f];
                            r->prof_bytes[f] = pre.prof.prof_bytes[f];
                        }
                }
                FEGB_TRY(estimate_class_batched(cfg, be, N, cb, yb, Wb, ids_b.data(), fe_b, bp.data(), sp.data(),
                                                rp.data(), s));
                for (int t = 0; t < ns; ++t) {
                    fegb_result* r = rp[t];
                    if (r->solver_info == 0 && r->dof_model > 0) finalize_stats(r, specs[idx[t]].n);
                    r->time_total = r->time_demean + r->time_regression + r->time_se;
                }
                if (trace_enabled())
                    std::fprintf(stderr,
                                 "fegb batch: class of %d columns: %d specs, %lld rows, within-transform %.1f ms "
                                 "(%d CG), batched estimation %.1f ms\n",
                                 cb, ns, N, t_within * 1e3, pre.iterations, seconds_since(tc0) * 1e3);
                continue;
            }
        }
        // every specification on its own demeaned rows; the fits are
        // independent, so a few host threads run them on their own streams
        auto fit_one = [&](int t, cudaStream_t ws) -> int {
            const int si = idx[t];
            const fegb_spec& S = specs[si];
            Scratch sub(ws);
            double *dy = nullptr, *dW = nullptr, *dZ = nullptr;
            FEGB_TRY(sub.alloc(&dy, (size_t)S.n, "spec y"));
            FEGB_TRY(sub.alloc(&dW, (size_t)S.n * std::max(1, S.k), "spec W"));
            FEGB_TRY(sub.alloc(&dZ, (size_t)S.n * std::max(1, S.l), "spec Z"));
            const long long r0 = hs[t].row0;
            FEGB_CUDA(cudaMemcpyAsync(dy, yb + r0, sizeof(double) * S.n, cudaMemcpyDeviceToDevice, ws), "spec y");
            if (S.k > 0)
                FEGB_CUDA(cudaMemcpy2DAsync(dW, sizeof(double) * S.n, Wb + r0, sizeof(double) * N,
                                            sizeof(double) * S.n, S.k, cudaMemcpyDeviceToDevice, ws),
                          "spec W");
            if (S.l > 0)
                FEGB_CUDA(cudaMemcpy2DAsync(dZ, sizeof(double) * S.n, Wb + (size_t)S.k * N + r0, sizeof(double) * N,
                                            sizeof(double) * S.n, S.l, cudaMemcpyDeviceToDevice, ws),
                          "spec Z");
            fegb_config cs = cfg;
            cs.stream = ws;
            cs.n_cluster_dims = S.n_cluster_dims;
            cs.cluster_dims = S.cluster_dims;
            cs.n_iv_regressors = S.n_iv_regressors;
            cs.iv_regressors = S.iv_regressors;
            cs.n_iv_instruments = S.n_iv_instruments;
            cs.iv_instruments = S.iv_instruments;
            std::vector<const int32_t*> sid(S.n_fe);
            for (int d = 0; d < S.n_fe; ++d) sid[d] = S.fe_ids[d];
            std::vector<int> gsz(Gs[t].begin(), Gs[t].begin() + S.n_fe);
            PreDemeaned mine = pre;
            mine.carry_profile = t == 0;  // the class's sweep timings are reported once, on its first spec
            return estimate_device_impl(&cs, S.n, S.k, S.l, S.n_fe, dy, dW, dZ, sid.data(), gsz.data(),
                                        beta + boff[si], se + boff[si], &results[si], 0.0, ws, &mine, S.y);
        };
        const int nthreads = std::min(ns, BATCH_FIT_THREADS);
        std::atomic<int> next{0};
        std::atomic<int> failed{0};
        std::mutex err_mu;
        std::string err_msg;
        int err_status = 0;
        auto worker = [&]() {
            cudaStream_t ws = nullptr;
            if (cudaStreamCreateWithFlags(&ws, cudaStreamNonBlocking) != cudaSuccess) {
                failed = 1;
                std::lock_guard<std::mutex> g(err_mu);
                if (!err_status) {
                    err_status = 1;
                    err_msg = "batch: cannot create a worker stream";
                }
                return;
            }
            for (int t = next++; t < ns && !failed; t = next++) {
                int st = fit_one(t, ws);
                if (st != 0) {
                    failed = 1;
                    std::lock_guard<std::mutex> g(err_mu);
                    if (!err_status) {
                        err_status = st;
                        err_msg = std::string("batch spec ") + std::to_string(idx[t]) + ": " + last_error();
                    }
                }
            }
            cudaStreamSynchronize(ws);
            cudaStreamDestroy(ws);
        };
        std::vector<std::thread> pool;
        for (int w = 1; w < nthreads; ++w) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
        if (err_status) return set_error("%s", err_msg.c_str());
        if (trace_enabled())
            std::fprintf(stderr, "fegb batch: class of %d columns: %d specs, %lld rows, within-transform %.1f ms (%d CG), "
                                 "per-spec fits %.1f ms\n",
                         cb, ns, N, t_within * 1e3, pre.iterations, seconds_since(tc0) * 1e3);
    }
    return set_ok();
}

}  // namespace

}  // namespace fegb

using namespace fegb;

extern "C" {

void fegb_config_init(fegb_config* cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->fe_tol = 1.0e-6;  // src/core/fe_config.f90:55
    cfg->fe_max_iter = 500;
    cfg->precision = FEGB_PREC_FP64;
    cfg->demean_method = FEGB_DEMEAN_AP;
    cfg->se_convention = FEGB_SE_GPU;
}

int fegb_estimate_device(const fegb_config* cfg, long long n, int k, int l, int n_fe, const double* d_y,
                         const double* d_W, const double* d_Z, const int* const* d_fe_ids, const int* group_sizes,
                         double* beta, double* se, fegb_result* result) {
    StreamHolder sh(cfg ? cfg->stream : nullptr);
    std::vector<const int32_t*> ids(n_fe);
    for (int d = 0; d < n_fe; ++d) ids[d] = d_fe_ids[d];
    return estimate_device_impl(cfg, n, k, l, n_fe, d_y, d_W, d_Z, ids.data(), group_sizes, beta, se, result, 0.0,
                                sh.get());
}

// Host-to-device upload over several copy streams: one cudaMemcpyAsync per
// piece (pieces of at least 32 MB, round-robin over the streams), so several
// copy engines run at once; the fit's stream waits on each copy stream's event.
// The streams and events are created once per host thread.
class Uploader {
  public:
    static constexpr int NS = 8;
    explicit Uploader(cudaStream_t s) : s_(s) {
        thread_local struct Pool {
            cudaStream_t st[NS] = {};
            cudaEvent_t ev[NS] = {};
            bool ok = false;
            Pool() {
                ok = true;
                for (int i = 0; i < NS; ++i) {
                    ok = ok && cudaStreamCreateWithFlags(&st[i], cudaStreamNonBlocking) == cudaSuccess;
                    ok = ok && cudaEventCreateWithFlags(&ev[i], cudaEventDisableTiming) == cudaSuccess;
                }
            }
        } pool;
        pool_ok_ = pool.ok;
        for (int i = 0; i < NS; ++i) {
            st_[i] = pool.st[i];
            ev_[i] = pool.ev[i];
        }
    }
    // copy streams start after the work already queued on s
    int begin() {
        if (!pool_ok_) return 0;
        FEGB_CUDA(cudaEventRecord(ev_[0], s_), "upload start");
        for (int i = 0; i < NS; ++i) FEGB_CUDA(cudaStreamWaitEvent(st_[i], ev_[0], 0), "upload start wait");
        return 0;
    }
    int copy(void* dst, const void* src, size_t bytes, const char* what) {
        if (!pool_ok_) {
            FEGB_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s_), what);
            return 0;
        }
        constexpr size_t PIECE = 32u << 20;
        const size_t pieces = std::max<size_t>(1, std::min<size_t>(NS, bytes / PIECE));
        const size_t per = (bytes + pieces - 1) / pieces;
        for (size_t o = 0; o < bytes; o += per) {
            const size_t b = std::min(per, bytes - o);
            FEGB_CUDA(cudaMemcpyAsync(static_cast<char*>(dst) + o, static_cast<const char*>(src) + o, b,
                                      cudaMemcpyHostToDevice, st_[next_]),
                      what);
            next_ = (next_ + 1) % NS;
        }
        return 0;
    }
    // s waits for every piece issued so far
    int join() {
        if (!pool_ok_) return 0;
        for (int i = 0; i < NS; ++i) {
            FEGB_CUDA(cudaEventRecord(ev_[i], st_[i]), "upload done");
            FEGB_CUDA(cudaStreamWaitEvent(s_, ev_[i], 0), "upload join");
        }
        return 0;
    }
    // one event recorded once every piece issued so far is done (s does not wait):
    // stream 0 waits for the others, then records it
    int done_event(cudaEvent_t* out) {
        *out = nullptr;
        if (!pool_ok_) return 0;
        for (int i = 1; i < NS; ++i) {
            FEGB_CUDA(cudaEventRecord(ev_[i], st_[i]), "upload done");
            FEGB_CUDA(cudaStreamWaitEvent(st_[0], ev_[i], 0), "upload gather");
        }
        FEGB_CUDA(cudaEventRecord(ev_[0], st_[0]), "upload done");
        *out = ev_[0];
        return 0;
    }

  private:
    cudaStream_t s_;
    cudaStream_t st_[NS];
    cudaEvent_t ev_[NS];
    bool pool_ok_ = false;
    int next_ = 0;
};

int fegb_estimate_host(const fegb_config* cfg, long long n, int k, int l, int n_fe, const double* y,
                       const double* W, const double* Z, const int* fe_ids, const int* group_sizes, double* beta,
                       double* se, fegb_result* result) {
    if (n < 0 || k < 0 || l < 0 || n_fe < 0) return set_error("invalid sizes");
    StreamHolder sh(cfg ? cfg->stream : nullptr);
    cudaStream_t s = sh.get();
    configure_mem_pool();
    auto t0 = Clock::now();
    Scratch scr(s);
    double *dy = nullptr, *dW = nullptr, *dZ = nullptr;
    int32_t *dids = nullptr, *dint = nullptr;
    size_t nn = (size_t)std::max(1LL, n);
    FEGB_TRY(scr.alloc(&dy, nn, "y upload"));
    FEGB_TRY(scr.alloc(&dW, nn * std::max(1, k), "W upload"));
    FEGB_TRY(scr.alloc(&dZ, nn * std::max(1, l), "Z upload"));
    FEGB_TRY(scr.alloc(&dint, nn * std::max(1, n_fe), "ids upload"));
    FEGB_TRY(scr.alloc(&dids, nn * std::max(1, n_fe), "ids"));
    trace_phase(s, t0, "upload buffers");
    // the ids first: the preparation starts on them while y, W and Z are in flight
    cudaEvent_t data_ready = nullptr;
    Uploader up(s);
    if (n > 0) {
        FEGB_TRY(up.begin());
        if (n_fe > 0) FEGB_TRY(up.copy(dint, fe_ids, sizeof(int32_t) * n * n_fe, "ids H2D"));
        FEGB_TRY(up.join());
        if (n_fe > 0) {
            deinterleave_ids_kernel<<<grid_stride_blocks(n * n_fe, 256), 256, 0, s>>>(dint, n_fe, n, dids);
            FEGB_LAUNCH_CHECK("ids deinterleave");
        }
        trace_phase(s, t0, "ids upload (alone)");
        FEGB_TRY(up.copy(dy, y, sizeof(double) * n, "y H2D"));
        if (k > 0) FEGB_TRY(up.copy(dW, W, sizeof(double) * n * k, "W H2D"));
        if (l > 0) FEGB_TRY(up.copy(dZ, Z, sizeof(double) * n * l, "Z H2D"));
        FEGB_TRY(up.done_event(&data_ready));
        if (!data_ready) FEGB_CUDA(cudaStreamSynchronize(s), "H2D sync");
    }
    double t_h2d = seconds_since(t0);  // issue time only: the copies overlap the preparation
    std::vector<const int32_t*> ids(n_fe);
    for (int d = 0; d < n_fe; ++d) ids[d] = dids + (size_t)d * n;
    return estimate_device_impl(cfg, n, k, l, n_fe, dy, dW, dZ, ids.data(), group_sizes, beta, se, result, t_h2d, s,
                                nullptr, nullptr, data_ready);
}

int fegb_within_transform(const fegb_config* cfg_in, long long n, int k, int l, int n_fe, double* d_y, double* d_W,
                          double* d_Z, const int* const* d_fe_ids, const int* group_sizes, int* converged,
                          int* iterations, double* max_update) {
    fegb_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        fegb_config_init(&cfg);
    StreamHolder sh(cfg.stream);
    std::vector<const int32_t*> ids(n_fe);
    for (int d = 0; d < n_fe; ++d) ids[d] = d_fe_ids[d];
    PreDemeaned st;
    FEGB_TRY(within_impl(cfg, n, k, l, n_fe, d_y, d_W, d_Z, ids.data(), group_sizes, sh.get(), &st));
    if (converged) *converged = st.converged;
    if (iterations) *iterations = st.iterations;
    if (max_update) *max_update = st.max_update;
    return set_ok();
}

int fegb_reconstruct_fe(const fegb_config* cfg_in, long long n, int k, int n_fe, const double* d_y, const double* d_W,
                        const double* beta, const int* const* d_fe_ids, const int* group_sizes, double* fe_values,
                        long long* fe_counts, int* iterations, double* max_update) {
    fegb_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        fegb_config_init(&cfg);
    if (n < 0 || k < 0 || n_fe < 0) return set_error("invalid sizes");
    if (n > 0x7fffffffLL) return set_error("n=%lld exceeds the int32 row range", n);
    if (n > 0 && (!d_y || (k > 0 && (!d_W || !beta)) || (n_fe > 0 && !d_fe_ids)))
        return set_error("fegb_reconstruct_fe: null argument");
    if (!fe_values || !fe_counts || !iterations || !max_update) return set_error("fegb_reconstruct_fe: null output");
    StreamHolder sh(cfg.stream);
    std::vector<const int32_t*> ids(n_fe);
    for (int d = 0; d < n_fe; ++d) ids[d] = d_fe_ids[d];
    FEGB_TRY(reconstruct_fe_impl(cfg, n, k, n_fe, d_y, d_W, beta, ids.data(), group_sizes, fe_values, fe_counts,
                                 iterations, max_update, sh.get()));
    return set_ok();
}

int fegb_estimate_batch(const fegb_config* cfg_in, int n_specs, const fegb_spec* specs, double* beta, double* se,
                        fegb_result* results) {
    fegb_config cfg;
    if (cfg_in)
        cfg = *cfg_in;
    else
        fegb_config_init(&cfg);
    StreamHolder sh(cfg.stream);
    return estimate_batch_impl(cfg, n_specs, specs, beta, se, results, sh.get());
}

int fegb_cluster_ids(const int* const* d_fe_ids, const int* sizes, int n_dims, long long n, int* d_out_ids,
                     int* n_clusters) {
    if (!d_fe_ids || !sizes || !d_out_ids || !n_clusters || n_dims <= 0) return set_error("invalid cluster-id arguments");
    if (n_dims > 4) return set_error("at most 4 cluster dimensions (got %d)", n_dims);
    if (n <= 0) {
        *n_clusters = 0;
        return set_ok();
    }
    StreamHolder sh(nullptr);
    cudaStream_t s = sh.get();
    configure_mem_pool();
    Scratch scr(s);
    std::vector<const int32_t*> ptrs(n_dims);
    std::vector<unsigned long long> strides(n_dims);
    unsigned long long span = 1;
    bool sort_ok = true;
    for (int j = 0; j < n_dims; ++j) {
        ptrs[j] = d_fe_ids[j];
        strides[j] = span;
        unsigned long long sz = (unsigned long long)(sizes[j] > 0 ? sizes[j] : 0);
        if (sz == 0 || sz > ~0ULL / span) {
            sort_ok = false;
            break;
        }
        span *= sz;
        if (span > (1ULL << 62)) {
            sort_ok = false;
            break;
        }
    }
    int nc = 0;
    if (sort_ok) {
        FEGB_TRY(cluster_ids_by_key(ptrs.data(), strides.data(), n_dims, n, bits_for(span), d_out_ids, &nc, nullptr,
                                    nullptr, s, scr));
    } else {
        FEGB_TRY(cluster_ids_first_appearance(ptrs.data(), sizes, n_dims, n, d_out_ids, &nc, s, scr));
    }
    FEGB_CUDA(cudaStreamSynchronize(s), "cluster ids sync");
    *n_clusters = nc;
    return set_ok();
}

int fegb_compact_ids(const int* d_raw, long long n, int* d_out, int* n_levels) {
    if (n > 0 && (!d_raw || !d_out)) return set_error("invalid compaction arguments");
    StreamHolder sh(nullptr);
    configure_mem_pool();
    Scratch scr(sh.get());
    FEGB_TRY(compact_ids(d_raw, n, d_out, n_levels, sh.get(), scr));
    FEGB_CUDA(cudaStreamSynchronize(sh.get()), "compact sync");
    return set_ok();
}

int fegb_group_sizes(const int* const* d_fe_ids, int n_fe, long long n, int* sizes) {
    StreamHolder sh(nullptr);
    configure_mem_pool();
    Scratch scr(sh.get());
    for (int d = 0; d < n_fe; ++d) {
        if (n <= 0) {
            sizes[d] = 0;
            continue;
        }
        int mn = 0, mx = 0;
        FEGB_TRY(ids_min_max(d_fe_ids[d], n, &mn, &mx, sh.get(), scr));
        if (mn < 1) return set_error("FE indices must be positive and contiguous (dimension %d)", d + 1);
        sizes[d] = std::max(0, mx);
    }
    return set_ok();
}

int fegb_drop_singletons(const int* const* d_fe_ids, const int* sizes, int n_fe, long long n, unsigned char* d_keep,
                         long long* n_dropped) {
    StreamHolder sh(nullptr);
    cudaStream_t s = sh.get();
    configure_mem_pool();
    Scratch scr(s);
    std::vector<int32_t*> g0(n_fe);
    for (int d = 0; d < n_fe; ++d) {
        FEGB_TRY(scr.alloc(&g0[d], (size_t)std::max(1LL, n), "singleton gid"));
        if (n > 0) {
            gather_gid_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(d_fe_ids[d], nullptr, n, g0[d]);
            FEGB_LAUNCH_CHECK("singleton gid");
        }
    }
    std::vector<int> G(sizes, sizes + n_fe);
    FEGB_TRY(drop_singletons(g0.data(), G.data(), n_fe, n, d_keep, n_dropped, s, scr));
    FEGB_CUDA(cudaStreamSynchronize(s), "singleton sync");
    return set_ok();
}

}  // extern "C"
