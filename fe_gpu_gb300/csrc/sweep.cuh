// Alternating-projection sweep kernels.
//
// Data layout: the N x C block [y W Z] is stored row-interleaved (AoS, row
// stride C elements) in "storage order" = rows stably sorted by the primary FE
// dimension. A projection onto FE dimension d needs the group sums of the
// current residual over d's groups. They are computed deterministically (no
// floating-point atomics) by one of two traversals:
//
//  * segment traversal: positions j = 0..N-1 of d's group-sorted order
//    (identity for the primary dimension, a permutation otherwise) are cut into
//    fixed chunks of R positions; one thread per (chunk, column) sums runs of
//    equal group id in position order. Runs complete inside a chunk are
//    written directly; runs crossing a chunk edge leave a head/tail partial
//    that the finalize kernel adds in chunk order.
//  * small-G streaming: storage order, each (row sub-range, column) thread
//    owns a private shared-memory table of the G group sums; tables are folded
//    in a fixed order per block and block partials in block order.
//
// Subtracting the means is deferred: each dimension keeps a "pending" table of
// means not yet removed from the stored rows. Every traversal subtracts all
// pending tables on the fly; storage-order traversals also write the updated
// rows back, which clears the pending set. The finalize kernel turns sums into
// means, applies the reference's over-relaxation (mixed = prev + r (mean -
// prev)), folds the result into the dimension's pending table, and tracks the
// max |mixed| for the convergence test and the adaptive relaxation rule
// (src/gpu/fe_gpu_demean.f90:171-218), entirely on the device.
#pragma once

#include "common.cuh"

namespace fegb {

constexpr int SWEEP_MAXP = 8;  // max FE dimensions whose means may be pending

template <typename T>
struct PendingSet {
    int n;
    const int32_t* gid[SWEEP_MAXP];  // group id of the traversal position (or storage row)
    const T* tab[SWEEP_MAXP];        // G_e x C tables of pending means
};

template <typename T>
struct SegSweepParams {
    T* X;                  // element (row, col) at X[row * rs + col * cs]
    long long rs;          // row stride (C for the AoS block)
    long long cs;          // column stride (1 for the AoS block)
    int C;                 // columns; also the width of sums/head/tail and pending tables
    long long n;
    const int32_t* perm;   // traversal position -> storage row; null = storage order
    const int32_t* gseq;   // 0-based group id at each traversal position (non-decreasing)
    PendingSet<T> pend;    // gid arrays indexed by traversal position
    int writeback;         // write the pending-adjusted rows back (storage order only)
    int no_data;           // 1: rows are not read (value = 0 - pending), used by the CG operator
    int R;                 // positions per chunk
    double* sums;          // G x C, runs complete inside one chunk
    double* head;          // nchunks x C
    double* tail;          // nchunks x C
};

template <typename T>
struct SmallGParams {
    T* X;
    int C;
    long long n;
    const int32_t* gid;    // 0-based group id of each storage row for the projected dimension
    int G;
    PendingSet<T> pend;    // gid arrays indexed by storage row
    int writeback;
    int no_data;
    long long rows_per_block;
    double* partials;      // nblocks x G x C
    int tld;               // row stride of the pending tables (0 = C)
};

struct FinalizeParams {
    int G;
    int C;
    // source of the group sums: segments (off/sums/head/tail, chunk size R) or
    // small-G block partials (partials, nblocks)
    // source of the group sums: off == null && partials == null means sums[]
    // already holds complete group sums
    const int32_t* off;
    const double* sums;
    const double* head;
    const double* tail;
    int R;
    const double* partials;
    int nblocks;
    const int32_t* counts;  // G group sizes
    const double* inv_counts;  // optional G reciprocals (0 for empty groups); used instead of dividing
    const double* bias;     // optional G x C added to the mean
    double* prev;           // optional over-relaxation memory; null = no mixing
    const double* relax;    // device scalar (relaxation of this dimension), used when prev != null
    double* pend64;         // optional pending table (FP64)
    float* pend32;          // optional pending table (FP32 copy)
    int pend_accumulate;    // add to the pending table instead of overwriting it
    double* alpha;          // optional accumulated FE coefficients (+= mixed)
    double* mean_out;       // optional plain means
    double* sum_out;        // optional plain sums
    // max |mixed| of this launch: per-block maxima in max_partials, folded by
    // a one-block kernel into change_bits (atomic max, one per launch) and,
    // with do_relax_update, into the adaptive relaxation state
    // (fe_gpu_demean.f90:213-218)
    double* max_partials;
    unsigned long long* change_bits;
    int do_relax_update;
    double* relax_rw;
    double* prev_change;
    unsigned long long* max_update_bits;
};

inline int finalize_blocks(long long gc) { return (int)((gc + 255) / 256); }

// Groups whose segment run spans more than SEG_LONG_SPAN chunks have their
// chunk-edge partials folded by a block-wide tree (launch_long_sums) into
// sums[g]; finalize-type kernels then read sums[g] for them.
constexpr int SEG_LONG_SPAN = 32;

// Lists the long groups of a segment traversal (device list, count on host).
int find_long_groups(const int32_t* off, int G, int R, int32_t* list, int* n_long, cudaStream_t s);
// sums[g][c] = tail[qs][c] + sum_{qs<q<=qe} head[q][c] for the listed groups.
int launch_long_sums(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                     int n_long, double* sums, cudaStream_t s);
// sums[g][c] = sum_b partials[b][g][c] (small-G block partials, fixed tree order).
int launch_fold_smallg(const double* partials, int nblocks, int G, int C, double* sums, cudaStream_t s);

// Launch helpers. Return 0 or a status.
template <typename T>
int launch_seg_sweep(const SegSweepParams<T>& p, cudaStream_t s);
template <typename T>
int launch_smallg_sweep(const SmallGParams<T>& p, int nblocks, cudaStream_t s);
int launch_finalize(const FinalizeParams& p, cudaStream_t s);

// Number of chunks for a segment traversal.
inline long long seg_nchunks(long long n, int R) { return (n + R - 1) / R; }
// Number of blocks used by the small-G kernel for n rows.
int smallg_nblocks(long long n);
// Whether the small-G path can hold G x C per thread slot in shared memory.
bool smallg_eligible(int G, int C);

// X[row][col] -= sum_e pend.tab[e][pend.gid[e][row]][col] over storage order.
template <typename T>
int launch_apply_pending(T* X, int C, long long n, const PendingSet<T>& pend, cudaStream_t s);

// dst (float) = (float) src (double), n elements
int launch_convert_f64_f32(const double* src, float* dst, long long n, cudaStream_t s);

// ---- row-per-lane operator sweep for the CG normal-equation operator ----
// Position j of a dimension's group-sorted order has destination group
// gseq[j] and source ids src_gid[e][j] for the other dimensions; the sweep
// forms, per destination group, sum over its positions of
// -(sum_e src_tab[e][src_gid[e][j]]) (no row data). Each warp owns a chunk of
// CG_CHUNK = 32 x 16 positions; each lane accumulates its 16 positions (runs
// of equal destination in registers, storage type T); runs that cross lanes
// are combined by a warp scan in FP64. Output layout as the segment sweep
// (sums / head / tail with chunk size CG_CHUNK).
constexpr int CG_LANE_POS = 16;
constexpr int CG_CHUNK = 32 * CG_LANE_POS;

template <typename T>
struct CGRowsParams {
    long long n;
    int C;                 // real columns
    int ld;                // row stride of the tables and of sums/head/tail (see cg_row_stride)
    const int32_t* gseq;
    int n_src;
    const int32_t* src_gid[SWEEP_MAXP];
    const T* src_tab[SWEEP_MAXP];
    double* sums;
    double* head;
    double* tail;
    // Optional side output of the storage-order (primary) pass: the operator
    // sums of one small-G dimension, accumulated in fixed point (int64, so
    // the result does not depend on the order of the adds). For each
    // position the pass adds v - p_primary (v = its own contribution) to the
    // small dimension's group; cg_sg_fold adds count * p_small afterwards.
    int sg_src = -1;              // index of the small dimension among the sources; -1 = none
    int sg_G = 0;                 // its groups
    int n_dims = 0;               // FE dimensions (bounds |v - p_primary| by n_dims * pmax)
    const T* prim_tab = nullptr;  // primary dimension's p rows (stride ld)
    const unsigned long long* pmax_bits = nullptr;  // max |p| (bits of a non-negative double)
    long long* sg_part = nullptr;  // per block: sg_G x C int64 sums
};

template <typename T>
int launch_cg_rows(const CGRowsParams<T>& p, cudaStream_t s);

// shared memory limit of the small-G side table (sg_G x C int64)
constexpr size_t CG_SG_SMEM_MAX = 40 * 1024;

// blocks of one operator launch over n positions and C columns with column tile `tile`
inline long long cg_rows_blocks(long long n, int C, int tile) {
    const int ntiles = (C + tile - 1) / tile;
    const long long warps = ((n + CG_CHUNK - 1) / CG_CHUNK) * ntiles;
    return (warps * 32 + 255) / 256;
}
// the column tile launch_cg_rows picks for C columns
inline int cg_rows_tile(int C) { return C <= 4 ? 4 : C <= 8 ? 8 : C == 9 ? 9 : C <= 12 ? 12 : 16; }

// the vector id path (needed by the small-G side output): 1..3 sources and
// 16-byte aligned id arrays
template <typename T>
inline bool cg_rows_vector_path(const CGRowsParams<T>& p) {
    if (p.n_src < 1 || p.n_src > 3) return false;
    bool aligned = (reinterpret_cast<uintptr_t>(p.gseq) & 15u) == 0;
    for (int e = 0; e < p.n_src; ++e) aligned = aligned && (reinterpret_cast<uintptr_t>(p.src_gid[e]) & 15u) == 0;
    return aligned;
}

// Fixed-point exponent of the small-G side output: values are scaled by
// 2^e so that n sums of |v| <= n_dims * pmax stay below 2^62.
__host__ __device__ inline int cg_sg_exponent(double pmax, int n_dims, long long n) {
    double b = (double)(n_dims > 0 ? n_dims : 1) * pmax;
    if (!(b > 0.0)) b = 1.0;
    int eb = 0;
    frexp(b, &eb);  // b < 2^eb
    int en = 1;
    while (en < 62 && (1LL << en) <= n) ++en;  // n < 2^en
    int e = 62 - en - eb;
    return e > 100 ? 100 : (e < -100 ? -100 : e);
}

// sums[g * C + c] = sum over blocks of part (exact int64) / 2^e + counts[g] * ps[g * ld + c]:
// the small dimension's operator sums (sums of -p over the other dimensions).
template <typename T>
int launch_cg_sg_fold(const long long* part, int nblocks, int G, int C, const unsigned long long* pmax_bits,
                      int n_dims, long long n, const int32_t* counts, const T* ps, int ld, double* sums, cudaStream_t s);

// max |p| over the G-space direction (bits of a non-negative double), from per-block maxima.
int launch_fold_max(const double* partials, int nb, unsigned long long* out, cudaStream_t s);

// Row stride of the CG G-space vectors: rows padded to 32-byte multiples (a
// multiple of 16 columns above 16) so that table rows load as 256-bit vectors.
inline int cg_row_stride(int C, int elem_bytes) {
    const int vec = 32 / elem_bytes;
    if (C <= 16) return ((C + vec - 1) / vec) * vec;
    return ((C + 15) / 16) * 16;
}

// ---- conjugate gradients on the FE normal equations (D'D a = D'e) ----
// G-space vectors of all dimensions are concatenated: element (g, c) of
// dimension d sits at ((goff_d + g) * C + c) for r, z, q and x (compact rows).
// The direction p, which the operator sweep gathers, has rows padded to the
// stride pld (cg_row_stride), its padding kept at zero. Per-column scalars
// (C values) live on the device; dot products use per-block partials folded
// in block order, so every reduction is deterministic.

// q_d = counts_d * p_d - S_d, where S_d are the group sums of a no-data sweep
// with pending tables {p_e, e != d} (sums of -p_e over the rows of each
// group). Also writes per-block partials of p.q per column.
// src.C is the padded row stride of the sweep sums; q is compact (C columns).
template <typename T>
int launch_cg_q(const FinalizeParams& src, int C, const T* p, int pld, T* q, double* pq_partials, cudaStream_t s);
int cg_partial_blocks(long long gc);

// out[c] = sum_b partials[b * C + c] for b < nb (fixed order)
int launch_fold_partials(const double* partials, int nb, int C, double* out, cudaStream_t s);

// a = rz / pq per column (0 where pq == 0), then for every element, in T:
// x += a p, r -= a q, z = r / count (0 for empty groups); partials of r.z
// per column and max |z| (bits, device scalar).
template <typename T>
int launch_cg_update(long long Gt, int C, const T* inv_counts, const double* rz, const double* pq, const T* p,
                     int pld, const T* q, T* x, T* r, T* z, double* rz_partials, double* zmax_partials,
                     unsigned long long* zmax, cudaStream_t s);
// dst[g * C + c] = (double) src[g * ld + c] for c < C
template <typename T>
int launch_to_f64(const T* src, int ld, double* dst, int C, long long G, cudaStream_t s);
// inv[g] = 1 / counts[g] in T (0 for empty groups)
template <typename T>
int launch_inv_counts_t(const int32_t* counts, long long G, T* inv, cudaStream_t s);

// b = rz_new / rz_old per column; p = z + b p; rz_old = rz_new
template <typename T>
// skip (device, optional): when *skip != 0 both kernels return at once (the
// direction step of a graph-driven loop that has stopped).
// pmax_partials (optional): per-block max |p| after the update (grid_stride_blocks(Gt * C, 256) entries),
// folded into pmax_bits.
int launch_cg_direction(long long Gt, int C, double* rz_old, const double* rz_new, const T* z, T* p, int pld,
                        cudaStream_t s, const int* skip = nullptr, double* pmax_partials = nullptr,
                        unsigned long long* pmax_bits = nullptr);

// r = counts * mu, z = p = mu (cast to T); partials of r.z and max |z|
// inv_counts[g] = 1 / counts[g] (0 for empty groups)
int launch_inv_counts(const int32_t* counts, long long G, double* inv_counts, cudaStream_t s);

// mu is G x C; p is written at the padded stride pld (its padding is left untouched).
template <typename T>
int launch_cg_init(long long Gt, int C, const int32_t* counts, const double* mu, T* r, T* z, T* p, int pld, T* x,
                   double* rz_partials, double* zmax_partials, unsigned long long* zmax, cudaStream_t s);

}  // namespace fegb
