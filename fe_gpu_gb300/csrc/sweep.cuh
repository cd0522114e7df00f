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
    long long rows_per_block;
    double* partials;      // nblocks x G x C
};

struct FinalizeParams {
    int G;
    int C;
    // source of the group sums: segments (off/sums/head/tail, chunk size R) or
    // small-G block partials (partials, nblocks)
    const int32_t* off;
    const double* sums;
    const double* head;
    const double* tail;
    int R;
    const double* partials;
    int nblocks;
    const int32_t* counts;  // G group sizes
    const double* bias;     // optional G x C added to the mean
    double* prev;           // optional over-relaxation memory; null = no mixing
    const double* relax;    // device scalar (relaxation of this dimension), used when prev != null
    double* pend64;         // optional pending table (FP64)
    float* pend32;          // optional pending table (FP32 copy)
    int pend_accumulate;    // add to the pending table instead of overwriting it
    double* alpha;          // optional accumulated FE coefficients (+= mixed)
    double* mean_out;       // optional plain means
    double* sum_out;        // optional plain sums
    unsigned long long* change_bits;  // optional absmax(mixed) of this launch (bits)
    // last-block relaxation update (fe_gpu_demean.f90:213-218)
    int do_relax_update;
    unsigned int* done_counter;
    double* relax_rw;
    double* prev_change;
    unsigned long long* max_update_bits;
};

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

}  // namespace fegb
