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
    int no_data;           // 1: rows are not read (value = 0 - pending); the fits leave it 0
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
    // already holds complete group sums (sums == null: all zero)
    const int32_t* off;
    const double* sums;
    const float* sums32;  // FP32 complete sums, used instead of sums when set
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
// Groups whose run crosses 1..SEG_LONG_SPAN chunk boundaries (list order unspecified).
int find_multi_groups(const int32_t* off, int G, int R, int32_t* list, int* n_multi, cudaStream_t s);
// Completes sums[g * C + c] of the listed long and multi-chunk groups from the
// chunk tail/head partials (each group summed in chunk order), so that sums
// then holds every group's complete sum.
template <typename S>
int launch_group_sums(const int32_t* off, const double* head, const double* tail, int R, int C,
                      const int32_t* long_list, int n_long, const int32_t* multi_list, int n_multi, S* sums,
                      cudaStream_t s);
// sums[g][c] = tail[qs][c] + sum_{qs<q<=qe} head[q][c] for the listed groups.
int launch_long_sums(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                     int n_long, double* sums, cudaStream_t s);
int launch_long_sums(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                     int n_long, float* sums, cudaStream_t s);
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

// ---- position sweep for the CG normal-equation operator ----
// Position j of a dimension's group-sorted stream has destination group
// gseq[j], source ids src_gid[e][j] for the other swept dimensions and an
// optional weight w[j] (the rows it stands for); the sweep forms, per
// destination group, the sum over its positions of
// -w[j] (sum_e src_tab[e][src_gid[e][j]]) (no row data). Each warp owns a
// chunk of CG_CHUNK = 32 x CG_LANE_POS positions; each lane accumulates its
// positions (runs of equal destination in registers, storage type T); runs
// that cross lanes are combined by a flag-precomputed warp scan in T. Output:
// complete-run sums (T) and chunk head/tail partials (FP64), compact rows.
constexpr int CG_LANE_POS = 8;
constexpr int CG_CHUNK = 32 * CG_LANE_POS;

template <typename T>
struct CGRowsParams {
    long long n;
    int C;                 // real columns
    int ld;                // row stride of the gathered tables (see cg_row_stride)
    const int32_t* gseq;
    int n_src;
    const int32_t* src_gid[SWEEP_MAXP];
    const T* src_tab[SWEEP_MAXP];
    // optional multiplicity of each position (a position then stands for that
    // many rows with the same ids); 16-byte aligned like the id arrays
    const float* weight;
    // outputs at the compact stride C: complete-run sums in the storage type
    // (runs are summed in T), chunk head/tail partials in FP64
    T* sums;
    double* head;
    double* tail;
};

template <typename T>
int launch_cg_rows(const CGRowsParams<T>& p, cudaStream_t s);

// Operator sweep of a stream whose groups all have few positions (at most
// CG_SHORT_MAX, on average at most CG_SHORT_MEAN): one thread per (group,
// column tile) writes the complete group sums into p.sums; the chunk heads,
// tails and the group-sum pass are not used. off: G + 1 offsets of the groups'
// positions; p.n_src from 1 to 3.
constexpr int CG_SHORT_MAX = 64;
constexpr int CG_SHORT_MEAN = 8;
template <typename T>
int launch_cg_short(const CGRowsParams<T>& p, const int32_t* off, int G, cudaStream_t s);
// Largest off[g + 1] - off[g] over the G groups (host result, synchronises s).
int max_group_length(const int32_t* off, int G, int* out, cudaStream_t s);

// Row stride of the CG G-space vectors: rows padded to 32-byte multiples so
// that table rows load as 256-bit vectors (a tile of 16 columns starts at a
// multiple of 64 bytes, its last piece ends inside the padded row). No more
// padding than that: every padded byte is gathered with the row (24 FP32
// columns: 96-byte rows, not 128).
inline int cg_row_stride(int C, int elem_bytes) {
    const int vec = 32 / elem_bytes;
    return ((C + vec - 1) / vec) * vec;
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
// extra (optional, G x C compact): added to q (contributions computed apart
// from the sweep, e.g. from dense small-G count matrices).
template <typename T>
int launch_cg_q(const FinalizeParams& src, int C, const T* p, int pld, T* q, double* pq_partials, cudaStream_t s,
                const T* extra = nullptr);

// ---- dense count matrices of small-G dimensions ----
// For a dimension s with few groups and any other dimension e, the operator
// coupling D_s' D_e is the G_e x G_s count matrix N (rows of each (group of e,
// group of s) pair), built once. N[g * Gs + t] counts the rows with gid_e = g
// and gid_s = t; stored as uint8 when every count is below 256.
constexpr int DENSE_SMALL_MAX_G = 64;
constexpr int DENSE_TILE = 64;          // groups per shared-memory tile of the dense products
constexpr int DENSE_MAX_BLOCKS = 608;   // partial blocks of a product (fixed: the same sums on any GPU)
int launch_count_pairs(const int32_t* gid_e, const int32_t* gid_s, long long n, int Gs, uint32_t* N, cudaStream_t s);
// *mx = max of N[0..cnt)
int launch_count_max(const uint32_t* N, long long cnt, unsigned* mx, cudaStream_t s);
// out = (uint8) N
int launch_narrow_counts(const uint32_t* N, long long cnt, uint8_t* out, cudaStream_t s);
// number of partial blocks of a product over Ge groups
inline int dense_chunks(long long Ge) {
    const long long tiles = (Ge + DENSE_TILE - 1) / DENSE_TILE;
    return (int)(tiles < DENSE_MAX_BLOCKS ? tiles : DENSE_MAX_BLOCKS);
}
// One pass over the count matrix M (Ge x Gs) of a small dimension s and a
// dimension e: partials[block][t][c] = sum over the block's groups g of
// M[g][t] * pe[g * ld + c] (dense_chunks(Ge) blocks), and, when extra is not
// null, extra[g * C + c] (+)= sum_t M[g][t] * ps[t * ld + c] (accumulate = 0
// overwrites). partials null: only the extra side (pe is not read). pe and M
// start on 16 bytes and ld is a multiple of 16 bytes.
// Schur form of the pass over the primary's count matrix (one small dimension):
// with sums set, each group g of e gets u = (sums[g * C + c] - sum_t M[g][t] ps[t])
// / counts[g], written to table (row stride ld), and u is the pe of the small
// side (extra must be null). Zero-initialised = the plain pass.
template <typename T>
struct DenseSchur {
    const T* sums = nullptr;
    const int32_t* counts = nullptr;
    T* table = nullptr;
};
template <typename T, typename CT>
int launch_dense_pair(const CT* M, long long Ge, int Gs, const T* pe, const T* ps, int ld, int C, double* partials,
                      T* extra, int accumulate, cudaStream_t s, const DenseSchur<T>& sch = DenseSchur<T>());
// Form of the uint8 / FP32 dense pair pass on the calling host thread: the
// tensor-core form (tcgen05, BF16 pieces, FP32 accumulation; dense_umma.cu)
// by default wherever its shapes allow it (C <= 16, Gs <= 64, 16-byte aligned
// operands), else the FP32 CUDA-core form. mode 0 forces the CUDA-core form,
// mode 1 the tensor-core form, -1 restores the default; FEGB_DENSE_TENSOR=0 in
// the environment makes the CUDA-core form the default.
bool dense_use_mma();
void dense_force_mode(int mode);
// The tensor-core form of launch_dense_pair for FP32 storage and uint8 counts.
// *launched = false (status 0) when the shapes or alignments do not allow it.
int launch_dense_pair_umma(const uint8_t* M, long long Ge, int Gs, const float* pe, const float* ps, int ld, int C,
                           double* partials, float* extra, int accumulate, const DenseSchur<float>& sch,
                           cudaStream_t s, bool* launched);
// Reads (synchronising s) and optionally resets the error word of the
// tensor-core pass: nonzero when one of its bounded waits ran out of time.
int dense_umma_error(int* flag, bool reset, cudaStream_t s);
// Schur-complement CG helpers (the primary dimension eliminated):
// table[g * L + c] = (sums[g * C + c] - extra[g * C + c]) / counts[g] (extra optional)
template <typename T>
int launch_schur_u(const T* sums, const T* extra, const int32_t* counts, long long G, int C, T* table, int L,
                   cudaStream_t s);
// table[g * L + c] = (T)(scale * src[g * C + c])
template <typename T>
int launch_table_from_f64(const double* src, long long G, int C, double scale, T* table, int L, cudaStream_t s);
// table[g * L + c] = src[g * C + c]
template <typename T>
int launch_table_from_compact(const T* src, long long G, int C, T* table, int L, cudaStream_t s);
// alpha[g * C + c] = mu[g * C + c] + table[g * L + c]
template <typename T>
int launch_alpha_primary(const double* mu, const T* table, long long G, int C, int L, double* alpha, cudaStream_t s);
// Diagonal of the Schur complement D_R'(I - P_P)D_R as fixed-point sums (20
// fraction bits) of n_wg (n_w - n_wg) / n_w over the (group, primary group)
// pairs: acc must be zeroed first. Stream form: one position per pair, in
// group order (gseq), weight w (null = 1), primary group pid, primary counts nP.
int launch_schur_diag_stream(const int32_t* gseq, long long m, const float* w, const int32_t* pid, const int32_t* nP,
                             unsigned long long* acc, cudaStream_t s);
// Pair form: perm and off (npairs + 1) are the rows sorted by (group of the
// dimension, primary group) and the segments of equal pairs; gid_e and gid_p
// the two dimensions' group ids by row.
int launch_schur_diag_pairs(const int32_t* perm, const int32_t* off, long long npairs, const int32_t* gid_e,
                            const int32_t* gid_p, const int32_t* nP, unsigned long long* acc, cudaStream_t s);
// Dense form: N is the Ge x Gs count matrix (primary groups x the dimension's
// Gs <= DENSE_SMALL_MAX_G groups), n the primary counts; adds into acc[0..Gs).
template <typename CT>
int launch_schur_diag_dense(const CT* N, long long Ge, int Gs, const int32_t* n, unsigned long long* acc,
                            cudaStream_t s);
// inv[g] = 1 / S_gg, or 0 when S_gg <= 1e-9 counts[g] (no identifying variation)
template <typename T>
int launch_inv_diag(const unsigned long long* acc, const int32_t* counts, long long G, T* inv, cudaStream_t s);
// sums[t * C + c] = -(sum over parts of partials[part][t][c]), parts in order
int launch_fold_dense(const double* partials, int nparts, int Gs, int C, double* sums, cudaStream_t s);
// Partial blocks (one FP64 partial per column each) of the CG vector kernels
// over a G x C table: VEC_STEPS steps of 256 / C rows per block (C <= 256),
// else one block per 256 elements.
constexpr int VEC_STEPS = 16;
int cg_partial_blocks(long long G, int C);

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
// skip (device, optional): when *skip != 0 both kernels return at once (the
// direction step of a graph-driven loop that has stopped).
template <typename T>
int launch_cg_direction(long long Gt, int C, double* rz_old, const double* rz_new, const T* z, T* p, int pld,
                        cudaStream_t s, const int* skip = nullptr);

// r = counts * mu + qb (in FP64, cast to T), z = inv * r, p = z, x = 0; partials
// of r.z and max |z| (the start of a solve from a right-hand side counts * mu + qb)
template <typename T>
int launch_cg_init_rhs(long long Gt, int C, const int32_t* counts, const double* mu, const T* qb, const T* inv, T* r,
                       T* z, T* p, int pld, T* x, double* rz_partials, double* zmax_partials, unsigned long long* zmax,
                       cudaStream_t s);
// r = counts * mu, z = p = mu (cast to T); partials of r.z and max |z|
// inv_counts[g] = 1 / counts[g] (0 for empty groups)
int launch_inv_counts(const int32_t* counts, long long G, double* inv_counts, cudaStream_t s);

// mu is G x C; p is written at the padded stride pld (its padding is left untouched).
template <typename T>
int launch_cg_init(long long Gt, int C, const int32_t* counts, const double* mu, T* r, T* z, T* p, int pld, T* x,
                   double* rz_partials, double* zmax_partials, unsigned long long* zmax, cudaStream_t s);

}  // namespace fegb
