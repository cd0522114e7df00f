// Alternating-projection sweep kernels (see sweep.cuh for the scheme).
#include "sweep.cuh"

#include <cstdlib>

#include <type_traits>

namespace fegb {

namespace {

constexpr int SW_THREADS = 256;

struct Geometry {
    int L;   // lanes per chunk slot (columns handled at once)
    int P;   // chunk slots per warp
    int CT;  // column tiles per chunk
};

inline Geometry geometry(int C) {
    Geometry g;
    g.L = C <= 32 ? C : 32;
    g.P = 32 / g.L;
    g.CT = (C + g.L - 1) / g.L;
    return g;
}

// Positions per lane loaded ahead of the accumulation: the sweeps are bound by
// the loads in flight (the FP64 segment sweep is given 80 registers, 3 blocks
// per SM, to hold 8 without spilling).
template <typename T>
struct SweepUnroll {
    static constexpr int U = 8;
};

template <typename T>
__global__ void __launch_bounds__(SW_THREADS, sizeof(T) == 8 ? 3 : 4)
    seg_sweep_kernel(SegSweepParams<T> p, int L, int P, int CT, long long n_items) {
    constexpr int U = SweepUnroll<T>::U;
    constexpr bool kF32 = sizeof(T) == 4;
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * SW_THREADS + threadIdx.x) >> 5;
    const int slot = lane / L;
    if (slot >= P) return;
    const long long item = warp * P + slot;
    if (item >= n_items) return;
    const int cl = lane - slot * L;
    const long long q = item / CT;
    const int C = p.C;
    const int col = (int)(item - q * CT) * L + cl;
    const bool col_ok = col < C;
    const int colc = col_ok ? col : C - 1;
    const long long j0 = q * (long long)p.R;
    const long long j1 = min(j0 + (long long)p.R, p.n);
    const int32_t* __restrict__ gseq = p.gseq;
    const int32_t* __restrict__ perm = p.perm;
    T* __restrict__ X = p.X;
    const int first_g = gseq[j0];
    const bool before = j0 > 0 && gseq[j0 - 1] == first_g;
    const int last_g = gseq[j1 - 1];
    const bool after = j1 < p.n && gseq[j1] == last_g;
    const int np = p.pend.n;

    int cur = first_g;
    bool first_run = true;
    double acc = 0.0;
    T part = T(0);

    for (long long j = j0; j < j1; j += U) {
        int g[U];
        int row[U];  // row indices fit in int32 (n < 2^31)
        T v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const long long jj = j + u;
            const bool ok = jj < j1;
            g[u] = ok ? gseq[jj] : cur;
            row[u] = ok ? ((perm && !p.no_data) ? perm[jj] : (int)jj) : -1;
        }
        if (p.no_data) {
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = T(0);
        } else {
#pragma unroll
            for (int u = 0; u < U; ++u) v[u] = row[u] >= 0 ? X[(long long)row[u] * p.rs + colc * p.cs] : T(0);
        }
        for (int e = 0; e < np; ++e) {
            const int32_t* __restrict__ pg = p.pend.gid[e];
            const T* __restrict__ tb = p.pend.tab[e];
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (row[u] >= 0) v[u] -= tb[(long long)pg[j + u] * C + colc];
        }
        if (p.writeback && col_ok && !p.no_data) {
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (row[u] >= 0) X[(long long)row[u] * p.rs + col * p.cs] = v[u];
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            if (row[u] < 0) continue;
            if (g[u] != cur) {
                if (kF32) {
                    acc += (double)part;
                    part = T(0);
                }
                if (col_ok) {
                    const bool is_head = first_run && before;
                    if (is_head)
                        p.head[q * C + col] = acc;
                    else
                        p.sums[(long long)cur * C + col] = acc;
                }
                acc = 0.0;
                first_run = false;
                cur = g[u];
            }
            if (kF32)
                part += v[u];
            else
                acc += (double)v[u];
        }
        if (kF32) {
            acc += (double)part;
            part = T(0);
        }
    }
    if (col_ok) {
        const bool is_head = first_run && before;
        if (is_head)
            p.head[q * C + col] = acc;
        else if (after)
            p.tail[q * C + col] = acc;
        else
            p.sums[(long long)cur * C + col] = acc;
    }
}

template <typename T>
__global__ void __launch_bounds__(256, 4) smallg_sweep_kernel(SmallGParams<T> p, int P) {
    constexpr int U = SweepUnroll<T>::U;
    // per-slot tables in the storage type (FP32 sums over a slot's short
    // row range in the FP32 form), folded across slots in FP64
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* tabs = reinterpret_cast<T*>(smem_raw);
    const int C = p.C;  // C <= 32, one column per lane
    const int nwarps = blockDim.x >> 5;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nslots = nwarps * P;
    const int GC = p.G * C;
    for (int i = threadIdx.x; i < nslots * GC; i += blockDim.x) tabs[i] = T(0);
    __syncthreads();
    const int slot = lane / C;
    if (slot < P) {
        const int s = warp * P + slot;
        T* tab = tabs + (long long)s * GC;
        const int col = lane - slot * C;
        const long long rb0 = (long long)blockIdx.x * p.rows_per_block;
        const long long rb1 = min(p.n, rb0 + p.rows_per_block);
        const long long sc = (p.rows_per_block + nslots - 1) / nslots;
        const long long r0 = rb0 + (long long)s * sc;
        const long long r1 = min(rb1, r0 + sc);
        const int32_t* __restrict__ gid = p.gid;
        T* __restrict__ X = p.X;
        const int np = p.pend.n;
        const long long tld = p.tld > 0 ? p.tld : C;
        for (long long j = r0; j < r1; j += U) {
            int g[U];
            T v[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ok[u] = (j + u) < r1;
                g[u] = ok[u] ? gid[j + u] : 0;
                v[u] = (ok[u] && !p.no_data) ? X[(j + u) * C + col] : T(0);
            }
            for (int e = 0; e < np; ++e) {
                const int32_t* __restrict__ pg = p.pend.gid[e];
                const T* __restrict__ tb = p.pend.tab[e];
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (ok[u]) v[u] -= tb[(long long)pg[j + u] * tld + col];
            }
            if (p.writeback && !p.no_data) {
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (ok[u]) X[(j + u) * C + col] = v[u];
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ok[u]) tab[g[u] * C + col] += v[u];
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < GC; e += blockDim.x) {
        double t = 0.0;
        for (int s = 0; s < nslots; ++s) t += (double)tabs[(long long)s * GC + e];
        p.partials[(long long)blockIdx.x * GC + e] = t;
    }
}

constexpr int FIN_THREADS = 256;

// Group sum (g, c) from a finalize source: small-G block partials in block
// order, or a segment run / chunk-edge partials in chunk order.
__device__ __forceinline__ double source_sum(const FinalizeParams& p, int g, int c, long long idx, long long total) {
    double sum = 0.0;
    if (p.partials) {
        for (int b = 0; b < p.nblocks; ++b) sum += p.partials[(long long)b * total + idx];
    } else if (!p.off) {
        // null: no swept source contributes
        sum = p.sums32 ? (double)p.sums32[idx] : (p.sums ? p.sums[idx] : 0.0);
    } else {
        const int s = p.off[g], e = p.off[g + 1];
        if (e > s) {
            const long long qs = s / p.R, qe = (e - 1) / p.R;
            if (qs == qe || qe - qs > SEG_LONG_SPAN) {
                sum = p.sums32 ? (double)p.sums32[idx] : p.sums[idx];  // complete run, or folded by launch_long_sums
            } else {
                sum = p.tail[qs * p.C + c];
                for (long long q = qs + 1; q <= qe; ++q) sum += p.head[q * p.C + c];
            }
        }
    }
    return sum;
}

__global__ void __launch_bounds__(FIN_THREADS) finalize_kernel(FinalizeParams p) {
    __shared__ double red[FIN_THREADS / 32];
    const long long idx = (long long)blockIdx.x * FIN_THREADS + threadIdx.x;
    const long long total = (long long)p.G * p.C;
    double amax = 0.0;
    if (idx < total) {
        // 32-bit division where the element count allows it (FP64-free integer path)
        const int g = total < 0x7fffffffLL ? (int)idx / p.C : (int)(idx / p.C);
        const int c = (int)(idx - (long long)g * p.C);
        const double sum = source_sum(p, g, c, idx, total);
        if (p.sum_out) p.sum_out[idx] = sum;
        // plain sums (cluster score sums): no mean, no reciprocal
        if (!(p.mean_out || p.prev || p.pend64 || p.pend32 || p.alpha || p.max_partials)) return;
        const int cnt = p.counts ? p.counts[g] : 0;
        // reciprocal multiply, as in src/gpu/fe_gpu_runtime.cu:195-200
        const double inv = p.inv_counts ? p.inv_counts[g] : (cnt > 0 ? 1.0 / (double)cnt : 0.0);
        double mean = sum * inv;
        if (p.bias) mean += p.bias[idx];
        if (p.mean_out) p.mean_out[idx] = mean;
        double mixed = mean;
        if (p.prev) {
            const double pv = p.prev[idx];
            mixed = pv + (*p.relax) * (mean - pv);
            p.prev[idx] = mixed;
        }
        if (p.pend64) {
            const double np = (p.pend_accumulate ? p.pend64[idx] : 0.0) + mixed;
            p.pend64[idx] = np;
            if (p.pend32) p.pend32[idx] = (float)np;
        } else if (p.pend32) {
            p.pend32[idx] = (p.pend_accumulate ? p.pend32[idx] : 0.0f) + (float)mixed;
        }
        if (p.alpha) p.alpha[idx] += mixed;
        amax = fabs(mixed);
    }
    if (p.max_partials) {
        amax = warp_max(amax);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = amax;
        __syncthreads();
        if (threadIdx.x == 0) {
            double m = red[0];
            for (int w = 1; w < FIN_THREADS / 32; ++w) m = fmax(m, red[w]);
            p.max_partials[blockIdx.x] = m;
        }
    }
}

// Folds the per-block maxima of one finalize launch; updates the dimension's
// relaxation from the change of this projection relative to the previous one.
__global__ void __launch_bounds__(FIN_THREADS) finalize_epilogue_kernel(FinalizeParams p, int nb) {
    __shared__ double smem[FIN_THREADS];
    double m = 0.0;
    for (int b = threadIdx.x; b < nb; b += FIN_THREADS) m = fmax(m, p.max_partials[b]);
    smem[threadIdx.x] = m;
    __syncthreads();
    for (int w = FIN_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) smem[threadIdx.x] = fmax(smem[threadIdx.x], smem[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double cd = smem[0];
    if (p.change_bits) atomic_max_nonneg(p.change_bits, cd);
    if (p.do_relax_update) {
        const double pc = *p.prev_change;
        double r = *p.relax_rw;
        if (cd > pc * 1.05)
            r = fmax(0.4, r * 0.5);
        else if (cd < pc * 0.8)
            r = fmin(2.0, r * 1.10);
        *p.relax_rw = r;
        *p.prev_change = cd;
        atomic_max_nonneg(p.max_update_bits, cd);
    }
}

template <typename T>
__global__ void apply_pending_kernel(T* __restrict__ X, int C, long long n, PendingSet<T> pend) {
    const long long total = n * (long long)C;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // (row, col) of i advanced incrementally: one 64-bit division per thread, not per element
    long long row = i / C;
    int col = (int)(i - row * C);
    const long long rstep = stride / C;
    const int cstep = (int)(stride - rstep * C);
    for (; i < total; i += stride) {
        T v = X[i];
        for (int e = 0; e < pend.n; ++e) v -= pend.tab[e][(long long)pend.gid[e][row] * C + col];
        X[i] = v;
        row += rstep;
        col += cstep;
        if (col >= C) {
            col -= C;
            ++row;
        }
    }
}

__global__ void convert_kernel(const double* __restrict__ src, float* __restrict__ dst, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) dst[i] = (float)src[i];
}


// Per-block, per-column partial sums of prod over a block's elements
// (element idx has column idx % C); fixed order, deterministic. Accumulates in
// A (FP32 for the FP32 form, FP64 otherwise); stored as FP64.
template <typename A>
__device__ __forceinline__ void column_partials(A prod, long long base, int C, A* smem, double* out) {
    smem[threadIdx.x] = prod;
    __syncthreads();
    if (threadIdx.x < C) {
        const int c = threadIdx.x;
        const int first = (int)((c - base % C + C) % C);
        A acc = A(0);
        for (int j = first; j < FIN_THREADS; j += C) acc += smem[j];
        out[(long long)blockIdx.x * C + c] = (double)acc;
    }
}

// ---- row-tiled CG vector kernels ----
// A block covers VEC_STEPS steps of rps = 256 / C rows of a G x C table
// (C <= 256); thread t handles column c = t % C of rows g0 + t / C + rps * k,
// so its column is fixed: products accumulate in one register per thread (in
// T, VEC_STEPS terms at most) and each block writes one FP64 partial per
// column, folded in row order. 32-bit index arithmetic per thread.
struct VecLane {
    int c;       // column
    int rr;      // row within a step
    int rps;     // rows per step
    bool active;
};

__device__ __forceinline__ VecLane vec_lane(int C) {
    VecLane v;
    v.rps = 256 / C;
    v.rr = (int)threadIdx.x / C;
    v.c = (int)threadIdx.x - v.rr * C;
    v.active = v.rr < v.rps;
    return v;
}

// partial[c] of this block = sum over its threads of column c (rows in order)
__device__ __forceinline__ void vec_column_partials(double prod, const VecLane& v, int C, double* red, double* out) {
    red[threadIdx.x] = v.active ? prod : 0.0;
    __syncthreads();
    if ((int)threadIdx.x < C) {
        double acc = 0.0;
        for (int j = 0; j < v.rps; ++j) acc += red[j * C + threadIdx.x];
        out[(long long)blockIdx.x * C + threadIdx.x] = acc;
    }
}

__device__ __forceinline__ void vec_block_max(double m, double* red8, double* out) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) red8[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double mm = red8[0];
        for (int w = 1; w < 8; ++w) mm = fmax(mm, red8[w]);
        out[blockIdx.x] = mm;
    }
}

template <typename T>
__global__ void __launch_bounds__(256) cg_q_rows_kernel(FinalizeParams src, int C, const T* __restrict__ p, int pld,
                                                        T* __restrict__ q, double* __restrict__ pq_partials,
                                                        const T* __restrict__ extra) {
    __shared__ double red[256];
    const VecLane v = vec_lane(C);
    T prod = T(0);
    if (v.active) {
        const long long g0 = (long long)blockIdx.x * v.rps * VEC_STEPS + v.rr;
#pragma unroll 4
        for (int k = 0; k < VEC_STEPS; ++k) {
            const long long gl = g0 + (long long)k * v.rps;
            if (gl >= src.G) break;
            const int g = (int)gl;
            const long long idx = gl * C + v.c;
            const int cnt = src.counts[g];
            // ssum = -(sum over the group's rows of the other dimensions' p); a group
            // without rows has none (and no sum written)
            const double ssum = cnt > 0 ? source_sum(src, g, v.c, gl * src.C + v.c, (long long)src.G * src.C) : 0.0;
            const T pv = p[gl * pld + v.c];
            T qv = (T)cnt * pv - (T)ssum;
            if (extra) qv += extra[idx];
            q[idx] = qv;
            prod += pv * qv;
        }
    }
    vec_column_partials((double)prod, v, C, red, pq_partials);
}

template <typename T>
__global__ void __launch_bounds__(256) cg_update_rows_kernel(long long Gt, int C, const T* __restrict__ inv_counts,
                                                             const double* __restrict__ rz,
                                                             const double* __restrict__ pq, const T* __restrict__ p,
                                                             int pld, const T* __restrict__ q, T* __restrict__ x,
                                                             T* __restrict__ r, T* __restrict__ z,
                                                             double* __restrict__ rz_partials,
                                                             double* __restrict__ zmax_partials) {
    __shared__ double red[256];
    __shared__ double red8[8];
    const VecLane v = vec_lane(C);
    T prod = T(0), az = T(0);
    if (v.active) {
        const double den = pq[v.c];
        const T a = (T)(den != 0.0 ? rz[v.c] / den : 0.0);
        const long long g0 = (long long)blockIdx.x * v.rps * VEC_STEPS + v.rr;
#pragma unroll 4
        for (int k = 0; k < VEC_STEPS; ++k) {
            const long long g = g0 + (long long)k * v.rps;
            if (g >= Gt) break;
            const long long idx = g * C + v.c;
            x[idx] += a * p[g * pld + v.c];
            const T rv = r[idx] - a * q[idx];
            const T zv = rv * inv_counts[g];
            r[idx] = rv;
            z[idx] = zv;
            prod += rv * zv;
            const T m = zv < T(0) ? -zv : zv;
            az = m > az ? m : az;
        }
    }
    vec_column_partials((double)prod, v, C, red, rz_partials);
    vec_block_max((double)az, red8, zmax_partials);
}

template <typename T>
__global__ void __launch_bounds__(256) cg_init_rows_kernel(long long Gt, int C, const int32_t* __restrict__ counts,
                                                           const double* __restrict__ mu, T* __restrict__ r,
                                                           T* __restrict__ z, T* __restrict__ p, int pld,
                                                           T* __restrict__ x, double* __restrict__ rz_partials,
                                                           double* __restrict__ zmax_partials) {
    __shared__ double red[256];
    __shared__ double red8[8];
    const VecLane v = vec_lane(C);
    T prod = T(0), az = T(0);
    if (v.active) {
        const long long g0 = (long long)blockIdx.x * v.rps * VEC_STEPS + v.rr;
        for (int k = 0; k < VEC_STEPS; ++k) {
            const long long g = g0 + (long long)k * v.rps;
            if (g >= Gt) break;
            const long long idx = g * C + v.c;
            const int cnt = counts[g];
            const T m = cnt > 0 ? (T)mu[idx] : T(0);
            const T rv = (T)cnt * m;
            r[idx] = rv;
            z[idx] = m;
            p[g * pld + v.c] = m;
            x[idx] = T(0);
            prod += rv * m;
            const T am = m < T(0) ? -m : m;
            az = am > az ? am : az;
        }
    }
    vec_column_partials((double)prod, v, C, red, rz_partials);
    vec_block_max((double)az, red8, zmax_partials);
}

template <typename T>
__global__ void __launch_bounds__(256) cg_init_rhs_rows_kernel(long long Gt, int C, const int32_t* __restrict__ counts,
                                                               const double* __restrict__ mu, const T* __restrict__ qb,
                                                               const T* __restrict__ inv, T* __restrict__ r,
                                                               T* __restrict__ z, T* __restrict__ p, int pld,
                                                               T* __restrict__ x, double* __restrict__ rz_partials,
                                                               double* __restrict__ zmax_partials) {
    __shared__ double red[256];
    __shared__ double red8[8];
    const VecLane v = vec_lane(C);
    T prod = T(0), az = T(0);
    if (v.active) {
        const long long g0 = (long long)blockIdx.x * v.rps * VEC_STEPS + v.rr;
        for (int k = 0; k < VEC_STEPS; ++k) {
            const long long g = g0 + (long long)k * v.rps;
            if (g >= Gt) break;
            const long long idx = g * C + v.c;
            const int cnt = counts[g];
            const T rv = cnt > 0 ? (T)((double)cnt * mu[idx] + (double)qb[idx]) : T(0);
            const T zv = rv * inv[g];
            r[idx] = rv;
            z[idx] = zv;
            p[g * pld + v.c] = zv;
            x[idx] = T(0);
            prod += rv * zv;
            const T am = zv < T(0) ? -zv : zv;
            az = am > az ? am : az;
        }
    }
    vec_column_partials((double)prod, v, C, red, rz_partials);
    vec_block_max((double)az, red8, zmax_partials);
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS) cg_q_kernel(FinalizeParams src, int C, const T* __restrict__ p,
                                                            int pld, T* __restrict__ q, double* __restrict__ pq_partials,
                                                            const T* __restrict__ extra) {
    // compact elements (g, c < C); p uses the padded stride pld
    __shared__ T smem[FIN_THREADS];
    const long long total = (long long)src.G * C;
    const long long base = (long long)blockIdx.x * FIN_THREADS;
    const long long idx = base + threadIdx.x;
    T prod = T(0);
    if (idx < total) {
        const int g = (int)(idx / C);
        const int c = (int)(idx - (long long)g * C);
        const double ssum = source_sum(src, g, c, (long long)g * src.C + c, (long long)src.G * src.C);
        const T pv = p[(long long)g * pld + c];
        // ssum = -(sum over the group's rows of the other dimensions' p)
        T qv = (T)src.counts[g] * pv - (T)ssum;
        if (extra) qv += extra[idx];
        q[idx] = qv;
        prod = pv * qv;
    }
    column_partials<T>(prod, base, C, smem, pq_partials);
}

// Fixed-shape block tree: thread t folds elements t, t + 256, ... in order,
// then a fixed pairwise tree over the 256 thread sums.
__device__ __forceinline__ double block_tree_sum(double v, double* smem) {
    smem[threadIdx.x] = v;
    __syncthreads();
    for (int w = FIN_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) smem[threadIdx.x] += smem[threadIdx.x + w];
        __syncthreads();
    }
    double r = smem[0];
    __syncthreads();
    return r;
}

// out[c] = fold over b of partials[b * C + c]; one block per column.
__global__ void __launch_bounds__(FIN_THREADS)
    fold_partials_kernel(const double* __restrict__ partials, int nb, int C, double* __restrict__ out) {
    __shared__ double smem[FIN_THREADS];
    const int c = blockIdx.x;
    double acc = 0.0;
    for (int b = threadIdx.x; b < nb; b += FIN_THREADS) acc += partials[(long long)b * C + c];
    double t = block_tree_sum(acc, smem);
    if (threadIdx.x == 0) out[c] = t;
}

// One block per long group: tail of its first chunk plus the heads of the
// following chunks, for every column.
template <typename S>
__global__ void __launch_bounds__(FIN_THREADS)
    long_sums_kernel(const int32_t* __restrict__ off, const double* __restrict__ head,
                     const double* __restrict__ tail, int R, int C, const int32_t* __restrict__ list,
                     S* __restrict__ sums) {
    __shared__ double smem[FIN_THREADS];
    const int g = list[blockIdx.x];
    const long long qs = off[g] / R, qe = (off[g + 1] - 1) / R;
    for (int c = 0; c < C; ++c) {
        double acc = 0.0;
        for (long long q = qs + 1 + threadIdx.x; q <= qe; q += FIN_THREADS) acc += head[q * C + c];
        double t = block_tree_sum(acc, smem);
        if (threadIdx.x == 0) sums[(long long)g * C + c] = (S)(tail[qs * C + c] + t);
    }
}

// One warp per (g, c): strided fold over the block partials, then a fixed
// shuffle tree.
__global__ void fold_smallg_kernel(const double* __restrict__ partials, int nblocks, long long GC,
                                   double* __restrict__ sums) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= GC) return;
    double acc = 0.0;
    for (int b = lane; b < nblocks; b += 32) acc += partials[(long long)b * GC + w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) sums[w] = acc;
}

__global__ void find_long_kernel(const int32_t* __restrict__ off, int G, int R, int32_t* __restrict__ list,
                                 int* __restrict__ count) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const int s = off[g], e = off[g + 1];
    if (e > s && (long long)((e - 1) / R) - (long long)(s / R) > SEG_LONG_SPAN) list[atomicAdd(count, 1)] = g;
}

// groups whose segment run crosses 1..SEG_LONG_SPAN chunk boundaries
__global__ void find_multi_kernel(const int32_t* __restrict__ off, int G, int R, int32_t* __restrict__ list,
                                  int* __restrict__ count) {
    int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const int s = off[g], e = off[g + 1];
    if (e <= s) return;
    const long long span = (long long)((e - 1) / R) - (long long)(s / R);
    if (span >= 1 && span <= SEG_LONG_SPAN) list[atomicAdd(count, 1)] = g;
}

// Completes the sums of the groups whose run crosses chunk boundaries: blocks
// [0, n_long) take one long group each (block tree over its chunk heads),
// later blocks take 8 multi-chunk groups, one warp each (lane = column,
// heads in chunk order). sums[g * C + c] = tail[qs] + head[qs + 1] + ... + head[qe].
template <typename S>
__global__ void __launch_bounds__(FIN_THREADS)
    group_sums_kernel(const int32_t* __restrict__ off, const double* __restrict__ head,
                      const double* __restrict__ tail, int R, int C, const int32_t* __restrict__ long_list,
                      int n_long, const int32_t* __restrict__ multi_list, int n_multi, S* __restrict__ sums) {
    __shared__ double smem[FIN_THREADS];
    if ((int)blockIdx.x < n_long) {
        const int g = long_list[blockIdx.x];
        const long long qs = off[g] / R, qe = (off[g + 1] - 1) / R;
        for (int c = 0; c < C; ++c) {
            double acc = 0.0;
            for (long long q = qs + 1 + threadIdx.x; q <= qe; q += FIN_THREADS) acc += head[q * C + c];
            const double t = block_tree_sum(acc, smem);
            if (threadIdx.x == 0) sums[(long long)g * C + c] = (S)(tail[qs * C + c] + t);
        }
        return;
    }
    const long long w = (long long)(blockIdx.x - n_long) * (FIN_THREADS / 32) + (threadIdx.x >> 5);
    if (w >= n_multi) return;
    const int g = multi_list[w];
    const long long qs = off[g] / R, qe = (off[g + 1] - 1) / R;
    for (int c = threadIdx.x & 31; c < C; c += 32) {
        double acc = tail[qs * C + c];
        for (long long q = qs + 1; q <= qe; ++q) acc += head[q * C + c];
        sums[(long long)g * C + c] = (S)acc;
    }
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS)
    cg_update_kernel(long long Gt, int C, const T* __restrict__ inv_counts, const double* __restrict__ rz,
                     const double* __restrict__ pq, const T* __restrict__ p, int pld, const T* __restrict__ q,
                     T* __restrict__ x, T* __restrict__ r, T* __restrict__ z, double* __restrict__ rz_partials,
                     double* __restrict__ zmax_partials) {
    __shared__ T smem[FIN_THREADS];
    __shared__ T red[FIN_THREADS / 32];
    __shared__ T step[64];
    const long long total = Gt * C;
    const long long base = (long long)blockIdx.x * FIN_THREADS;
    const long long idx = base + threadIdx.x;
    if (threadIdx.x < C && threadIdx.x < 64) {
        const double den = pq[threadIdx.x];
        step[threadIdx.x] = (T)(den != 0.0 ? rz[threadIdx.x] / den : 0.0);
    }
    __syncthreads();
    T prod = T(0), az = T(0);
    if (idx < total) {
        const long long g = idx / C;
        const int c = (int)(idx - g * C);
        const T a = C <= 64 ? step[c] : (T)(pq[c] != 0.0 ? rz[c] / pq[c] : 0.0);
        x[idx] += a * p[g * pld + c];
        const T rv = r[idx] - a * q[idx];
        const T zv = rv * inv_counts[g];
        r[idx] = rv;
        z[idx] = zv;
        prod = rv * zv;
        az = zv < T(0) ? -zv : zv;
    }
    column_partials<T>(prod, base, C, smem, rz_partials);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T y = __shfl_xor_sync(0xffffffffu, az, o);
        az = y > az ? y : az;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = az;
    __syncthreads();
    if (threadIdx.x == 0) {
        T m = red[0];
        for (int w = 1; w < FIN_THREADS / 32; ++w) m = red[w] > m ? red[w] : m;
        zmax_partials[blockIdx.x] = (double)m;
    }
}

template <typename T>
__global__ void cg_direction_kernel(long long Gt, int C, const double* __restrict__ rz_old,
                                    const double* __restrict__ rz_new, const T* __restrict__ z, T* __restrict__ p,
                                    int pld, const int* __restrict__ skip) {
    if (skip && *skip) return;  // the loop has stopped (graph-driven loop)
    __shared__ double beta[64];
    if (threadIdx.x < C && threadIdx.x < 64)
        beta[threadIdx.x] = rz_old[threadIdx.x] != 0.0 ? rz_new[threadIdx.x] / rz_old[threadIdx.x] : 0.0;
    __syncthreads();
    const long long total = Gt * C;
    long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    // (g, c) of idx, advanced incrementally (no 64-bit division per element)
    long long g = idx / C;
    int c = (int)(idx - g * C);
    const long long gstep = st / C;
    const int cstep = (int)(st - gstep * C);
    for (; idx < total; idx += st) {
        const T b = C <= 64 ? (T)beta[c] : (T)(rz_old[c] != 0.0 ? rz_new[c] / rz_old[c] : 0.0);
        T* pe = p + g * pld + c;
        *pe = z[idx] + b * *pe;
        g += gstep;
        c += cstep;
        if (c >= C) {
            c -= C;
            ++g;
        }
    }
}

__global__ void inv_counts_kernel(const int32_t* __restrict__ counts, long long G, double* __restrict__ inv) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < G) inv[g] = counts[g] > 0 ? 1.0 / (double)counts[g] : 0.0;
}

__global__ void copy_scalars_kernel(const double* __restrict__ src, double* __restrict__ dst, int C,
                                    const int* __restrict__ skip) {
    if (skip && *skip) return;
    const int c = threadIdx.x;
    if (c < C) dst[c] = src[c];
}

template <typename T>
__global__ void __launch_bounds__(FIN_THREADS)
    cg_init_kernel(long long Gt, int C, const int32_t* __restrict__ counts, const double* __restrict__ mu,
                   T* __restrict__ r, T* __restrict__ z, T* __restrict__ p, int pld, T* __restrict__ x,
                   double* __restrict__ rz_partials, double* __restrict__ zmax_partials) {
    __shared__ T smem[FIN_THREADS];
    __shared__ T red[FIN_THREADS / 32];
    const long long total = Gt * C;
    const long long base = (long long)blockIdx.x * FIN_THREADS;
    const long long idx = base + threadIdx.x;
    T prod = T(0), az = T(0);
    if (idx < total) {
        const long long g = idx / C;
        const int c = (int)(idx - g * C);
        const int cnt = counts[g];
        const T m = cnt > 0 ? (T)mu[g * C + c] : T(0);
        const T rv = (T)cnt * m;
        r[idx] = rv;
        z[idx] = m;
        p[g * pld + c] = m;
        x[idx] = T(0);
        prod = rv * m;
        az = m < T(0) ? -m : m;
    }
    column_partials<T>(prod, base, C, smem, rz_partials);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const T y = __shfl_xor_sync(0xffffffffu, az, o);
        az = y > az ? y : az;
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = az;
    __syncthreads();
    if (threadIdx.x == 0) {
        T mm = red[0];
        for (int w = 1; w < FIN_THREADS / 32; ++w) mm = red[w] > mm ? red[w] : mm;
        zmax_partials[blockIdx.x] = (double)mm;
    }
}

template <typename T>
__global__ void to_f64_kernel(const T* __restrict__ src, int ld, double* __restrict__ dst, int C, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        const long long g = i / C;
        dst[i] = (double)src[g * ld + (i - g * C)];
    }
}

template <typename T>
__global__ void inv_counts_t_kernel(const int32_t* __restrict__ counts, long long G, T* __restrict__ inv) {
    long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g < G) inv[g] = counts[g] > 0 ? T(1) / (T)counts[g] : T(0);
}

// out (bits) = max over partials (one block, fixed tree); max is exact.
__global__ void __launch_bounds__(FIN_THREADS) fold_max_kernel(const double* __restrict__ partials, int nb,
                                                              unsigned long long* __restrict__ out) {
    __shared__ double smem[FIN_THREADS];
    double m = 0.0;
    for (int b = threadIdx.x; b < nb; b += FIN_THREADS) m = fmax(m, partials[b]);
    smem[threadIdx.x] = m;
    __syncthreads();
    for (int w = FIN_THREADS / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) smem[threadIdx.x] = fmax(smem[threadIdx.x], smem[threadIdx.x + w]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = dbl_bits(smem[0]);
}

constexpr int SMALLG_SMEM_BUDGET = 96 * 1024;

}  // namespace

template <typename T>
int launch_seg_sweep(const SegSweepParams<T>& p, cudaStream_t s) {
    if (p.n <= 0) return 0;
    Geometry g = geometry(p.C);
    long long nchunks = seg_nchunks(p.n, p.R);
    long long n_items = nchunks * g.CT;
    long long warps = (n_items + g.P - 1) / g.P;
    long long blocks = (warps * 32 + SW_THREADS - 1) / SW_THREADS;
    seg_sweep_kernel<T><<<(unsigned)blocks, SW_THREADS, 0, s>>>(p, g.L, g.P, g.CT, n_items);
    FEGB_LAUNCH_CHECK("segment sweep");
    return 0;
}

bool smallg_eligible(int G, int C) {
    if (C > 32 || G <= 0) return false;
    const int P = 32 / C;
    return (long long)P * G * C * (long long)sizeof(double) <= SMALLG_SMEM_BUDGET;
}

int smallg_nblocks(long long n) {
    long long nb = (long long)num_sms() * 4;
    long long min_rows = 4096;
    if (n / nb < min_rows) nb = (n + min_rows - 1) / min_rows;
    if (nb < 1) nb = 1;
    return (int)nb;
}

template <typename T>
int launch_smallg_sweep(const SmallGParams<T>& p, int nblocks, cudaStream_t s) {
    if (p.n <= 0) return 0;
    if (!smallg_eligible(p.G, p.C)) return set_error("small-G sweep: G=%d C=%d not eligible", p.G, p.C);
    const int P = 32 / p.C;
    const long long per_warp = (long long)P * p.G * p.C * sizeof(T);
    int nwarps = (int)(SMALLG_SMEM_BUDGET / per_warp);
    if (nwarps > 8) nwarps = 8;
    if (nwarps < 1) nwarps = 1;
    size_t smem = (size_t)nwarps * per_warp;
    // set once per instantiation (thread-safe static initialisation)
    static const cudaError_t attr_status =
        cudaFuncSetAttribute(smallg_sweep_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMALLG_SMEM_BUDGET);
    if (attr_status != cudaSuccess) return set_cuda_error(attr_status, "small-G smem attribute");
    smallg_sweep_kernel<T><<<nblocks, nwarps * 32, smem, s>>>(p, P);
    FEGB_LAUNCH_CHECK("small-G sweep");
    return 0;
}

int launch_finalize(const FinalizeParams& p, cudaStream_t s) {
    long long total = (long long)p.G * p.C;
    if (total <= 0) return 0;
    unsigned blocks = (unsigned)((total + FIN_THREADS - 1) / FIN_THREADS);
    finalize_kernel<<<blocks, FIN_THREADS, 0, s>>>(p);
    FEGB_LAUNCH_CHECK("finalize");
    if (p.max_partials && (p.change_bits || p.do_relax_update)) {
        finalize_epilogue_kernel<<<1, FIN_THREADS, 0, s>>>(p, (int)blocks);
        FEGB_LAUNCH_CHECK("finalize epilogue");
    }
    return 0;
}

template <typename T>
int launch_apply_pending(T* X, int C, long long n, const PendingSet<T>& pend, cudaStream_t s) {
    if (pend.n == 0 || n <= 0) return 0;
    apply_pending_kernel<T><<<grid_stride_blocks(n * C, 256), 256, 0, s>>>(X, C, n, pend);
    FEGB_LAUNCH_CHECK("apply pending");
    return 0;
}

int launch_convert_f64_f32(const double* src, float* dst, long long n, cudaStream_t s) {
    if (n <= 0) return 0;
    convert_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(src, dst, n);
    FEGB_LAUNCH_CHECK("convert");
    return 0;
}


int cg_partial_blocks(long long G, int C) {
    if (C <= 256) {
        const long long rows = (long long)(256 / C) * VEC_STEPS;
        return (int)((G + rows - 1) / rows);
    }
    return (int)((G * C + FIN_THREADS - 1) / FIN_THREADS);
}

template <typename T>
int launch_cg_q(const FinalizeParams& src, int C, const T* p, int pld, T* q, double* pq_partials, cudaStream_t s,
                const T* extra) {
    long long total = (long long)src.G * C;
    if (total <= 0) return 0;
    const int nb = cg_partial_blocks(src.G, C);
    if (C <= 256)
        cg_q_rows_kernel<T><<<nb, 256, 0, s>>>(src, C, p, pld, q, pq_partials, extra);
    else
        cg_q_kernel<T><<<nb, FIN_THREADS, 0, s>>>(src, C, p, pld, q, pq_partials, extra);
    FEGB_LAUNCH_CHECK("cg q");
    return 0;
}

int launch_fold_partials(const double* partials, int nb, int C, double* out, cudaStream_t s) {
    fold_partials_kernel<<<C, FIN_THREADS, 0, s>>>(partials, nb, C, out);
    FEGB_LAUNCH_CHECK("fold partials");
    return 0;
}

int find_multi_groups(const int32_t* off, int G, int R, int32_t* list, int* n_multi, cudaStream_t s) {
    *n_multi = 0;
    if (G <= 0) return 0;
    int* cnt = nullptr;
    FEGB_CUDA(cudaMallocAsync(&cnt, sizeof(int), s), "multi groups counter");
    FEGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), s), "multi groups reset");
    find_multi_kernel<<<(G + 255) / 256, 256, 0, s>>>(off, G, R, list, cnt);
    FEGB_LAUNCH_CHECK("find multi-chunk groups");
    FEGB_CUDA(cudaMemcpyAsync(n_multi, cnt, sizeof(int), cudaMemcpyDeviceToHost, s), "multi groups count");
    FEGB_CUDA(cudaFreeAsync(cnt, s), "multi groups free");
    FEGB_CUDA(cudaStreamSynchronize(s), "multi groups sync");
    return 0;
}

template <typename S>
int launch_group_sums(const int32_t* off, const double* head, const double* tail, int R, int C,
                      const int32_t* long_list, int n_long, const int32_t* multi_list, int n_multi, S* sums,
                      cudaStream_t s) {
    const long long nb = (long long)n_long + ((long long)n_multi + FIN_THREADS / 32 - 1) / (FIN_THREADS / 32);
    if (nb <= 0) return 0;
    group_sums_kernel<S><<<(unsigned)nb, FIN_THREADS, 0, s>>>(off, head, tail, R, C, long_list, n_long, multi_list,
                                                              n_multi, sums);
    FEGB_LAUNCH_CHECK("group sums across chunks");
    return 0;
}
template int launch_group_sums<float>(const int32_t*, const double*, const double*, int, int, const int32_t*, int,
                                      const int32_t*, int, float*, cudaStream_t);
template int launch_group_sums<double>(const int32_t*, const double*, const double*, int, int, const int32_t*, int,
                                       const int32_t*, int, double*, cudaStream_t);

int find_long_groups(const int32_t* off, int G, int R, int32_t* list, int* n_long, cudaStream_t s) {
    *n_long = 0;
    if (G <= 0) return 0;
    int* cnt = nullptr;
    FEGB_CUDA(cudaMallocAsync(&cnt, sizeof(int), s), "long groups counter");
    FEGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int), s), "long groups reset");
    find_long_kernel<<<(G + 255) / 256, 256, 0, s>>>(off, G, R, list, cnt);
    FEGB_LAUNCH_CHECK("find long groups");
    FEGB_CUDA(cudaMemcpyAsync(n_long, cnt, sizeof(int), cudaMemcpyDeviceToHost, s), "long groups count");
    FEGB_CUDA(cudaFreeAsync(cnt, s), "long groups free");
    FEGB_CUDA(cudaStreamSynchronize(s), "long groups sync");
    return 0;
}

template <typename S>
int long_sums_t(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                int n_long, S* sums, cudaStream_t s) {
    if (n_long <= 0) return 0;
    long_sums_kernel<S><<<n_long, FIN_THREADS, 0, s>>>(off, head, tail, R, C, list, sums);
    FEGB_LAUNCH_CHECK("long group sums");
    return 0;
}

int launch_long_sums(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                     int n_long, double* sums, cudaStream_t s) {
    return long_sums_t<double>(off, head, tail, R, C, list, n_long, sums, s);
}

int launch_long_sums(const int32_t* off, const double* head, const double* tail, int R, int C, const int32_t* list,
                     int n_long, float* sums, cudaStream_t s) {
    return long_sums_t<float>(off, head, tail, R, C, list, n_long, sums, s);
}

int launch_fold_smallg(const double* partials, int nblocks, int G, int C, double* sums, cudaStream_t s) {
    long long GC = (long long)G * C;
    if (GC <= 0) return 0;
    fold_smallg_kernel<<<(unsigned)((GC * 32 + 255) / 256), 256, 0, s>>>(partials, nblocks, GC, sums);
    FEGB_LAUNCH_CHECK("fold small-G partials");
    return 0;
}

int launch_inv_counts(const int32_t* counts, long long G, double* inv_counts, cudaStream_t s) {
    if (G <= 0) return 0;
    inv_counts_kernel<<<(unsigned)((G + 255) / 256), 256, 0, s>>>(counts, G, inv_counts);
    FEGB_LAUNCH_CHECK("inverse counts");
    return 0;
}

template <typename T>
int launch_cg_update(long long Gt, int C, const T* inv_counts, const double* rz, const double* pq, const T* p,
                     int pld, const T* q, T* x, T* r, T* z, double* rz_partials, double* zmax_partials,
                     unsigned long long* zmax, cudaStream_t s) {
    long long total = Gt * C;
    if (total <= 0) return 0;
    const int nb = cg_partial_blocks(Gt, C);
    if (C <= 256)
        cg_update_rows_kernel<T><<<nb, 256, 0, s>>>(Gt, C, inv_counts, rz, pq, p, pld, q, x, r, z, rz_partials,
                                                    zmax_partials);
    else
        cg_update_kernel<T><<<nb, FIN_THREADS, 0, s>>>(Gt, C, inv_counts, rz, pq, p, pld, q, x, r, z, rz_partials,
                                                       zmax_partials);
    FEGB_LAUNCH_CHECK("cg update");
    fold_max_kernel<<<1, FIN_THREADS, 0, s>>>(zmax_partials, nb, zmax);
    FEGB_LAUNCH_CHECK("cg max fold");
    return 0;
}

template <typename T>
int launch_cg_direction(long long Gt, int C, double* rz_old, const double* rz_new, const T* z, T* p, int pld,
                        cudaStream_t s, const int* skip) {
    long long total = Gt * C;
    if (total > 0) {
        cg_direction_kernel<T><<<grid_stride_blocks(total, 256), 256, 0, s>>>(Gt, C, rz_old, rz_new, z, p, pld,
                                                                             skip);
        FEGB_LAUNCH_CHECK("cg direction");
    }
    copy_scalars_kernel<<<1, ((C + 31) / 32) * 32, 0, s>>>(rz_new, rz_old, C, skip);
    FEGB_LAUNCH_CHECK("cg scalars");
    return 0;
}

template <typename T>
int launch_cg_init(long long Gt, int C, const int32_t* counts, const double* mu, T* r, T* z, T* p, int pld, T* x,
                   double* rz_partials, double* zmax_partials, unsigned long long* zmax, cudaStream_t s) {
    long long total = Gt * C;
    if (total <= 0) return 0;
    const int nb = cg_partial_blocks(Gt, C);
    if (C <= 256)
        cg_init_rows_kernel<T><<<nb, 256, 0, s>>>(Gt, C, counts, mu, r, z, p, pld, x, rz_partials, zmax_partials);
    else
        cg_init_kernel<T><<<nb, FIN_THREADS, 0, s>>>(Gt, C, counts, mu, r, z, p, pld, x, rz_partials,
                                                     zmax_partials);
    FEGB_LAUNCH_CHECK("cg init");
    fold_max_kernel<<<1, FIN_THREADS, 0, s>>>(zmax_partials, nb, zmax);
    FEGB_LAUNCH_CHECK("cg max fold");
    return 0;
}

template <typename T>
int launch_cg_init_rhs(long long Gt, int C, const int32_t* counts, const double* mu, const T* qb, const T* inv, T* r,
                       T* z, T* p, int pld, T* x, double* rz_partials, double* zmax_partials, unsigned long long* zmax,
                       cudaStream_t s) {
    if (Gt * C <= 0) return 0;
    if (C > 256) return set_error("cg: %d columns exceed the right-hand-side initialisation", C);
    const int nb = cg_partial_blocks(Gt, C);
    cg_init_rhs_rows_kernel<T><<<nb, 256, 0, s>>>(Gt, C, counts, mu, qb, inv, r, z, p, pld, x, rz_partials,
                                                  zmax_partials);
    FEGB_LAUNCH_CHECK("cg init (rhs)");
    fold_max_kernel<<<1, FIN_THREADS, 0, s>>>(zmax_partials, nb, zmax);
    FEGB_LAUNCH_CHECK("cg max fold");
    return 0;
}
template int launch_cg_init_rhs<float>(long long, int, const int32_t*, const double*, const float*, const float*,
                                       float*, float*, float*, int, float*, double*, double*, unsigned long long*,
                                       cudaStream_t);
template int launch_cg_init_rhs<double>(long long, int, const int32_t*, const double*, const double*, const double*,
                                        double*, double*, double*, int, double*, double*, double*,
                                        unsigned long long*, cudaStream_t);

template int launch_cg_q<double>(const FinalizeParams&, int, const double*, int, double*, double*, cudaStream_t,
                                 const double*);
template int launch_cg_q<float>(const FinalizeParams&, int, const float*, int, float*, double*, cudaStream_t,
                                const float*);

// ---- dense count matrices of small-G dimensions ----

__global__ void count_pairs_kernel(const int32_t* __restrict__ ge, const int32_t* __restrict__ gs, long long n,
                                   int Gs, uint32_t* __restrict__ N) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) atomicAdd(N + (long long)ge[i] * Gs + gs[i], 1u);  // integer: order-free
}

int launch_count_pairs(const int32_t* gid_e, const int32_t* gid_s, long long n, int Gs, uint32_t* N, cudaStream_t s) {
    if (n <= 0) return 0;
    count_pairs_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(gid_e, gid_s, n, Gs, N);
    FEGB_LAUNCH_CHECK("count pairs");
    return 0;
}

__global__ void count_max_kernel(const uint32_t* __restrict__ N, long long cnt, unsigned* __restrict__ mx) {
    unsigned m = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x)
        m = max(m, N[i]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(mx, m);  // integer max: order-free
}

__global__ void narrow_counts_kernel(const uint32_t* __restrict__ N, long long cnt, uint8_t* __restrict__ out) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x)
        out[i] = (uint8_t)N[i];
}

int launch_count_max(const uint32_t* N, long long cnt, unsigned* mx, cudaStream_t s) {
    FEGB_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned), s), "count max reset");
    if (cnt <= 0) return 0;
    count_max_kernel<<<grid_stride_blocks(cnt, 256), 256, 0, s>>>(N, cnt, mx);
    FEGB_LAUNCH_CHECK("count max");
    return 0;
}

int launch_narrow_counts(const uint32_t* N, long long cnt, uint8_t* out, cudaStream_t s) {
    if (cnt <= 0) return 0;
    narrow_counts_kernel<<<grid_stride_blocks(cnt, 256), 256, 0, s>>>(N, cnt, out);
    FEGB_LAUNCH_CHECK("narrow counts");
    return 0;
}

namespace {

constexpr int DENSE_WARPS = 8;

// 16-byte vector of T (4 floats or 2 doubles)
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
    using type = float4;
    static constexpr int n = 4;
};
template <>
struct Vec16<double> {
    using type = double2;
    static constexpr int n = 2;
};

// acc[c] += m * row[c] for c < NC (NC a multiple of 4; row 16-byte aligned)
template <typename T, int NC>
__device__ __forceinline__ void fma_row(T m, const T* __restrict__ row, T* acc) {
    using V = typename Vec16<T>::type;
    constexpr int W = Vec16<T>::n;
#pragma unroll
    for (int c = 0; c < NC; c += W) {
        const V v = *reinterpret_cast<const V*>(row + c);
        if constexpr (W == 4) {
            acc[c] = fmaf(m, v.x, acc[c]);
            acc[c + 1] = fmaf(m, v.y, acc[c + 1]);
            acc[c + 2] = fmaf(m, v.z, acc[c + 2]);
            acc[c + 3] = fmaf(m, v.w, acc[c + 3]);
        } else {
            acc[c] = fma(m, v.x, acc[c]);
            acc[c + 1] = fma(m, v.y, acc[c + 1]);
        }
    }
}

// 16-byte global -> shared copy that completes asynchronously (L2 only)
__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Bytes of the first part of a tile slot in the Schur form: the primary's
// sums rows (DENSE_TILE x C, storage type), rounded to 16; its group counts follow.
template <typename T>
__host__ __device__ inline size_t dense_sums_bytes(int C) {
    return ((sizeof(T) * (size_t)DENSE_TILE * C + 15) / 16) * 16;
}
// Shared-memory bytes of one tile slot's row part: pe rows (ld values) or, in
// the Schur form, the primary's sums rows and group counts.
template <typename T>
__host__ __device__ inline size_t dense_slot_bytes(int ld, int C) {
    const size_t p = sizeof(T) * (size_t)DENSE_TILE * ld;
    const size_t u = dense_sums_bytes<T>(C) + sizeof(int32_t) * DENSE_TILE;
    return p > u ? p : u;
}

// bytes [0, whole 16-byte pieces of n) of gsrc -> sdst asynchronously (both 16-byte aligned)
__device__ __forceinline__ void stage_async(void* sdst, const void* gsrc, long long bytes) {
    const char* g = reinterpret_cast<const char*>(gsrc);
    char* d = reinterpret_cast<char*>(sdst);
    for (long long o = (long long)threadIdx.x * 16; o + 16 <= bytes; o += 256 * 16) cp_async16(d + o, g + o);
}
// the elements of [0, n) not covered by whole 16-byte pieces, with plain loads
template <typename E>
__device__ __forceinline__ void stage_tail(E* sdst, const E* __restrict__ gsrc, long long n) {
    const long long whole = (n * (long long)sizeof(E)) / 16 * 16 / (long long)sizeof(E);
    for (long long i = whole + threadIdx.x; i < n; i += 256) sdst[i] = gsrc[i];
}

// Stage the count rows and the row part of groups [tile, tile + nt) into one
// tile slot: the pe rows (pe set) or, in the Schur form (usums set), the
// primary's sums rows and group counts. Whole 16-byte pieces go
// asynchronously; the ragged tails (the last tile of a range) follow with
// plain loads through dense_tail.
template <typename T, typename CT>
__device__ __forceinline__ void dense_issue(const CT* __restrict__ M, const T* __restrict__ pe, int Gs, int ld,
                                            long long tile, int nt, CT* sM, T* sP, const T* usums = nullptr,
                                            const int32_t* ucnt = nullptr, int C = 0) {
    stage_async(sM, M + tile * Gs, (long long)nt * Gs * sizeof(CT));
    if (usums) {
        // asynchronous only from 16-byte aligned rows; dense_tail loads the rest
        if ((reinterpret_cast<uintptr_t>(usums + tile * C) & 15u) == 0)
            stage_async(sP, usums + tile * C, (long long)nt * C * sizeof(T));
        if ((reinterpret_cast<uintptr_t>(ucnt + tile) & 15u) == 0)
            stage_async(reinterpret_cast<char*>(sP) + dense_sums_bytes<T>(C), ucnt + tile, (long long)nt * 4);
        return;
    }
    if (!pe) return;
    const long long pbytes = (long long)nt * ld * sizeof(T);
    const char* gp = reinterpret_cast<const char*>(pe + tile * ld);
    for (long long o = (long long)threadIdx.x * 16; o < pbytes; o += 256 * 16)
        cp_async16(reinterpret_cast<char*>(sP) + o, gp + o);
}

template <typename T, typename CT>
__device__ __forceinline__ void dense_tail(const CT* __restrict__ M, int Gs, long long tile, int nt, CT* sM,
                                           T* sP = nullptr, const T* usums = nullptr, const int32_t* ucnt = nullptr,
                                           int C = 0) {
    stage_tail(sM, M + tile * Gs, (long long)nt * Gs);
    if (usums) {
        const T* us = usums + tile * C;
        if ((reinterpret_cast<uintptr_t>(us) & 15u) == 0)
            stage_tail(sP, us, (long long)nt * C);
        else
            for (long long i = threadIdx.x; i < (long long)nt * C; i += 256) sP[i] = us[i];
        int32_t* sc = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(sP) + dense_sums_bytes<T>(C));
        const int32_t* uc = ucnt + tile;
        if ((reinterpret_cast<uintptr_t>(uc) & 15u) == 0)
            stage_tail(sc, uc, (long long)nt);
        else
            for (int i = threadIdx.x; i < nt; i += 256) sc[i] = uc[i];
    }
}

// Dense pair product of a small dimension s (Gs groups) and a dimension e
// (Ge groups) through their count matrix M (Ge x Gs, row g: the rows of each
// group of s within group g of e):
//   partials[block][t][c] = sum over the block's groups g of M[g][t] pe[g][c]
//   extra[g][c] (+)= sum_t M[g][t] ps[t][c]                 (extra != null)
// Block b covers groups [b * per, (b + 1) * per) (per a multiple of
// DENSE_TILE) in tiles of DENSE_TILE groups, double-buffered in shared memory
// by asynchronous copies (the next tile loads while this one is used). Small
// side: warp w takes the tile's groups g = w mod 8, lane = group t of s (and
// t + 32 when TWO), all columns in registers, pe rows read as 16-byte
// broadcasts; the 8 warps' sums are folded in warp order into FP64 at the
// end. Extra side: thread = (group of e, quad of 4 columns).
template <typename T, typename CT, int CQ, bool TWO>
__global__ void __launch_bounds__(256) dense_pair_kernel(const CT* __restrict__ M, long long Ge, int Gs,
                                                         const T* __restrict__ pe, const T* __restrict__ ps, int ld,
                                                         int C, long long per, double* __restrict__ partials,
                                                         T* __restrict__ extra, int accumulate, DenseSchur<T> sch) {
    extern __shared__ __align__(16) unsigned char dense_smem[];
    // layout: sS (Gs x CQ) | sU (DENSE_TILE x CQ) |
    //         2 x [sP (DENSE_TILE x ld) | sM (DENSE_TILE x Gs, padded to 16 bytes)]
    T* sS = reinterpret_cast<T*>(dense_smem);
    const size_t s_bytes = sizeof(T) * (size_t)DENSE_SMALL_MAX_G * CQ;
    T* sU = reinterpret_cast<T*>(dense_smem + s_bytes);
    const size_t u_bytes = sizeof(T) * (size_t)DENSE_TILE * CQ;
    const size_t p_bytes = dense_slot_bytes<T>(ld, C);
    const size_t m_bytes = ((sizeof(CT) * (size_t)DENSE_TILE * Gs + 15) / 16) * 16;
    unsigned char* const buf0 = dense_smem + s_bytes + u_bytes;
    unsigned char* const buf1 = buf0 + p_bytes + m_bytes;
    double* red = reinterpret_cast<double*>(dense_smem);  // Gs x C (after the tiles)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (extra || sch.sums)
        for (int i = threadIdx.x; i < Gs * CQ; i += 256) {
            const int t = i / CQ, c = i - t * CQ;
            sS[i] = c < C ? ps[(long long)t * ld + c] : T(0);
        }
    T acc0[CQ], acc1[TWO ? CQ : 1];
#pragma unroll
    for (int c = 0; c < CQ; ++c) acc0[c] = T(0);
#pragma unroll
    for (int c = 0; c < (TWO ? CQ : 1); ++c) acc1[c] = T(0);
    const long long g0 = (long long)blockIdx.x * per;
    const long long g1 = min(Ge, g0 + per);
    const bool schur = sch.sums != nullptr;       // the small side's pe rows are computed, not read
    const bool small_side = partials != nullptr;  // else only the extra side (pe is not read)
    if (g0 < g1)
        dense_issue<T, CT>(M, small_side && !schur ? pe : nullptr, Gs, ld, g0, (int)min((long long)DENSE_TILE, g1 - g0),
                           reinterpret_cast<CT*>(buf0 + p_bytes), reinterpret_cast<T*>(buf0), sch.sums, sch.counts, C);
    cp_async_commit();
    bool odd = false;
    for (long long tile = g0; tile < g1; tile += DENSE_TILE, odd = !odd) {
        unsigned char* const cur = odd ? buf1 : buf0;
        unsigned char* const nxt = odd ? buf0 : buf1;
        const int nt = (int)min((long long)DENSE_TILE, g1 - tile);
        const long long next = tile + DENSE_TILE;
        if (next < g1)
            dense_issue<T, CT>(M, small_side && !schur ? pe : nullptr, Gs, ld, next, (int)min((long long)DENSE_TILE, g1 - next),
                               reinterpret_cast<CT*>(nxt + p_bytes), reinterpret_cast<T*>(nxt), sch.sums, sch.counts, C);
        cp_async_commit();
        cp_async_wait_prev();  // this tile's copies are done (the next tile's may be in flight)
        CT* const m = reinterpret_cast<CT*>(cur + p_bytes);
        const T* const pt = reinterpret_cast<const T*>(cur);
        dense_tail<T, CT>(M, Gs, tile, nt, m, reinterpret_cast<T*>(cur), sch.sums, sch.counts, C);
        __syncthreads();
        const int32_t* const tcnt = reinterpret_cast<const int32_t*>(cur + dense_sums_bytes<T>(C));
        if (schur) {
            // u = (sums - sum_t M[g][t] ps[t]) / counts for the tile's groups: written to the
            // primary's table and kept in shared memory as this tile's pe rows
            constexpr int QN = CQ / 4;
            for (int i = threadIdx.x; i < nt * QN; i += 256) {
                const int gl = i / QN, c0 = (i - gl * QN) * 4;
                const long long g = tile + gl;
                T a[4] = {T(0), T(0), T(0), T(0)};
                const CT* mr = m + gl * Gs;
                for (int t = 0; t < Gs; ++t) fma_row<T, 4>((T)mr[t], sS + t * CQ + c0, a);
                const int n = tcnt[gl];
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    const int col = c0 + c;
                    T u = T(0);
                    if (col < C && n > 0) u = (pt[gl * C + col] - a[c]) / (T)n;
                    sU[gl * CQ + col] = u;
                    if (col < C) sch.table[g * ld + col] = u;
                }
            }
            __syncthreads();
        }
        for (int gl = warp; small_side && gl < nt; gl += DENSE_WARPS) {
            const T* prow = schur ? sU + gl * CQ : pt + gl * ld;
            if (lane < Gs) fma_row<T, CQ>((T)m[gl * Gs + lane], prow, acc0);
            if constexpr (TWO)
                if (lane + 32 < Gs) fma_row<T, CQ>((T)m[gl * Gs + lane + 32], prow, acc1);
        }
        if (extra && !schur) {
            constexpr int QN = CQ / 4;
            for (int i = threadIdx.x; i < nt * QN; i += 256) {
                const int gl = i / QN, c0 = (i - gl * QN) * 4;
                T a[4] = {T(0), T(0), T(0), T(0)};
                const CT* mr = m + gl * Gs;
                for (int t = 0; t < Gs; ++t) fma_row<T, 4>((T)mr[t], sS + t * CQ + c0, a);
                T* o = extra + (tile + gl) * C + c0;
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (c0 + c < C) o[c] = accumulate ? o[c] + a[c] : a[c];
            }
        }
        __syncthreads();  // this buffer is refilled two tiles on
    }
    // fold the warps' small-side sums in warp order (FP64); red overlays sS
    __syncthreads();
    for (int w = 0; w < DENSE_WARPS; ++w) {
        if (warp == w) {
#pragma unroll
            for (int c = 0; c < CQ; ++c) {
                if (c >= C) break;
                if (lane < Gs) red[lane * C + c] = (w ? red[lane * C + c] : 0.0) + (double)acc0[c];
                if constexpr (TWO)
                    if (lane + 32 < Gs) red[(lane + 32) * C + c] = (w ? red[(lane + 32) * C + c] : 0.0) + (double)acc1[c];
            }
        }
        __syncthreads();
    }
    if (small_side)
        for (int i = threadIdx.x; i < Gs * C; i += 256) partials[(long long)blockIdx.x * Gs * C + i] = red[i];
}

template <typename T, typename CT, int CQ, bool TWO>
int dense_pair_cq(const CT* M, long long Ge, int Gs, const T* pe, const T* ps, int ld, int C, double* partials,
                  T* extra, int accumulate, const DenseSchur<T>& sch, cudaStream_t s) {
    static const cudaError_t attr = cudaFuncSetAttribute(dense_pair_kernel<T, CT, CQ, TWO>,
                                                         cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024);
    if (attr != cudaSuccess) return set_cuda_error(attr, "dense pair attr");
    const int nb = dense_chunks(Ge);
    long long per = (Ge + nb - 1) / nb;
    per = (per + DENSE_TILE - 1) / DENSE_TILE * DENSE_TILE;  // tiles (and their copies) start on 16 bytes
    const size_t p_bytes = dense_slot_bytes<T>(ld, C);
    const size_t m_bytes = ((sizeof(CT) * (size_t)DENSE_TILE * Gs + 15) / 16) * 16;
    const size_t smem = std::max(sizeof(T) * (size_t)(DENSE_SMALL_MAX_G + DENSE_TILE) * CQ + 2 * (p_bytes + m_bytes),
                                 sizeof(double) * (size_t)Gs * C);
    dense_pair_kernel<T, CT, CQ, TWO><<<nb, 256, smem, s>>>(M, Ge, Gs, pe, ps, ld, C, per, partials, extra,
                                                            accumulate, sch);
    FEGB_LAUNCH_CHECK("dense small-G pair product");
    return 0;
}

template <typename T, typename CT, int CQ>
int dense_pair_two(const CT* M, long long Ge, int Gs, const T* pe, const T* ps, int ld, int C, double* partials,
                   T* extra, int accumulate, const DenseSchur<T>& sch, cudaStream_t s) {
    if (Gs > 32) return dense_pair_cq<T, CT, CQ, true>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    return dense_pair_cq<T, CT, CQ, false>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
}

}  // namespace

namespace {
thread_local int t_dense_mode = -1;  // -1: the default form; 0: the FP32 CUDA-core form; 1: the tensor-core form
}  // namespace

bool dense_use_mma() {
    if (t_dense_mode >= 0) return t_dense_mode > 0;
    const int knob = tuning(TUNE_DENSE_FORM);
    if (knob >= 0) return knob > 0;
    static const bool env = [] {  // FEGB_DENSE_TENSOR=0 selects the FP32 CUDA-core form by default
        const char* v = std::getenv("FEGB_DENSE_TENSOR");
        return !(v && v[0] == '0');
    }();
    return env;
}
void dense_force_mode(int mode) { t_dense_mode = mode; }

template <typename T, typename CT>
int launch_dense_pair(const CT* M, long long Ge, int Gs, const T* pe, const T* ps, int ld, int C, double* partials,
                      T* extra, int accumulate, cudaStream_t s, const DenseSchur<T>& sch) {
    if (Ge <= 0 || Gs <= 0 || C <= 0) return 0;
    if (Gs > DENSE_SMALL_MAX_G || C > 32) return set_error("dense small-G product: Gs=%d C=%d too large", Gs, C);
    // pe and ps rows are copied whole (ld values, 16-byte pieces) and read CQ wide
    if (ld % (16 / (int)sizeof(T)) != 0 || (reinterpret_cast<uintptr_t>(pe) & 15u) != 0 ||
        (!partials && !extra) || (reinterpret_cast<uintptr_t>(M) & 15u) != 0 ||
        (sch.sums && (extra || !partials || !sch.counts || !sch.table)))
        return set_error("dense small-G product: invalid arguments (ld %d)", ld);
    if constexpr (std::is_same<T, float>::value && std::is_same<CT, uint8_t>::value) {
        // tensor-core form (tcgen05, dense_umma.cu) where its shapes allow it
        if (dense_use_mma()) {
            bool launched = false;
            FEGB_TRY(launch_dense_pair_umma(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s, &launched));
            if (launched) return 0;
        }
    }
    if (C <= 4 && ld >= 4) return dense_pair_two<T, CT, 4>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    if (C <= 8 && ld >= 8) return dense_pair_two<T, CT, 8>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    if (C <= 12 && ld >= 12)
        return dense_pair_two<T, CT, 12>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    if (C <= 16 && ld >= 16)
        return dense_pair_two<T, CT, 16>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    if (C <= 24 && ld >= 24)
        return dense_pair_two<T, CT, 24>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    if (C <= 32 && ld >= 32)
        return dense_pair_two<T, CT, 32>(M, Ge, Gs, pe, ps, ld, C, partials, extra, accumulate, sch, s);
    return set_error("dense small-G product: row stride %d below the %d-column read", ld, C);
}
template int launch_dense_pair<float, uint8_t>(const uint8_t*, long long, int, const float*, const float*, int, int,
                                               double*, float*, int, cudaStream_t, const DenseSchur<float>&);
template int launch_dense_pair<float, uint32_t>(const uint32_t*, long long, int, const float*, const float*, int, int,
                                                double*, float*, int, cudaStream_t, const DenseSchur<float>&);
template int launch_dense_pair<double, uint8_t>(const uint8_t*, long long, int, const double*, const double*, int, int,
                                                double*, double*, int, cudaStream_t, const DenseSchur<double>&);
template int launch_dense_pair<double, uint32_t>(const uint32_t*, long long, int, const double*, const double*, int,
                                                 int, double*, double*, int, cudaStream_t, const DenseSchur<double>&);

// ---- Schur-complement CG helpers ----

// table[g * L + c] = (sums[g * C + c] - extra[g * C + c]) / counts[g] (0 for an
// empty group); extra may be null.
template <typename T>
__global__ void schur_u_kernel(const T* __restrict__ sums, const T* __restrict__ extra,
                               const int32_t* __restrict__ counts, long long G, int C, T* __restrict__ table, int L) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < G * C; i += st) {
        const long long g = i / C;
        const int c = (int)(i - g * C);
        const int n = counts[g];
        T v = sums[i];
        if (extra) v -= extra[i];
        table[g * L + c] = n > 0 ? v / (T)n : T(0);
    }
}

template <typename T>
int launch_schur_u(const T* sums, const T* extra, const int32_t* counts, long long G, int C, T* table, int L,
                   cudaStream_t s) {
    if (G <= 0) return 0;
    schur_u_kernel<T><<<grid_stride_blocks(G * C, 256), 256, 0, s>>>(sums, extra, counts, G, C, table, L);
    FEGB_LAUNCH_CHECK("schur u");
    return 0;
}
template int launch_schur_u<float>(const float*, const float*, const int32_t*, long long, int, float*, int,
                                   cudaStream_t);
template int launch_schur_u<double>(const double*, const double*, const int32_t*, long long, int, double*, int,
                                    cudaStream_t);

// table[g * L + c] = (T)(scale * src[g * C + c])
template <typename T>
__global__ void table_from_f64_kernel(const double* __restrict__ src, long long G, int C, double scale,
                                      T* __restrict__ table, int L) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < G * C; i += st) {
        const long long g = i / C;
        table[g * L + (i - g * C)] = (T)(scale * src[i]);
    }
}

// table[g * L + c] = src[g * C + c]
template <typename T>
__global__ void table_from_compact_kernel(const T* __restrict__ src, long long G, int C, T* __restrict__ table, int L) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < G * C; i += st) {
        const long long g = i / C;
        table[g * L + (i - g * C)] = src[i];
    }
}

// alpha[g * C + c] = mu[g * C + c] + table[g * L + c]
template <typename T>
__global__ void alpha_primary_kernel(const double* __restrict__ mu, const T* __restrict__ table, long long G, int C,
                                     int L, double* __restrict__ alpha) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < G * C; i += st) {
        const long long g = i / C;
        alpha[i] = mu[i] + (double)table[g * L + (i - g * C)];
    }
}

template <typename T>
int launch_table_from_f64(const double* src, long long G, int C, double scale, T* table, int L, cudaStream_t s) {
    if (G <= 0) return 0;
    table_from_f64_kernel<T><<<grid_stride_blocks(G * C, 256), 256, 0, s>>>(src, G, C, scale, table, L);
    FEGB_LAUNCH_CHECK("table from fp64");
    return 0;
}
template <typename T>
int launch_table_from_compact(const T* src, long long G, int C, T* table, int L, cudaStream_t s) {
    if (G <= 0) return 0;
    table_from_compact_kernel<T><<<grid_stride_blocks(G * C, 256), 256, 0, s>>>(src, G, C, table, L);
    FEGB_LAUNCH_CHECK("table from compact");
    return 0;
}
template <typename T>
int launch_alpha_primary(const double* mu, const T* table, long long G, int C, int L, double* alpha, cudaStream_t s) {
    if (G <= 0) return 0;
    alpha_primary_kernel<T><<<grid_stride_blocks(G * C, 256), 256, 0, s>>>(mu, table, G, C, L, alpha);
    FEGB_LAUNCH_CHECK("primary increment");
    return 0;
}
template int launch_table_from_f64<float>(const double*, long long, int, double, float*, int, cudaStream_t);
template int launch_table_from_f64<double>(const double*, long long, int, double, double*, int, cudaStream_t);
template int launch_table_from_compact<float>(const float*, long long, int, float*, int, cudaStream_t);
template int launch_table_from_compact<double>(const double*, long long, int, double*, int, cudaStream_t);
template int launch_alpha_primary<float>(const double*, const float*, long long, int, int, double*, cudaStream_t);
template int launch_alpha_primary<double>(const double*, const double*, long long, int, int, double*, cudaStream_t);

// ---- diagonal of the Schur complement (the CG's Jacobi preconditioner) ----

// S_gg = n_g - sum_w n_wg^2 / n_w is accumulated as the sum of the
// nonnegative terms n_wg (n_w - n_wg) / n_w (the weights n_wg of a group add up
// to n_g), each term in FP32 and rounded to a fixed-point integer with 20
// fraction bits: integer sums are exact and independent of the order, so the
// 64-bit atomics leave the result deterministic, no term cancels another, and a
// group whose every primary group lies inside it sums to exactly 0. A nonzero
// term is at least 1/2 (n_wg >= 1, n_w - n_wg >= 1), so 2^-20 is far below the
// resolution a Jacobi preconditioner needs. Nothing here runs on the FP64 pipe.
__device__ __forceinline__ unsigned long long schur_term_fixed(float w, int nw) {
    const int wi = (int)w;
    if (nw <= 0 || wi >= nw) return 0ull;
    const float t = w * (float)(nw - wi) / (float)nw;
    return __float2ull_rn(t * 1048576.0f);
}

// acc[gseq[j]] += term(w[j], n_P[pid[j]]) over the positions of a stream in
// group order; each thread takes SCHUR_RUN consecutive positions and issues one
// atomic per group run it sees.
constexpr int SCHUR_RUN = 16;
__global__ void schur_diag_stream_kernel(const int32_t* __restrict__ gseq, long long m, const float* __restrict__ w,
                                         const int32_t* __restrict__ pid, const int32_t* __restrict__ nP,
                                         unsigned long long* __restrict__ acc) {
    const long long j0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * SCHUR_RUN;
    if (j0 >= m) return;
    const long long j1 = min(m, j0 + SCHUR_RUN);
    int g = gseq[j0];
    unsigned long long a = 0;
    for (long long j = j0; j < j1; ++j) {
        const int gj = gseq[j];
        if (gj != g) {
            if (a) atomicAdd(acc + g, a);
            g = gj;
            a = 0;
        }
        a += schur_term_fixed(w ? w[j] : 1.0f, nP[pid[j]]);
    }
    if (a) atomicAdd(acc + g, a);
}

// Pair form: the rows sorted by (group of the dimension, primary group) give
// the pairs as segments off[p] .. off[p+1] of perm; acc[group] += term(segment
// length, n_P[primary group]), SCHUR_RUN consecutive pairs per thread.
__global__ void schur_diag_pairs_kernel(const int32_t* __restrict__ perm, const int32_t* __restrict__ off,
                                        long long npairs, const int32_t* __restrict__ gid_e,
                                        const int32_t* __restrict__ gid_p, const int32_t* __restrict__ nP,
                                        unsigned long long* __restrict__ acc) {
    const long long p0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) * SCHUR_RUN;
    if (p0 >= npairs) return;
    const long long p1 = min(npairs, p0 + SCHUR_RUN);
    int g = gid_e[perm[off[p0]]];
    unsigned long long a = 0;
    for (long long p = p0; p < p1; ++p) {
        const int s = off[p];
        const int row = perm[s];
        const int gp = gid_e[row];
        if (gp != g) {
            if (a) atomicAdd(acc + g, a);
            g = gp;
            a = 0;
        }
        a += schur_term_fixed((float)(off[p + 1] - s), nP[gid_p[row]]);
    }
    if (a) atomicAdd(acc + g, a);
}

// acc[t] += term(N[g][t], n[g]) over the Ge x Gs count matrix: thread i of the
// first S = (threads / Gs) * Gs takes elements i, i + S, ... (one column each),
// folded per block in shared memory, one global atomic per column per block.
template <typename CT>
__global__ void schur_diag_dense_kernel(const CT* __restrict__ N, long long Ge, int Gs, const int32_t* __restrict__ n,
                                        unsigned long long* __restrict__ acc) {
    __shared__ unsigned long long col[DENSE_SMALL_MAX_G];
    for (int t = threadIdx.x; t < Gs; t += blockDim.x) col[t] = 0ull;
    __syncthreads();
    const long long T = (long long)gridDim.x * blockDim.x;
    const long long S = T - T % Gs;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < S) {
        const int t = (int)(i % Gs);
        const long long gstep = S / Gs;
        unsigned long long a = 0;
        for (long long g = i / Gs; g < Ge; g += gstep) {
            const unsigned mv = (unsigned)N[g * Gs + t];
            if (mv) a += schur_term_fixed((float)mv, n[g]);
        }
        if (a) atomicAdd(col + t, a);
    }
    __syncthreads();
    for (int t = threadIdx.x; t < Gs; t += blockDim.x)
        if (col[t]) atomicAdd(acc + t, col[t]);
}

// inv[g] = 1 / S_gg, or 0 when S_gg <= 1e-9 counts[g] (no identifying variation)
template <typename T>
__global__ void inv_diag_kernel(const unsigned long long* __restrict__ acc, const int32_t* __restrict__ counts,
                                long long G, T* __restrict__ inv) {
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= G) return;
    const float d = (float)acc[g] * (1.0f / 1048576.0f);
    inv[g] = (counts[g] > 0 && d > 1e-9f * (float)counts[g]) ? (T)(1.0f / d) : T(0);
}

int launch_schur_diag_stream(const int32_t* gseq, long long m, const float* w, const int32_t* pid, const int32_t* nP,
                             unsigned long long* acc, cudaStream_t s) {
    if (m <= 0) return 0;
    const long long threads = (m + SCHUR_RUN - 1) / SCHUR_RUN;
    schur_diag_stream_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(gseq, m, w, pid, nP, acc);
    FEGB_LAUNCH_CHECK("schur diagonal (stream)");
    return 0;
}

int launch_schur_diag_pairs(const int32_t* perm, const int32_t* off, long long npairs, const int32_t* gid_e,
                            const int32_t* gid_p, const int32_t* nP, unsigned long long* acc, cudaStream_t s) {
    if (npairs <= 0) return 0;
    const long long threads = (npairs + SCHUR_RUN - 1) / SCHUR_RUN;
    schur_diag_pairs_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(perm, off, npairs, gid_e, gid_p, nP,
                                                                             acc);
    FEGB_LAUNCH_CHECK("schur diagonal (pairs)");
    return 0;
}

template <typename CT>
int launch_schur_diag_dense(const CT* N, long long Ge, int Gs, const int32_t* n, unsigned long long* acc,
                            cudaStream_t s) {
    if (Ge <= 0 || Gs <= 0) return 0;
    if (Gs > DENSE_SMALL_MAX_G) return set_error("schur diagonal: %d columns above %d", Gs, DENSE_SMALL_MAX_G);
    const long long elems = Ge * Gs;
    const long long blocks = std::min<long long>(DENSE_MAX_BLOCKS * 2, (elems + 255) / 256);
    schur_diag_dense_kernel<CT><<<(unsigned)std::max(1LL, blocks), 256, 0, s>>>(N, Ge, Gs, n, acc);
    FEGB_LAUNCH_CHECK("schur diagonal (dense)");
    return 0;
}
template int launch_schur_diag_dense<uint8_t>(const uint8_t*, long long, int, const int32_t*, unsigned long long*,
                                              cudaStream_t);
template int launch_schur_diag_dense<uint32_t>(const uint32_t*, long long, int, const int32_t*, unsigned long long*,
                                               cudaStream_t);

template <typename T>
int launch_inv_diag(const unsigned long long* acc, const int32_t* counts, long long G, T* inv, cudaStream_t s) {
    if (G <= 0) return 0;
    inv_diag_kernel<T><<<(unsigned)((G + 255) / 256), 256, 0, s>>>(acc, counts, G, inv);
    FEGB_LAUNCH_CHECK("inverse diagonal");
    return 0;
}
template int launch_inv_diag<float>(const unsigned long long*, const int32_t*, long long, float*, cudaStream_t);
template int launch_inv_diag<double>(const unsigned long long*, const int32_t*, long long, double*, cudaStream_t);

// One warp per (t, c): strided fold over the parts, fixed shuffle tree.
__global__ void fold_dense_kernel(const double* __restrict__ partials, int nparts, int TC, double* __restrict__ sums) {
    const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= TC) return;
    double acc = 0.0;
    for (int b = lane; b < nparts; b += 32) acc += partials[(long long)b * TC + w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) sums[w] = -acc;  // sums of -p, the sweep convention
}

int launch_fold_dense(const double* partials, int nparts, int Gs, int C, double* sums, cudaStream_t s) {
    const int TC = Gs * C;
    if (TC <= 0) return 0;
    fold_dense_kernel<<<(unsigned)((TC * 32 + 255) / 256), 256, 0, s>>>(partials, nparts, TC, sums);
    FEGB_LAUNCH_CHECK("small-G dense fold");
    return 0;
}

template int launch_cg_update<double>(long long, int, const double*, const double*, const double*, const double*, int,
                                      const double*, double*, double*, double*, double*, double*,
                                      unsigned long long*, cudaStream_t);
template int launch_cg_update<float>(long long, int, const float*, const double*, const double*, const float*, int,
                                     const float*, float*, float*, float*, double*, double*, unsigned long long*,
                                     cudaStream_t);

template <typename T>
int launch_to_f64(const T* src, int ld, double* dst, int C, long long G, cudaStream_t s) {
    const long long n = G * C;
    if (n <= 0) return 0;
    to_f64_kernel<T><<<grid_stride_blocks(n, 256), 256, 0, s>>>(src, ld, dst, C, n);
    FEGB_LAUNCH_CHECK("to fp64");
    return 0;
}
template int launch_to_f64<float>(const float*, int, double*, int, long long, cudaStream_t);
template int launch_to_f64<double>(const double*, int, double*, int, long long, cudaStream_t);

template <typename T>
int launch_inv_counts_t(const int32_t* counts, long long G, T* inv, cudaStream_t s) {
    if (G <= 0) return 0;
    inv_counts_t_kernel<T><<<(unsigned)((G + 255) / 256), 256, 0, s>>>(counts, G, inv);
    FEGB_LAUNCH_CHECK("inverse counts");
    return 0;
}
template int launch_inv_counts_t<float>(const int32_t*, long long, float*, cudaStream_t);
template int launch_inv_counts_t<double>(const int32_t*, long long, double*, cudaStream_t);
template int launch_cg_direction<double>(long long, int, double*, const double*, const double*, double*, int,
                                         cudaStream_t, const int*);
template int launch_cg_direction<float>(long long, int, double*, const double*, const float*, float*, int,
                                        cudaStream_t, const int*);
template int launch_cg_init<double>(long long, int, const int32_t*, const double*, double*, double*, double*, int,
                                    double*, double*, double*, unsigned long long*, cudaStream_t);
template int launch_cg_init<float>(long long, int, const int32_t*, const double*, float*, float*, float*, int, float*,
                                   double*, double*, unsigned long long*, cudaStream_t);


// ----------------------- row-per-lane CG operator sweep -----------------------
//
// The kernel is bound by L1 sector lookups: gathers of scattered table rows
// cost one lookup per 32-byte sector per lane, about one lookup per SM cycle.
// So ids are read 4 positions per 128-bit load (not kept in L1,
// marked evict-first in L2), and table rows, padded to 32-byte multiples, are
// read with 256-bit loads marked evict-last in L2 so the G-space tables stay
// cached across the positions that revisit them.

__device__ __forceinline__ unsigned long long l2_policy_evict_last() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ unsigned long long l2_policy_evict_first() {
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

// CG_IDV consecutive int32 ids from a 16-byte aligned address
constexpr int CG_IDV = 4;
__device__ __forceinline__ void ld_ids(const int32_t* ptr, int (&o)[CG_IDV], unsigned long long pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.b32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(o[0]), "=r"(o[1]), "=r"(o[2]), "=r"(o[3])
                 : "l"(ptr), "l"(pol));
}

__device__ __forceinline__ void ld_weights(const float* ptr, float (&o)[CG_IDV], unsigned long long pol) {
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
                 : "l"(ptr), "l"(pol));
}

// Pieces of a table row: NE consecutive elements at an address aligned to
// the piece's vector size (pieces start at 32-byte boundaries of the row).
template <int NE>
__device__ __forceinline__ void ld_piece(const float* ptr, float (&o)[NE], unsigned long long pol) {
    if constexpr (NE == 8) {
        asm("ld.global.nc.L2::cache_hint.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                     : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3]), "=f"(o[4]), "=f"(o[5]), "=f"(o[6]), "=f"(o[7])
                     : "l"(ptr), "l"(pol));
    } else if constexpr (NE == 4) {
        asm("ld.global.nc.L2::cache_hint.v4.f32 {%0,%1,%2,%3}, [%4], %5;"
                     : "=f"(o[0]), "=f"(o[1]), "=f"(o[2]), "=f"(o[3])
                     : "l"(ptr), "l"(pol));
    } else if constexpr (NE == 2) {
        asm("ld.global.nc.L2::cache_hint.v2.f32 {%0,%1}, [%2], %3;" : "=f"(o[0]), "=f"(o[1]) : "l"(ptr), "l"(pol));
    } else {
        static_assert(NE == 1, "piece width");
        asm("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(o[0]) : "l"(ptr), "l"(pol));
    }
}
template <int NE>
__device__ __forceinline__ void ld_piece(const double* ptr, double (&o)[NE], unsigned long long pol) {
    if constexpr (NE == 4) {
        asm("ld.global.nc.L2::cache_hint.v4.f64 {%0,%1,%2,%3}, [%4], %5;"
                     : "=d"(o[0]), "=d"(o[1]), "=d"(o[2]), "=d"(o[3])
                     : "l"(ptr), "l"(pol));
    } else if constexpr (NE == 2) {
        asm("ld.global.nc.L2::cache_hint.v2.f64 {%0,%1}, [%2], %3;" : "=d"(o[0]), "=d"(o[1]) : "l"(ptr), "l"(pol));
    } else {
        static_assert(NE == 1, "piece width");
        asm("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(o[0]) : "l"(ptr), "l"(pol));
    }
}

// smallest supported piece width holding w elements of a row (W = 256-bit width)
template <int W>
__host__ __device__ constexpr int piece_width(int w) {
    return w >= W ? W : (w > W / 2 ? W : (w > 2 ? (W >= 4 ? 4 : W) : (w == 2 ? 2 : 1)));
}

// v[0..TILE) += row[0..cw) of one source table (row already offset to column
// c0); FIRST: v = row instead (columns past cw keep their zeros)
template <typename T, int TILE, bool FIRST, int K = 0>
__device__ __forceinline__ void cg_add_row(const T* __restrict__ row, int cw, T (&v)[TILE], unsigned long long pol) {
    constexpr int W = 32 / (int)sizeof(T);  // elements per 256-bit load
    if constexpr (K * W < TILE) {
        if (K * W >= cw) return;
        constexpr int left = TILE - K * W;
        constexpr int NE = piece_width<W>(left < W ? left : W);
        T w[NE];
        ld_piece<NE>(row + W * K, w, pol);
#pragma unroll
        for (int m = 0; m < NE; ++m)
            if (W * K + m < TILE) {
                if (FIRST)
                    v[W * K + m] = w[m];
                else
                    v[W * K + m] += w[m];
            }
        cg_add_row<T, TILE, FIRST, K + 1>(row, cw, v, pol);
    }
}

#ifndef CG_ROWS_MINB
#define CG_ROWS_MINB 4
#endif

// Run state of one lane. The lane's first run (its head, which may continue
// the previous lane's last run) is parked in shared memory (head[i * 32], one
// column per 32 consecutive words, no bank conflicts) once a second run starts,
// so that only the current run is held in registers.
template <typename T, int TILE>
struct CGRun {
    T run[TILE];
    T* head;  // this lane's head slot: head[i * 32] = column i
    int firstg;
    int cur;
    bool single;
    bool started;
};

// Adds one position (group g, contribution a * v) to the lane's run state: a
// run that continues takes run += a * v as one fused multiply-add (a = -1
// without weights: exactly run - v).
template <typename T, int TILE>
__device__ __forceinline__ void cg_run_push(CGRun<T, TILE>& st, int g, T a, const T (&v)[TILE], T* __restrict__ sums,
                                            int SC, int c0, int cw) {
    if (!st.started) {
        st.started = true;
        st.firstg = st.cur = g;
#pragma unroll
        for (int i = 0; i < TILE; ++i) st.run[i] = a * v[i];
        return;
    }
    if (g != st.cur) {
        if (st.single) {
#pragma unroll
            for (int i = 0; i < TILE; ++i) st.head[i * 32] = st.run[i];
            st.single = false;
        } else {
            // a run that starts and ends inside this lane is complete
            T* dst = sums + (long long)st.cur * SC + c0;
#pragma unroll
            for (int i = 0; i < TILE; ++i)
                if (i < cw) dst[i] = st.run[i];
        }
        st.cur = g;
#pragma unroll
        for (int i = 0; i < TILE; ++i) st.run[i] = a * v[i];
    } else {
#pragma unroll
        for (int i = 0; i < TILE; ++i) st.run[i] = fma(a, v[i], st.run[i]);
    }
}

// TILE = columns per pass (compile-time register tile; all per-column arrays
// stay in registers because every loop over TILE is fully unrolled).
// NSRC = number of source dimensions when the vector id path is used
// (1..3); NSRC = 0 reads ids one position at a time for any n_src.
template <typename T, int CGR_TILE, int NSRC>
__global__ void __launch_bounds__(256, (sizeof(T) == 4 && CGR_TILE <= 12) ? CG_ROWS_MINB : 2)
    cg_rows_kernel(CGRowsParams<T> p, int ntiles) {
    const int lane = threadIdx.x & 31;
    const long long warp = ((long long)blockIdx.x * 256 + threadIdx.x) >> 5;
    const long long nchunks = (p.n + CG_CHUNK - 1) / CG_CHUNK;
    if (warp >= nchunks * ntiles) return;  // whole warp exits together
    const long long q = warp / ntiles;
    const int c0 = (int)(warp - q * ntiles) * CGR_TILE;
    const int C = p.C;
    const int LD = p.ld;
    const int cw = min(CGR_TILE, C - c0);
    const long long j0 = q * CG_CHUNK;
    const long long j1 = min(j0 + (long long)CG_CHUNK, p.n);
    const long long ls = j0 + (long long)lane * CG_LANE_POS;
    const long long le = min(ls + CG_LANE_POS, j1);
    const bool empty = ls >= le;
    const int32_t* __restrict__ gseq = p.gseq;
    const unsigned long long keep = l2_policy_evict_last();

    __shared__ T s_head[8][CGR_TILE * 32];  // one slot per lane of each of the block's 8 warps
    CGRun<T, CGR_TILE> st;
    st.head = &s_head[threadIdx.x >> 5][lane];
#pragma unroll
    for (int i = 0; i < CGR_TILE; ++i) st.run[i] = T(0);
    st.firstg = -1;
    st.cur = -1;
    st.single = true;
    st.started = false;

    if constexpr (NSRC > 0) {
        const unsigned long long stream = l2_policy_evict_first();
        const T* tabs[NSRC];
        const int32_t* sgid[NSRC];
#pragma unroll
        for (int e = 0; e < NSRC; ++e) {
            tabs[e] = p.src_tab[e] + c0;
            sgid[e] = p.src_gid[e];
        }
#pragma unroll 1
        for (int h = 0; h < CG_LANE_POS / CG_IDV; ++h) {
            const long long jb = ls + CG_IDV * h;
            if (jb + CG_IDV <= le) {
                int gq[CG_IDV];
                int sid[NSRC][CG_IDV];
                float wq[CG_IDV];
                ld_ids(gseq + jb, gq, stream);
#pragma unroll
                for (int e = 0; e < NSRC; ++e) ld_ids(sgid[e] + jb, sid[e], stream);
                if (p.weight) ld_weights(p.weight + jb, wq, stream);
#pragma unroll
                for (int m = 0; m < CG_IDV; ++m) {
                    T v[CGR_TILE];
#pragma unroll
                    for (int i = 0; i < CGR_TILE; ++i) v[i] = T(0);
                    cg_add_row<T, CGR_TILE, true>(tabs[0] + (long long)sid[0][m] * LD, cw, v, keep);
#pragma unroll
                    for (int e = 1; e < NSRC; ++e)
                        cg_add_row<T, CGR_TILE, false>(tabs[e] + (long long)sid[e][m] * LD, cw, v, keep);
                    cg_run_push(st, gq[m], p.weight ? -(T)wq[m] : T(-1), v, p.sums, C, c0, cw);
                }
            } else {
                // ragged end of the last chunk
                for (long long j = jb; j < le; ++j) {
                    T v[CGR_TILE];
#pragma unroll
                    for (int i = 0; i < CGR_TILE; ++i) v[i] = T(0);
#pragma unroll
                    for (int e = 0; e < NSRC; ++e)
                        cg_add_row<T, CGR_TILE, false>(tabs[e] + (long long)__ldg(sgid[e] + j) * LD, cw, v, keep);
                    cg_run_push(st, __ldg(gseq + j), p.weight ? -(T)__ldg(p.weight + j) : T(-1), v, p.sums, C, c0,
                                cw);
                }
            }
        }
    } else {
        for (long long j = ls; j < le; ++j) {
            T v[CGR_TILE];
#pragma unroll
            for (int i = 0; i < CGR_TILE; ++i) v[i] = T(0);
            for (int e = 0; e < p.n_src; ++e)
                cg_add_row<T, CGR_TILE, false>(p.src_tab[e] + (long long)__ldcs(p.src_gid[e] + j) * LD + c0, cw, v,
                                               keep);
            cg_run_push(st, __ldcs(gseq + j), p.weight ? -(T)__ldcs(p.weight + j) : T(-1), v, p.sums, C, c0, cw);
        }
    }
    const int firstg = st.firstg;
    const bool single = st.single;
    const int lastg = st.cur;
    // empty lanes (only in the last chunk) are transparent: they continue the
    // previous lane's run with a zero contribution
    const unsigned full = 0xffffffffu;
    const int lane_end = 31 - __clz(__ballot_sync(full, !empty));
    const int fill_g = __shfl_sync(full, lastg, lane_end);
    const int fg = empty ? fill_g : firstg;
    const int lg = empty ? fill_g : lastg;
    const int prev_lg = __shfl_up_sync(full, lg, 1);
    const bool cont = lane > 0 && (empty || fg == prev_lg);
    const bool sgl = empty || single;
    const unsigned next_cont_mask = __ballot_sync(full, cont);
    // lanes whose last run starts inside them (every lane except a single-run
    // lane that continues its left neighbour's run); lane 0 always qualifies
    const unsigned tail_start_mask = __ballot_sync(full, !(sgl && cont));
    const unsigned below = lane == 0 ? 0u : (tail_start_mask & ((1u << lane) - 1u));
    const int head_start_lane = cont ? (31 - __clz(below)) : lane;
    // a run reaching this lane from the left began at the chunk's first
    // position only if it began in lane 0 and lane 0 holds a single run
    const bool lane0_single = __shfl_sync(full, sgl ? 1 : 0, 0) != 0;
    const bool head_from_start = cont ? (head_start_lane == 0 && lane0_single) : (lane == 0);
    const bool before = j0 > 0 && gseq[j0 - 1] == gseq[j0];
    const bool after = j1 < p.n && gseq[j1] == gseq[j1 - 1];
    const bool tail_ends_here = !empty && (lane == lane_end || !((next_cont_mask >> (lane + 1)) & 1u));

    // Lane carries: out_l = b_l + (a_l ? out_{l-1} : 0), a_l = 1 when this lane is
    // one run continuing from the left. The flags are the same for every
    // column: the inclusive scan's per-level flags are computed once, and each
    // column then costs one shuffle and one conditional add per level, in the
    // storage type.
    bool ak[5];
    {
        bool acur = sgl && cont;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const int o = 1 << k;
            ak[k] = acur && lane >= o;
            const bool a_up = __shfl_up_sync(full, acur ? 1 : 0, o) != 0;
            if (lane >= o) acur = acur && a_up;
        }
    }
#pragma unroll
    for (int i = 0; i < CGR_TILE; ++i) {
        if (i >= cw) continue;  // uniform across the warp
        T b = empty ? T(0) : st.run[i];  // a single-run lane's head is its run
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const T b_up = __shfl_up_sync(full, b, 1 << k);
            if (ak[k]) b += b_up;
        }
        const T out = b;
        T in = __shfl_up_sync(full, out, 1);
        if (lane == 0) in = T(0);
        const long long col = c0 + i;
        if (!empty && !single) {
            // head run of a multi-run lane ends inside this lane
            const T val = (cont ? in : T(0)) + st.head[i * 32];
            if (head_from_start && before)
                p.head[q * C + col] = (double)val;
            else
                p.sums[(long long)fg * C + col] = val;
        }
        if (tail_ends_here) {
            const bool from_start = sgl && head_from_start;
            const bool at_end = lane == lane_end;
            if (from_start && before)
                p.head[q * C + col] = (double)out;
            else if (at_end && after)
                p.tail[q * C + col] = (double)out;
            else
                p.sums[(long long)lg * C + col] = out;
        }
    }
}

template <typename T, int TILE, int NSRC>
int launch_cg_rows_tile(const CGRowsParams<T>& p, cudaStream_t s) {
    const int ntiles = (p.C + TILE - 1) / TILE;
    const long long warps = ((p.n + CG_CHUNK - 1) / CG_CHUNK) * ntiles;
    const long long blocks = (warps * 32 + 255) / 256;
    cg_rows_kernel<T, TILE, NSRC><<<(unsigned)blocks, 256, 0, s>>>(p, ntiles);
    FEGB_LAUNCH_CHECK("cg operator sweep");
    return 0;
}

template <typename T, int TILE>
int launch_cg_rows_nsrc(const CGRowsParams<T>& p, cudaStream_t s) {
    // the vector id path needs 16-byte aligned id arrays
    bool aligned = (reinterpret_cast<uintptr_t>(p.gseq) & 15u) == 0 && (reinterpret_cast<uintptr_t>(p.weight) & 15u) == 0;
    for (int e = 0; e < p.n_src; ++e) aligned = aligned && (reinterpret_cast<uintptr_t>(p.src_gid[e]) & 15u) == 0;
    if (aligned) {
        if (p.n_src == 1) return launch_cg_rows_tile<T, TILE, 1>(p, s);
        if (p.n_src == 2) return launch_cg_rows_tile<T, TILE, 2>(p, s);
        if (p.n_src == 3) return launch_cg_rows_tile<T, TILE, 3>(p, s);
    }
    return launch_cg_rows_tile<T, TILE, 0>(p, s);
}

template <typename T>
int launch_cg_rows(const CGRowsParams<T>& p, cudaStream_t s) {
    if (p.n <= 0) return 0;
    // table rows are read in 32-byte pieces: the stride and the tables must allow it
    if (p.ld % (32 / (int)sizeof(T)) != 0) return set_error("cg operator: row stride %d is not a 32-byte multiple", p.ld);
    for (int e = 0; e < p.n_src; ++e)
        if ((reinterpret_cast<uintptr_t>(p.src_tab[e]) & 31u) != 0) return set_error("cg operator: unaligned table");
    const int cap = tuning(TUNE_CG_COLS_PER_PASS);  // columns per pass (0: all, up to 16)
    if (p.C <= 4 || cap == 4) return launch_cg_rows_nsrc<T, 4>(p, s);
    if (p.C <= 8 || cap == 8) return launch_cg_rows_nsrc<T, 8>(p, s);
    if (p.C == 9) return launch_cg_rows_nsrc<T, 9>(p, s);
    if (p.C <= 12) return launch_cg_rows_nsrc<T, 12>(p, s);
    return launch_cg_rows_nsrc<T, 16>(p, s);
}

constexpr int CGS_U = 4;  // positions per step of the short-group sweep

// Operator sweep of a stream whose groups are all short (every group at most
// CG_SHORT_MAX positions, on average at most CG_SHORT_MEAN): thread t takes
// column tile t / G of group t % G, so a warp covers 32 consecutive groups and
// their contiguous positions. The thread sums its group's positions in order
// (run = fma(a, v, run) from zero: the first step is the rounded product a * v,
// as in a lane of the chunked sweep) and writes the complete sum; empty groups
// get zeros. CGS_U positions are
// loaded ahead so that their row gathers are in flight together.
template <typename T, int TILE, int NSRC>
__global__ void __launch_bounds__(256) cg_short_kernel(CGRowsParams<T> p, const int32_t* __restrict__ off, int G,
                                                       int ntiles) {
    const long long t = (long long)blockIdx.x * 256 + threadIdx.x;
    if (t >= (long long)G * ntiles) return;
    const int tile = (int)(t / G);
    const int g = (int)(t - (long long)tile * G);
    const int c0 = tile * TILE;
    const int cw = min(TILE, p.C - c0);
    const int j0 = __ldg(off + g), j1 = __ldg(off + g + 1);
    const unsigned long long keep = l2_policy_evict_last();
    const T* tabs[NSRC];
#pragma unroll
    for (int e = 0; e < NSRC; ++e) tabs[e] = p.src_tab[e] + c0;
    T run[TILE];
#pragma unroll
    for (int i = 0; i < TILE; ++i) run[i] = T(0);
    // CGS_U positions a step, all their row gathers issued before the first
    // is consumed; positions past the group's end add zero
    for (int j = j0; j < j1; j += CGS_U) {
        T v[CGS_U][TILE];
        T a[CGS_U];
        int sid[CGS_U][NSRC];
#pragma unroll
        for (int u = 0; u < CGS_U; ++u) {
            const bool ok = j + u < j1;
#pragma unroll
            for (int i = 0; i < TILE; ++i) v[u][i] = T(0);
#pragma unroll
            for (int e = 0; e < NSRC; ++e) sid[u][e] = ok ? __ldcs(p.src_gid[e] + j + u) : 0;
            a[u] = ok ? (p.weight ? -(T)__ldcs(p.weight + j + u) : T(-1)) : T(0);
        }
#pragma unroll
        for (int u = 0; u < CGS_U; ++u) {
            if (j + u < j1) {
                cg_add_row<T, TILE, true>(tabs[0] + (long long)sid[u][0] * p.ld, cw, v[u], keep);
#pragma unroll
                for (int e = 1; e < NSRC; ++e)
                    cg_add_row<T, TILE, false>(tabs[e] + (long long)sid[u][e] * p.ld, cw, v[u], keep);
            }
        }
#pragma unroll
        for (int u = 0; u < CGS_U; ++u)
#pragma unroll
            for (int i = 0; i < TILE; ++i) run[i] = fma(a[u], v[u][i], run[i]);
    }
    T* dst = p.sums + (long long)g * p.C + c0;
#pragma unroll
    for (int i = 0; i < TILE; ++i)
        if (i < cw) dst[i] = run[i];
}

template <typename T, int TILE>
int launch_cg_short_tile(const CGRowsParams<T>& p, const int32_t* off, int G, cudaStream_t s) {
    const int ntiles = (p.C + TILE - 1) / TILE;
    const long long threads = (long long)G * ntiles;
    const long long blocks = (threads + 255) / 256;
    if (p.n_src == 1)
        cg_short_kernel<T, TILE, 1><<<(unsigned)blocks, 256, 0, s>>>(p, off, G, ntiles);
    else if (p.n_src == 2)
        cg_short_kernel<T, TILE, 2><<<(unsigned)blocks, 256, 0, s>>>(p, off, G, ntiles);
    else
        cg_short_kernel<T, TILE, 3><<<(unsigned)blocks, 256, 0, s>>>(p, off, G, ntiles);
    FEGB_LAUNCH_CHECK("cg operator sweep (short groups)");
    return 0;
}

template <typename T>
int launch_cg_short(const CGRowsParams<T>& p, const int32_t* off, int G, cudaStream_t s) {
    if (G <= 0) return 0;
    if (p.n_src < 1 || p.n_src > 3) return set_error("cg short-group sweep: %d sources", p.n_src);
    if (p.ld % (32 / (int)sizeof(T)) != 0) return set_error("cg operator: row stride %d is not a 32-byte multiple", p.ld);
    for (int e = 0; e < p.n_src; ++e)
        if ((reinterpret_cast<uintptr_t>(p.src_tab[e]) & 31u) != 0) return set_error("cg operator: unaligned table");
    const int cap = tuning(TUNE_CG_COLS_PER_PASS);
    if (p.C <= 4 || cap == 4) return launch_cg_short_tile<T, 4>(p, off, G, s);
    if (p.C <= 8 || cap == 8) return launch_cg_short_tile<T, 8>(p, off, G, s);
    if (p.C == 9) return launch_cg_short_tile<T, 9>(p, off, G, s);
    if (p.C <= 12) return launch_cg_short_tile<T, 12>(p, off, G, s);
    return launch_cg_short_tile<T, 16>(p, off, G, s);
}

__global__ void max_group_length_kernel(const int32_t* __restrict__ off, int G, int* __restrict__ out) {
    int m = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < G; g += gridDim.x * blockDim.x)
        m = max(m, off[g + 1] - off[g]);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

int max_group_length(const int32_t* off, int G, int* out, cudaStream_t s) {
    *out = 0;
    if (G <= 0) return 0;
    int* d = nullptr;
    FEGB_CUDA(cudaMallocAsync(&d, sizeof(int), s), "max group length");
    FEGB_CUDA(cudaMemsetAsync(d, 0, sizeof(int), s), "max group length reset");
    max_group_length_kernel<<<grid_stride_blocks(G, 256), 256, 0, s>>>(off, G, d);
    FEGB_LAUNCH_CHECK("max group length");
    FEGB_CUDA(cudaMemcpyAsync(out, d, sizeof(int), cudaMemcpyDeviceToHost, s), "max group length copy");
    FEGB_CUDA(cudaFreeAsync(d, s), "max group length free");
    FEGB_CUDA(cudaStreamSynchronize(s), "max group length sync");
    return 0;
}

template int launch_cg_short<double>(const CGRowsParams<double>&, const int32_t*, int, cudaStream_t);
template int launch_cg_short<float>(const CGRowsParams<float>&, const int32_t*, int, cudaStream_t);

template int launch_cg_rows<double>(const CGRowsParams<double>&, cudaStream_t);
template int launch_cg_rows<float>(const CGRowsParams<float>&, cudaStream_t);

template int launch_seg_sweep<double>(const SegSweepParams<double>&, cudaStream_t);
template int launch_seg_sweep<float>(const SegSweepParams<float>&, cudaStream_t);
template int launch_smallg_sweep<double>(const SmallGParams<double>&, int, cudaStream_t);
template int launch_smallg_sweep<float>(const SmallGParams<float>&, int, cudaStream_t);
template int launch_apply_pending<double>(double*, int, long long, const PendingSet<double>&, cudaStream_t);
template int launch_apply_pending<float>(float*, int, long long, const PendingSet<float>&, cudaStream_t);

}  // namespace fegb
