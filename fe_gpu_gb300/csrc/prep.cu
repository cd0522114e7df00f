// Integer preparation: scans, stable radix sorts, segment offsets, id
// compaction, cluster-intersection ids and singleton removal.
//
// The radix sort is an LSD sort with 8-bit digits. Each pass runs a per-tile
// digit histogram, a device-wide exclusive scan over the digit-major count
// table and a stable scatter in which every warp ranks 32 consecutive keys with
// __match_any_sync and keeps running per-digit counters in shared memory, so
// the output order depends only on the input (no atomics decide positions).
#include "prep.cuh"

#include <algorithm>

namespace fegb {

namespace {

constexpr int SC_THREADS = 256;
constexpr int SC_ITEMS = 8;
constexpr int SC_TILE = SC_THREADS * SC_ITEMS;

// Block-wide exclusive scan of SC_TILE uint32 values held SC_ITEMS per thread.
__device__ uint32_t block_exclusive_scan(uint32_t (&v)[SC_ITEMS], uint32_t* warp_sums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t local = 0;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) {
        uint32_t t = v[i];
        v[i] = local;
        local += t;
    }
    uint32_t incl = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t ws = lane < (SC_THREADS / 32) ? warp_sums[lane] : 0;
        uint32_t wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < (SC_THREADS / 32)) warp_sums[lane] = wi - ws;  // exclusive
        if (lane == (SC_THREADS / 32) - 1) warp_sums[SC_THREADS / 32] = wi;
    }
    __syncthreads();
    uint32_t base = warp_sums[warp] + (incl - local);
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) v[i] += base;
    uint32_t total = warp_sums[SC_THREADS / 32];
    __syncthreads();
    return total;
}

__global__ void scan_tile_sums_kernel(const uint32_t* __restrict__ in, long long n, uint32_t* __restrict__ sums) {
    __shared__ uint32_t ws[SC_THREADS / 32 + 1];
    uint32_t v[SC_ITEMS];
    long long base = (long long)blockIdx.x * SC_TILE + (long long)threadIdx.x * SC_ITEMS;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) v[i] = (base + i < n) ? in[base + i] : 0u;
    uint32_t total = block_exclusive_scan(v, ws);
    if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void scan_tile_apply_kernel(const uint32_t* __restrict__ in, long long n, const uint32_t* __restrict__ offs,
                                       uint32_t* __restrict__ out) {
    __shared__ uint32_t ws[SC_THREADS / 32 + 1];
    uint32_t v[SC_ITEMS];
    long long base = (long long)blockIdx.x * SC_TILE + (long long)threadIdx.x * SC_ITEMS;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i) v[i] = (base + i < n) ? in[base + i] : 0u;
    block_exclusive_scan(v, ws);
    uint32_t off = offs ? offs[blockIdx.x] : 0u;
#pragma unroll
    for (int i = 0; i < SC_ITEMS; ++i)
        if (base + i < n) out[base + i] = v[i] + off;
}

__global__ void write_total_kernel(const uint32_t* in_last, const uint32_t* out_last, uint32_t* total) {
    *total = *in_last + *out_last;
}

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;
constexpr int RS_SUB = RS_TILE / RS_WARPS;
constexpr int RS_BINS = 256;

template <typename K>
__global__ void __launch_bounds__(RS_THREADS) rs_hist_kernel(const K* __restrict__ keys, long long n, int shift,
                                                            uint32_t* __restrict__ counts, int nblocks) {
    __shared__ uint32_t h[RS_BINS];
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) h[i] = 0;
    __syncthreads();
    long long base = (long long)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int it = 0; it < RS_ITEMS; ++it) {
        long long j = base + (long long)it * RS_THREADS + threadIdx.x;
        if (j < n) atomicAdd(&h[(unsigned)((keys[j] >> shift) & 255u)], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < RS_BINS; i += RS_THREADS) counts[(size_t)i * nblocks + blockIdx.x] = h[i];
}

template <typename K>
__global__ void __launch_bounds__(RS_THREADS)
    rs_scatter_kernel(const K* __restrict__ kin, const int32_t* __restrict__ vin, K* __restrict__ kout,
                      int32_t* __restrict__ vout, long long n, int shift, const uint32_t* __restrict__ offs,
                      int nblocks) {
    __shared__ uint32_t cnt[RS_WARPS][RS_BINS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE + (long long)warp * RS_SUB;
    for (int r = 0; r < RS_SUB / 32; ++r) {
        long long j = base + r * 32 + lane;
        if (j < n) atomicAdd(&cnt[warp][(unsigned)((kin[j] >> shift) & 255u)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < RS_BINS; d += RS_THREADS) {
        uint32_t run = offs[(size_t)d * nblocks + blockIdx.x];
#pragma unroll
        for (int w = 0; w < RS_WARPS; ++w) {
            uint32_t c = cnt[w][d];
            cnt[w][d] = run;
            run += c;
        }
    }
    __syncthreads();
    const unsigned lt_mask = (1u << lane) - 1u;
    for (int r = 0; r < RS_SUB / 32; ++r) {
        long long j = base + r * 32 + lane;
        bool valid = j < n;
        K key = valid ? kin[j] : K(0);
        unsigned d = valid ? (unsigned)((key >> shift) & 255u) : 256u;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        unsigned rank = __popc(peers & lt_mask);
        if (valid) {
            uint32_t pos = cnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = vin ? vin[j] : (int32_t)j;
        }
        __syncwarp();
        if (valid && lane == __ffs(peers) - 1) cnt[warp][d] += __popc(peers);
        __syncwarp();
    }
}

template <typename K>
__global__ void copy_pairs_kernel(const K* kin, const int32_t* vin, K* kout, int32_t* vout, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        kout[i] = kin[i];
        vout[i] = vin ? vin[i] : (int32_t)i;
    }
}

template <typename K>
int radix_sort_impl(const K* keys_in, const int32_t* vals_in, K* keys_out, int32_t* vals_out, long long n, int bits,
                    cudaStream_t s, Scratch& scr) {
    if (n <= 0) return 0;
    if (n > 0x7fffffffLL) return set_error("radix sort: n=%lld exceeds the int32 index range", n);
    int passes = (bits + 7) / 8;
    if (passes <= 0) {
        copy_pairs_kernel<K><<<grid_stride_blocks(n, 256), 256, 0, s>>>(keys_in, vals_in, keys_out, vals_out, n);
        FEGB_LAUNCH_CHECK("radix sort copy");
        return 0;
    }
    int nblocks = (int)((n + RS_TILE - 1) / RS_TILE);
    K* ktmp = nullptr;
    int32_t* vtmp = nullptr;
    uint32_t *counts = nullptr, *offs = nullptr;
    FEGB_TRY(scr.alloc(&ktmp, (size_t)n, "radix sort keys"));
    FEGB_TRY(scr.alloc(&vtmp, (size_t)n, "radix sort values"));
    FEGB_TRY(scr.alloc(&counts, (size_t)RS_BINS * nblocks, "radix sort counts"));
    FEGB_TRY(scr.alloc(&offs, (size_t)RS_BINS * nblocks, "radix sort offsets"));
    const K* kcur = keys_in;
    const int32_t* vcur = vals_in;
    for (int p = 0; p < passes; ++p) {
        // the last pass must land in keys_out
        bool to_out = ((passes - 1 - p) % 2) == 0;
        K* kdst = to_out ? keys_out : ktmp;
        int32_t* vdst = to_out ? vals_out : vtmp;
        int shift = 8 * p;
        rs_hist_kernel<K><<<nblocks, RS_THREADS, 0, s>>>(kcur, n, shift, counts, nblocks);
        FEGB_LAUNCH_CHECK("radix histogram");
        FEGB_TRY(scan_exclusive_u32(counts, offs, (long long)RS_BINS * nblocks, nullptr, s, scr));
        rs_scatter_kernel<K><<<nblocks, RS_THREADS, 0, s>>>(kcur, vcur, kdst, vdst, n, shift, offs, nblocks);
        FEGB_LAUNCH_CHECK("radix scatter");
        kcur = kdst;
        vcur = vdst;
    }
    return 0;
}

__global__ void offsets_kernel(const uint32_t* __restrict__ ids, long long n, int G, int32_t* __restrict__ off) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; j <= n; j += stride) {
        long long lo = (j == 0) ? -1 : (long long)ids[j - 1];
        long long hi = (j == n) ? (long long)G - 1 : (long long)ids[j];
        for (long long g = lo + 1; g <= hi; ++g) off[g] = (int32_t)j;
        if (j == n) off[G] = (int32_t)n;
    }
}

__global__ void min_max_kernel(const int32_t* __restrict__ ids, long long n, int* mn, int* mx) {
    int lmin = 0x7fffffff, lmax = (int)0x80000000;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) {
        int v = ids[i];
        lmin = min(lmin, v);
        lmax = max(lmax, v);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
        lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMin(mn, lmin);
        atomicMax(mx, lmax);
    }
}

__global__ void init_min_max_kernel(int* mn, int* mx) {
    *mn = 0x7fffffff;
    *mx = (int)0x80000000;
}

__global__ void flip_sign_kernel(const int32_t* in, uint32_t* out, long long n) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += stride) out[i] = (uint32_t)in[i] ^ 0x80000000u;
}

template <typename K>
__global__ void change_flags_kernel(const K* __restrict__ sorted, long long n, uint32_t* __restrict__ flags) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; j < n; j += stride) flags[j] = (j == 0 || sorted[j] != sorted[j - 1]) ? 1u : 0u;
}

// ids[perm[j]] = excl[j] + flags[j] (1-based rank); cluster offsets at starts.
__global__ void scatter_ranks_kernel(const int32_t* __restrict__ perm, const uint32_t* __restrict__ excl,
                                     const uint32_t* __restrict__ flags, long long n, int32_t* __restrict__ ids,
                                     int32_t* __restrict__ offsets, int32_t* __restrict__ gseq) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long stride = (long long)gridDim.x * blockDim.x;
    for (; j < n; j += stride) {
        uint32_t rank = excl[j] + flags[j];
        if (ids) ids[perm[j]] = (int32_t)rank;
        if (offsets && flags[j]) offsets[rank - 1] = (int32_t)j;
        if (gseq) gseq[j] = (int32_t)rank - 1;
    }
}

__global__ void set_int_kernel(int32_t* p, int32_t v) { *p = v; }

__global__ void max_u64_kernel(const unsigned long long* __restrict__ keys, long long n, unsigned long long* out) {
    unsigned long long m = 0;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) m = keys[i] > m ? keys[i] : m;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long y = __shfl_xor_sync(0xffffffffu, m, o);
        m = y > m ? y : m;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

struct DimPtrs {
    const int32_t* p[4];
    unsigned long long stride[4];
    int n;
    int zero_based;
};

template <typename K>
__global__ void keys_kernel(DimPtrs dp, long long n, K* __restrict__ keys) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) {
        unsigned long long key = 0;
        for (int d = 0; d < dp.n; ++d) {
            int v = dp.p[d][i];
            if (dp.zero_based)
                key += (unsigned long long)v * dp.stride[d];
            else if (v > 0)
                key += (unsigned long long)(v - 1) * dp.stride[d];
        }
        keys[i] = (K)key;
    }
}

__global__ void gather_u32_kernel(const int32_t* __restrict__ src, const int32_t* __restrict__ perm, long long n,
                                  int add, uint32_t* __restrict__ out) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) out[i] = (uint32_t)(src[perm ? perm[i] : i] + add);
}

// tuple-change flags over rows in perm order
struct TupleDims {
    const int32_t* p[4];
    int n;
};
__global__ void tuple_flags_kernel(TupleDims td, const int32_t* __restrict__ perm, long long n,
                                   uint32_t* __restrict__ flags) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; j < n; j += st) {
        uint32_t f = 1u;
        if (j > 0) {
            int a = perm[j], b = perm[j - 1];
            f = 0u;
            for (int d = 0; d < td.n; ++d) f |= (td.p[d][a] != td.p[d][b]) ? 1u : 0u;
        }
        flags[j] = f;
    }
}

// segment first positions: first[seg] = perm[j] where flags[j]
__global__ void seg_first_kernel(const int32_t* __restrict__ perm, const uint32_t* __restrict__ excl,
                                 const uint32_t* __restrict__ flags, long long n, uint32_t* __restrict__ first) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; j < n; j += st)
        if (flags[j]) first[excl[j]] = (uint32_t)perm[j];
}

__global__ void seg_rank_kernel(const int32_t* __restrict__ seg_sorted, long long m, int32_t* __restrict__ id_of_seg) {
    long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; r < m; r += st) id_of_seg[seg_sorted[r]] = (int32_t)(r + 1);
}

__global__ void assign_first_ids_kernel(const int32_t* __restrict__ perm, const uint32_t* __restrict__ excl,
                                        const uint32_t* __restrict__ flags, const int32_t* __restrict__ id_of_seg,
                                        long long n, int32_t* __restrict__ ids) {
    long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; j < n; j += st) {
        uint32_t seg = excl[j] + flags[j] - 1u;
        ids[perm[j]] = id_of_seg[seg];
    }
}

__global__ void count_kept_kernel(const int32_t* __restrict__ gid, const uint8_t* __restrict__ keep, long long n,
                                  int32_t* __restrict__ cnt) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st)
        if (keep[i]) atomicAdd(&cnt[gid[i]], 1);
}

__global__ void drop_single_kernel(const int32_t* __restrict__ gid, uint8_t* __restrict__ keep, long long n,
                                   const int32_t* __restrict__ cnt, unsigned long long* __restrict__ dropped) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    unsigned long long local = 0;
    for (; i < n; i += st)
        if (keep[i] && cnt[gid[i]] == 1) {
            keep[i] = 0;
            ++local;
        }
    if (local) atomicAdd(dropped, local);
}

__global__ void fill_u8_kernel(uint8_t* p, long long n, uint8_t v) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) p[i] = v;
}

}  // namespace

int bits_for(unsigned long long span) {
    int b = 0;
    unsigned long long v = span > 0 ? span - 1 : 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

int scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n, uint32_t* total_dev, cudaStream_t s,
                       Scratch& scr) {
    if (n <= 0) return 0;
    long long nb = (n + SC_TILE - 1) / SC_TILE;
    if (nb == 1) {
        scan_tile_apply_kernel<<<1, SC_THREADS, 0, s>>>(in, n, nullptr, out);
        FEGB_LAUNCH_CHECK("scan tile");
    } else {
        uint32_t *sums = nullptr, *offs = nullptr;
        FEGB_TRY(scr.alloc(&sums, (size_t)nb, "scan sums"));
        FEGB_TRY(scr.alloc(&offs, (size_t)nb, "scan offsets"));
        scan_tile_sums_kernel<<<(unsigned)nb, SC_THREADS, 0, s>>>(in, n, sums);
        FEGB_LAUNCH_CHECK("scan tile sums");
        FEGB_TRY(scan_exclusive_u32(sums, offs, nb, nullptr, s, scr));
        scan_tile_apply_kernel<<<(unsigned)nb, SC_THREADS, 0, s>>>(in, n, offs, out);
        FEGB_LAUNCH_CHECK("scan apply");
    }
    if (total_dev) {
        write_total_kernel<<<1, 1, 0, s>>>(in + (n - 1), out + (n - 1), total_dev);
        FEGB_LAUNCH_CHECK("scan total");
    }
    return 0;
}

int radix_sort_u32(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out, int32_t* vals_out, long long n,
                   int bits, cudaStream_t s, Scratch& scr) {
    return radix_sort_impl<uint32_t>(keys_in, vals_in, keys_out, vals_out, n, bits, s, scr);
}

int radix_sort_u64(const unsigned long long* keys_in, const int32_t* vals_in, unsigned long long* keys_out,
                   int32_t* vals_out, long long n, int bits, cudaStream_t s, Scratch& scr) {
    return radix_sort_impl<unsigned long long>(keys_in, vals_in, keys_out, vals_out, n, bits, s, scr);
}

int segment_offsets(const uint32_t* sorted_ids, long long n, int G, int32_t* offsets, cudaStream_t s) {
    offsets_kernel<<<grid_stride_blocks(n + 1, 256), 256, 0, s>>>(sorted_ids, n, G, offsets);
    FEGB_LAUNCH_CHECK("segment offsets");
    return 0;
}

int ids_min_max(const int32_t* ids, long long n, int* out_min, int* out_max, cudaStream_t s, Scratch& scr) {
    int* d = nullptr;
    FEGB_TRY(scr.alloc(&d, 2, "min/max"));
    init_min_max_kernel<<<1, 1, 0, s>>>(d, d + 1);
    if (n > 0) min_max_kernel<<<grid_stride_blocks(n, 256), 256, 0, s>>>(ids, n, d, d + 1);
    FEGB_LAUNCH_CHECK("min/max");
    int h[2];
    FEGB_CUDA(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s), "min/max copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "min/max sync");
    *out_min = h[0];
    *out_max = h[1];
    return 0;
}

int compact_ids(const int32_t* raw, long long n, int32_t* out, int* n_levels, cudaStream_t s, Scratch& scr) {
    if (n <= 0) {
        *n_levels = 0;
        return 0;
    }
    uint32_t *keys = nullptr, *sorted = nullptr, *flags = nullptr, *excl = nullptr, *total = nullptr;
    int32_t* perm = nullptr;
    FEGB_TRY(scr.alloc(&keys, (size_t)n, "compact keys"));
    FEGB_TRY(scr.alloc(&sorted, (size_t)n, "compact sorted"));
    FEGB_TRY(scr.alloc(&perm, (size_t)n, "compact perm"));
    FEGB_TRY(scr.alloc(&flags, (size_t)n, "compact flags"));
    FEGB_TRY(scr.alloc(&excl, (size_t)n, "compact scan"));
    FEGB_TRY(scr.alloc(&total, 1, "compact total"));
    unsigned g = grid_stride_blocks(n, 256);
    flip_sign_kernel<<<g, 256, 0, s>>>(raw, keys, n);
    FEGB_LAUNCH_CHECK("compact keys");
    FEGB_TRY(radix_sort_u32(keys, nullptr, sorted, perm, n, 32, s, scr));
    change_flags_kernel<uint32_t><<<g, 256, 0, s>>>(sorted, n, flags);
    FEGB_LAUNCH_CHECK("compact flags");
    FEGB_TRY(scan_exclusive_u32(flags, excl, n, total, s, scr));
    scatter_ranks_kernel<<<g, 256, 0, s>>>(perm, excl, flags, n, out, nullptr, nullptr);
    FEGB_LAUNCH_CHECK("compact ranks");
    uint32_t h = 0;
    FEGB_CUDA(cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, s), "compact total copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "compact sync");
    *n_levels = (int)h;
    return 0;
}

int cluster_ids_by_key(const int32_t* const* dims, const unsigned long long* strides, int n_dims, long long n,
                       int key_bits, int32_t* out_ids, int* out_n_clusters, int32_t* perm_out, int32_t* offsets_out,
                       cudaStream_t s, Scratch& scr, bool zero_based, int32_t* gseq_out) {
    if (n_dims < 1 || n_dims > 4) return set_error("cluster ids: n_dims=%d outside [1,4]", n_dims);
    if (n <= 0) {
        *out_n_clusters = 0;
        return 0;
    }
    DimPtrs dp{};
    dp.n = n_dims;
    dp.zero_based = zero_based ? 1 : 0;
    for (int d = 0; d < n_dims; ++d) {
        dp.p[d] = dims[d];
        dp.stride[d] = strides[d];
    }
    int32_t* perm = perm_out;
    uint32_t *flags = nullptr, *excl = nullptr, *total = nullptr;
    if (!perm) FEGB_TRY(scr.alloc(&perm, (size_t)n, "cluster perm"));
    FEGB_TRY(scr.alloc(&flags, (size_t)n, "cluster flags"));
    FEGB_TRY(scr.alloc(&excl, (size_t)n, "cluster scan"));
    FEGB_TRY(scr.alloc(&total, 1, "cluster total"));
    unsigned g = grid_stride_blocks(n, 256);
    if (key_bits >= 0 && key_bits <= 32) {
        // keys that fit 32 bits: half the bytes moved by every radix pass
        uint32_t *keys = nullptr, *sorted = nullptr;
        FEGB_TRY(scr.alloc(&keys, (size_t)n, "cluster keys"));
        FEGB_TRY(scr.alloc(&sorted, (size_t)n, "cluster sorted keys"));
        keys_kernel<uint32_t><<<g, 256, 0, s>>>(dp, n, keys);
        FEGB_LAUNCH_CHECK("cluster keys");
        FEGB_TRY(radix_sort_u32(keys, nullptr, sorted, perm, n, key_bits, s, scr));
        change_flags_kernel<uint32_t><<<g, 256, 0, s>>>(sorted, n, flags);
        FEGB_LAUNCH_CHECK("cluster flags");
    } else {
        unsigned long long *keys = nullptr, *sorted = nullptr;
        FEGB_TRY(scr.alloc(&keys, (size_t)n, "cluster keys"));
        FEGB_TRY(scr.alloc(&sorted, (size_t)n, "cluster sorted keys"));
        keys_kernel<unsigned long long><<<g, 256, 0, s>>>(dp, n, keys);
        FEGB_LAUNCH_CHECK("cluster keys");
        if (key_bits < 0) {
            unsigned long long* mx = nullptr;
            FEGB_TRY(scr.alloc(&mx, 1, "max key"));
            FEGB_CUDA(cudaMemsetAsync(mx, 0, sizeof(unsigned long long), s), "max key reset");
            max_u64_kernel<<<g, 256, 0, s>>>(keys, n, mx);
            FEGB_LAUNCH_CHECK("max key");
            unsigned long long h = 0;
            FEGB_CUDA(cudaMemcpyAsync(&h, mx, sizeof(h), cudaMemcpyDeviceToHost, s), "max key copy");
            FEGB_CUDA(cudaStreamSynchronize(s), "max key sync");
            key_bits = 0;
            while (key_bits < 64 && (h >> key_bits) != 0ull) ++key_bits;
        }
        FEGB_TRY(radix_sort_u64(keys, nullptr, sorted, perm, n, key_bits, s, scr));
        change_flags_kernel<unsigned long long><<<g, 256, 0, s>>>(sorted, n, flags);
        FEGB_LAUNCH_CHECK("cluster flags");
    }
    FEGB_TRY(scan_exclusive_u32(flags, excl, n, total, s, scr));
    scatter_ranks_kernel<<<g, 256, 0, s>>>(perm, excl, flags, n, out_ids, offsets_out, gseq_out);
    FEGB_LAUNCH_CHECK("cluster ranks");
    uint32_t h = 0;
    FEGB_CUDA(cudaMemcpyAsync(&h, total, sizeof(h), cudaMemcpyDeviceToHost, s), "cluster count copy");
    FEGB_CUDA(cudaStreamSynchronize(s), "cluster count sync");
    *out_n_clusters = (int)h;
    if (offsets_out) {
        set_int_kernel<<<1, 1, 0, s>>>(offsets_out + h, (int32_t)n);
        FEGB_LAUNCH_CHECK("cluster offsets end");
    }
    return 0;
}

int cluster_ids_first_appearance(const int32_t* const* dims, const int* sizes, int n_dims, long long n,
                                 int32_t* out_ids, int* out_n_clusters, cudaStream_t s, Scratch& scr) {
    if (n_dims < 1 || n_dims > 4) return set_error("cluster ids: n_dims=%d outside [1,4]", n_dims);
    if (n <= 0) {
        *out_n_clusters = 0;
        return 0;
    }
    uint32_t *k = nullptr, *ks = nullptr, *flags = nullptr, *excl = nullptr, *total = nullptr, *first = nullptr,
             *first_sorted = nullptr;
    int32_t *pa = nullptr, *pb = nullptr, *seg_sorted = nullptr, *id_of_seg = nullptr;
    FEGB_TRY(scr.alloc(&k, (size_t)n, "fa keys"));
    FEGB_TRY(scr.alloc(&ks, (size_t)n, "fa sorted keys"));
    FEGB_TRY(scr.alloc(&pa, (size_t)n, "fa perm a"));
    FEGB_TRY(scr.alloc(&pb, (size_t)n, "fa perm b"));
    unsigned g = grid_stride_blocks(n, 256);
    // LSD over tuple components: the last component first; stability keeps
    // rows of equal tuples in original order.
    const int32_t* cur_perm = nullptr;
    for (int d = n_dims - 1; d >= 0; --d) {
        gather_u32_kernel<<<g, 256, 0, s>>>(dims[d], cur_perm, n, -1, k);
        FEGB_LAUNCH_CHECK("fa gather");
        int32_t* dst = (cur_perm == pa) ? pb : pa;
        FEGB_TRY(radix_sort_u32(k, cur_perm, ks, dst, n, bits_for((unsigned long long)(sizes[d] > 0 ? sizes[d] : 1)) + 1,
                                s, scr));
        cur_perm = dst;
    }
    TupleDims td{};
    td.n = n_dims;
    for (int d = 0; d < n_dims; ++d) td.p[d] = dims[d];
    FEGB_TRY(scr.alloc(&flags, (size_t)n, "fa flags"));
    FEGB_TRY(scr.alloc(&excl, (size_t)n, "fa scan"));
    FEGB_TRY(scr.alloc(&total, 1, "fa total"));
    tuple_flags_kernel<<<g, 256, 0, s>>>(td, cur_perm, n, flags);
    FEGB_LAUNCH_CHECK("fa flags");
    FEGB_TRY(scan_exclusive_u32(flags, excl, n, total, s, scr));
    uint32_t m = 0;
    FEGB_CUDA(cudaMemcpyAsync(&m, total, sizeof(m), cudaMemcpyDeviceToHost, s), "fa count");
    FEGB_CUDA(cudaStreamSynchronize(s), "fa sync");
    FEGB_TRY(scr.alloc(&first, (size_t)m, "fa first"));
    FEGB_TRY(scr.alloc(&first_sorted, (size_t)m, "fa first sorted"));
    FEGB_TRY(scr.alloc(&seg_sorted, (size_t)m, "fa seg sorted"));
    FEGB_TRY(scr.alloc(&id_of_seg, (size_t)m, "fa id of seg"));
    seg_first_kernel<<<g, 256, 0, s>>>(cur_perm, excl, flags, n, first);
    FEGB_LAUNCH_CHECK("fa first");
    FEGB_TRY(radix_sort_u32(first, nullptr, first_sorted, seg_sorted, m, bits_for((unsigned long long)n), s, scr));
    seg_rank_kernel<<<grid_stride_blocks(m, 256), 256, 0, s>>>(seg_sorted, m, id_of_seg);
    FEGB_LAUNCH_CHECK("fa seg rank");
    assign_first_ids_kernel<<<g, 256, 0, s>>>(cur_perm, excl, flags, id_of_seg, n, out_ids);
    FEGB_LAUNCH_CHECK("fa assign");
    *out_n_clusters = (int)m;
    return 0;
}

int drop_singletons(const int32_t* const* gid, const int* G, int n_fe, long long n, uint8_t* keep,
                    long long* n_dropped, cudaStream_t s, Scratch& scr) {
    *n_dropped = 0;
    unsigned g = grid_stride_blocks(n, 256);
    fill_u8_kernel<<<g, 256, 0, s>>>(keep, n, 1);
    FEGB_LAUNCH_CHECK("singletons init");
    int gmax = 1;
    for (int d = 0; d < n_fe; ++d) gmax = std::max(gmax, G[d]);
    int32_t* cnt = nullptr;
    unsigned long long* dropped = nullptr;
    FEGB_TRY(scr.alloc(&cnt, (size_t)gmax, "singleton counts"));
    FEGB_TRY(scr.alloc(&dropped, 1, "singleton dropped"));
    for (int round = 0; round < 1000000; ++round) {
        unsigned long long total = 0;
        FEGB_CUDA(cudaMemsetAsync(dropped, 0, sizeof(unsigned long long), s), "singleton reset");
        for (int d = 0; d < n_fe; ++d) {
            FEGB_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)G[d], s), "singleton count reset");
            count_kept_kernel<<<g, 256, 0, s>>>(gid[d], keep, n, cnt);
            drop_single_kernel<<<g, 256, 0, s>>>(gid[d], keep, n, cnt, dropped);
            FEGB_LAUNCH_CHECK("singleton pass");
        }
        FEGB_CUDA(cudaMemcpyAsync(&total, dropped, sizeof(total), cudaMemcpyDeviceToHost, s), "singleton copy");
        FEGB_CUDA(cudaStreamSynchronize(s), "singleton sync");
        *n_dropped += (long long)total;
        if (total == 0) break;
    }
    return 0;
}

}  // namespace fegb
