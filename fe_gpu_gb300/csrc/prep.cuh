// Integer preparation primitives: device-wide scans, stable LSD radix sorts,
// segment offsets, id compaction and multi-way cluster-intersection ids.
// Everything here is integer work and bit-exact.
#pragma once

#include "common.cuh"

namespace fegb {

// out[i] = sum_{j<i} in[j]; *total_dev (device, optional) = sum of all.
int scan_exclusive_u32(const uint32_t* in, uint32_t* out, long long n, uint32_t* total_dev, cudaStream_t s,
                       Scratch& scr);

// Stable LSD radix sort of (key, value) pairs on key bits [0, bits).
// keys_in/vals_in are not modified; outputs must not alias inputs.
// vals_in may be null: values are then the input positions 0..n-1.
int radix_sort_u32(const uint32_t* keys_in, const int32_t* vals_in, uint32_t* keys_out, int32_t* vals_out, long long n,
                   int bits, cudaStream_t s, Scratch& scr);
int radix_sort_u64(const unsigned long long* keys_in, const int32_t* vals_in, unsigned long long* keys_out,
                   int32_t* vals_out, long long n, int bits, cudaStream_t s, Scratch& scr);

// offsets[g] = first position of group g in a sorted id array (ids in [0, G)),
// offsets[G] = n. Empty groups get equal consecutive offsets.
int segment_offsets(const uint32_t* sorted_ids, long long n, int G, int32_t* offsets, cudaStream_t s);

// Max and min of an int32 array (device results written to host pointers).
int ids_min_max(const int32_t* ids, long long n, int* out_min, int* out_max, cudaStream_t s, Scratch& scr);

// Number of bits needed to represent values < span (span >= 1).
int bits_for(unsigned long long span);

// 1-based rank among the sorted distinct values of raw (int32, any sign):
// pandas factorize(sort=True) + 1. *n_levels is written on the host.
int compact_ids(const int32_t* raw, long long n, int32_t* out, int* n_levels, cudaStream_t s, Scratch& scr);

// Multi-way cluster-intersection ids (1-based), bit-identical to the
// reference's CPU builder: ranks of the distinct mixed-radix keys
// key = sum_j (v_j - 1) * stride_j in increasing key order. dims[j] are device
// pointers to 1-based id arrays; ids <= 0 contribute nothing to the key (as in
// the reference GPU builder). When perm_out/offsets_out are non-null the sort
// permutation (rows in key order) and per-cluster offsets (n_clusters+1) are
// returned too; offsets_out must hold n+1 entries.
// When zero_based is set the id arrays hold 0-based ids and every value enters
// the key (v * stride). gseq_out (optional, n) receives the 0-based cluster of
// each sorted position.
int cluster_ids_by_key(const int32_t* const* dims, const unsigned long long* strides, int n_dims, long long n,
                       int key_bits, int32_t* out_ids, int* out_n_clusters, int32_t* perm_out, int32_t* offsets_out,
                       cudaStream_t s, Scratch& scr, bool zero_based = false, int32_t* gseq_out = nullptr);

// First-appearance ids for tuples whose mixed-radix span does not fit 2^62
// (reference src/core/cluster_id_builder.c:202-257 hash fallback).
int cluster_ids_first_appearance(const int32_t* const* dims, const int* sizes, int n_dims, long long n,
                                 int32_t* out_ids, int* out_n_clusters, cudaStream_t s, Scratch& scr);

// Iterated singleton removal over n_fe id arrays (0-based ids < G[d]).
// keep[i] = 1 for surviving rows; returns number dropped in *n_dropped.
int drop_singletons(const int32_t* const* gid, const int* G, int n_fe, long long n, uint8_t* keep,
                    long long* n_dropped, cudaStream_t s, Scratch& scr);

}  // namespace fegb
