// Shared helpers for the fegb CUDA library: status/last-error handling,
// launch geometry, stream-ordered scratch allocation and small device utilities.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace fegb {

// ---------------------------------------------------------------------------
// Status and last-error text (one buffer per host thread, like the reference
// runtime's thread_local message at src/gpu/fe_gpu_runtime.cu:26).
// ---------------------------------------------------------------------------
int set_ok();
int set_error(const char* fmt, ...);
int set_cuda_error(cudaError_t err, const char* context);
const char* last_error();

#define FEGB_TRY(expr)              \
    do {                            \
        int _st = (expr);           \
        if (_st != 0) return _st;   \
    } while (0)

#define FEGB_CUDA(call, ctx)                                                   \
    do {                                                                       \
        cudaError_t _e = (call);                                               \
        if (_e != cudaSuccess) return ::fegb::set_cuda_error(_e, (ctx));       \
    } while (0)

// Counts every kernel launch of the library (each launch site is followed by
// exactly one FEGB_LAUNCH_CHECK).
void count_launch();
#define FEGB_LAUNCH_CHECK(ctx)                                   \
    do {                                                         \
        ::fegb::count_launch();                                  \
        FEGB_CUDA(cudaPeekAtLastError(), (ctx));                 \
    } while (0)

int num_sms();
long long launches();

inline unsigned grid_1d(long long n, int threads, long long max_blocks = 1LL << 30) {
    long long b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > max_blocks) b = max_blocks;
    return (unsigned)b;
}

// Grid-stride launch size: a few waves of resident blocks.
inline unsigned grid_stride_blocks(long long n, int threads) {
    long long want = (n + threads - 1) / threads;
    long long cap = (long long)num_sms() * 8;
    if (want < 1) want = 1;
    return (unsigned)(want < cap ? want : cap);
}

// ---------------------------------------------------------------------------
// Stream-ordered scratch: a list of cudaMallocAsync blocks freed together.
// ---------------------------------------------------------------------------
class Scratch {
  public:
    explicit Scratch(cudaStream_t s) : stream_(s) {}
    ~Scratch() { release(); }
    Scratch(const Scratch&) = delete;
    Scratch& operator=(const Scratch&) = delete;

    template <typename T>
    int alloc(T** out, size_t count, const char* what) {
        void* p = nullptr;
        size_t bytes = count * sizeof(T);
        if (bytes == 0) bytes = 16;
        bytes = (bytes + 255) & ~size_t(255);
        cudaError_t e = cudaMallocAsync(&p, bytes, stream_);
        if (e != cudaSuccess) {
            *out = nullptr;
            return set_cuda_error(e, what);
        }
        ptrs_.push_back(p);
        *out = static_cast<T*>(p);
        return 0;
    }
    void release() {
        for (void* p : ptrs_) cudaFreeAsync(p, stream_);
        ptrs_.clear();
    }
    cudaStream_t stream() const { return stream_; }

  private:
    cudaStream_t stream_;
    std::vector<void*> ptrs_;
};

// Keep the default memory pool's freed blocks cached across calls.
void configure_mem_pool();

// Launch-shape knobs (process-wide), set through fegb_set_tuning by the host
// from the autotuner's table (fe_gpu_gb300/autotune.py):
//   TUNE_DENSE_FORM       -1 default, 0 CUDA-core, 1 tensor-core count-matrix passes
//   TUNE_CG_COLS_PER_PASS 0 all columns of a row in one pass of the operator
//                         sweep, else at most 4 or 8 (more passes, fewer registers)
//   TUNE_SPLIT_GRAM       output pairs per input column from which Gram
//                         products use the split-FP32 form (>= 1)
//   TUNE_CG_GRAPH         1 the CG loop runs as a CUDA graph, 0 host-driven
//   TUNE_BATCH_ESTIMATOR  1 batched specifications are estimated class by
//                         class in one batched pass, 0 one by one
//   TUNE_CG_SHORT         1 operator sweeps of streams whose groups are all
//                         short run one thread per group, 0 the chunked sweep
enum TuneKey {
    TUNE_DENSE_FORM = 0,
    TUNE_CG_COLS_PER_PASS,
    TUNE_SPLIT_GRAM,
    TUNE_CG_GRAPH,
    TUNE_BATCH_ESTIMATOR,
    TUNE_CG_SHORT,
    TUNE_COUNT
};
int tuning(TuneKey key);

// ---------------------------------------------------------------------------
// Device helpers
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long dbl_bits(double v) {
    return (unsigned long long)__double_as_longlong(v);
}
__device__ __forceinline__ double bits_dbl(unsigned long long b) { return __longlong_as_double((long long)b); }

// atomicMax on a non-negative double stored as its bit pattern (the order of
// the bit patterns of non-negative doubles is the numeric order). Max is order
// independent, so the result is deterministic.
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long* slot, double v) {
    atomicMax(slot, dbl_bits(v));
}

// (hi, lo) FP32 pair of an FP64 value from its IEEE-754 fields, without the
// FP64 pipe: hi = the leading 24 significant bits (truncated), lo = the
// remaining 29 bits times their power of two (rounded to 24 bits by the
// integer conversion, scaled exactly), so |v - hi - lo| <= 2^-48 |v| for
// 2^-60 <= |v| < 2^(EMAX+1). Below 2^-60 lo is dropped (relative error <= 2^-23
// of a value that small); below 2^-126 the value counts as zero. From
// 2^(EMAX+1) up, and for non-finite values, bad is set and (0, 0) returned.
template <int EMAX>
__device__ __forceinline__ float2 split_f64(double v, bool& bad) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7FF);
    if (e > 1023 + EMAX) {
        bad = true;
        return make_float2(0.f, 0.f);
    }
    if (e < 1023 - 126) return make_float2(0.f, 0.f);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const unsigned long long mant = b & ((1ULL << 52) - 1ULL);
    const float hi = __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(mant >> 29));
    if (e < 1023 - 60) return make_float2(hi, 0.f);
    const unsigned rem = (unsigned)(mant & ((1ULL << 29) - 1ULL));
    const float scale = __uint_as_float((unsigned)(e - 1075 + 127) << 23);  // 2^(e - 1075), a normal float here
    const float lo = __uint_as_float(__float_as_uint((float)rem * scale) | sign);
    return make_float2(hi, lo);
}

// Max over the warp of non-negative doubles, taken on their bit patterns: the
// integer pipe instead of the FP64 one, which is narrow on this part.
__device__ __forceinline__ double warp_max(double v) {
    unsigned long long b = dbl_bits(v);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ob = __shfl_xor_sync(0xffffffffu, b, o);
        b = ob > b ? ob : b;
    }
    return bits_dbl(b);
}

}  // namespace fegb
