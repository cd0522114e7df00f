// Tensor-core (tcgen05) form of the dense count-matrix pass of the CG operator.
//
// One pass over the count matrix M (Ge x Gs, uint8, row g = the rows of each
// group t of a small dimension s inside group g of a dimension e) forms two
// small products per tile of UT = 128 groups of e:
//
//   E = M_tile . S            (128 x Gs by Gs x C)   the e side / Schur u
//   D2 += U_tile' . M_tile    (C x 128 by 128 x Gs)  the small side
//
// where S holds the small dimension's rows ps and U the tile's rows of pe (or,
// in the Schur form, u = (sums - E) / counts, which the pass also writes to the
// primary's table). Both products run on the 5th-generation tensor cores:
// tcgen05.mma kind::f16 with BF16 operands and FP32 accumulation in tensor
// memory, issued by one thread of the CTA.
//
// Exactness of the operands: counts up to 255 are exact in BF16 (8 significant
// bits). Every FP32 value v of S and U is split into three BF16 pieces
// h = bf16(v), m = bf16(v - h), l = bf16(v - h - m) with v = h + m + l exactly,
// so every product of a count and a piece is exact in FP32 and the three
// pieces are accumulated as separate columns (E) or rows (D2) and added in the
// order l + m + h afterwards. The result carries FP32 accumulation rounding
// only, as the FP32 CUDA-core form does.
//
// Data movement: the tile's count bytes and row data are contiguous runs in
// global memory and are fetched by cp.async.bulk (the TMA's bulk copy engine)
// into double-buffered stages completing on mbarriers, the counts three tiles
// and the rows two tiles ahead of their use. A 2-D tensor map does not apply:
// its row strides must be multiples of 16 bytes, and these rows are Gs bytes
// (30 at the 150M-row panel) and C floats (36 bytes) long. The CUDA cores
// convert the counts to BF16 in the MMA operand layout (a byte placed in the
// mantissa of 2^23 and 2^23 subtracted: exact, no conversion unit), form u and
// its pieces, and read the accumulators back from tensor memory with
// tcgen05.ld. E is double-buffered in tensor memory, so the MMA of tile i + 1
// runs while the CUDA cores finish tile i.
//
// The small-side product uses M = 64 (48 rows used): its accumulator row r
// sits in tensor-memory lane (r / 16) * 32 + r % 16, so piece p's 16 rows are
// lanes 0..15 of warp p.
//
// Grid: one wave of persistent CTAs (4 per SM at these shared-memory sizes),
// each over a contiguous range of whole tiles; the small-side partial sums are
// one slot per CTA, and the slots past the grid are written as zeros, so the
// fold that follows sees a fixed number of slots.
//
// Shared-memory operand layout: the canonical no-swizzle layout of tcgen05
// descriptors, built of 8 x 16-byte core matrices. A core matrix holds 8 rows
// of 8 BF16 values; LBO is the byte distance between core matrices adjacent in
// the contraction (K) direction and SBO between those adjacent in the M or N
// direction. The count tile (128 groups x KT small groups, KT = Gs padded to
// 32 or 64) is stored once as core matrices (g/8, t/8) and read both as the
// K-major A operand of E (M = g, K = t) and as the MN-major B operand of D2
// (K = g, N = t).
//
// Every wait (mbarrier phases of the copies and of the MMAs) is bounded by a
// globaltimer limit; a CTA that runs out of time records it in an error word
// that the host reads after the within-transform, waits (each wait bounded
// again) for the copies and MMAs it still has in flight, releases its tensor
// memory and returns.
#include "common.cuh"
#include "sweep.cuh"

#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>

namespace fegb {

namespace {

constexpr int UT = 128;        // groups per tile (two threads per group, each with half of its columns)
constexpr int UCP = 16;        // columns per piece block (C <= 16)
constexpr int UNP = 3;         // BF16 pieces per FP32 value
constexpr int UN1 = UNP * UCP; // N of the e-side product
constexpr int UM2 = 64;        // M of the small-side product (rows p * 16 + c; 48 used)
constexpr unsigned long long WAIT_LIMIT_NS = 2000000000ull;  // 2 s per wait

// Tensor-memory columns: two E buffers (tile i in buffer i & 1) and the D2
// accumulator; 128 columns when the small dimension has at most 32 groups.
template <int KT>
struct TmemPlan {
    static constexpr int E0 = 0;
    static constexpr int E1 = UN1;
    static constexpr int D2 = KT <= 32 ? 2 * UN1 : 128;
    static constexpr int COLS = KT <= 32 ? 128 : 256;
};

__device__ int g_umma_error;  // nonzero: a wait of the tensor-core pass ran out of time

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// tcgen05 shared-memory matrix descriptor, no swizzle: start address, LBO and
// SBO in 16-byte units, fixed version bits 0b001 at 46-48.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, the
// majorness of each operand (0 = K-major, 1 = MN-major), N >> 3 and M >> 4.
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N, int a_mn, int b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)a_mn << 15) | ((uint32_t)b_mn << 16) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, int acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// true once the phase of the given parity has completed, false after the time
// limit. Each try suspends the thread in hardware (up to the hint, or until
// the phase completes), so waiting warps take no issue slots from the warps
// that work.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity), "r"(1000000u)
        : "memory");
    if (ok) return true;
    const unsigned long long t0 = globaltimer();
    while (true) {
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\nselp.b32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity), "r"(1000000u)
            : "memory");
        if (ok) return true;
        if (globaltimer() - t0 > WAIT_LIMIT_NS) return false;
    }
}

// bulk global -> shared copy completing on bar (16-byte aligned, size a multiple of 16)
__device__ __forceinline__ void bulk_copy(void* sdst, const void* gsrc, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(sdst)),
                 "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

template <int N>
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[N], int base) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int j = 0; j < 16; ++j) v[base + j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// v = h + m + l with BF16 pieces (exact for finite FP32 v)
__device__ __forceinline__ void split3(float v, __nv_bfloat16& h, __nv_bfloat16& m, __nv_bfloat16& l) {
    h = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(h);
    m = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(m);
    l = __float2bfloat16_rn(r2);
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
    return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// the BF16 roundings of (a, b) packed as pack2 does (a in the low half), one
// paired conversion
__device__ __forceinline__ uint32_t bf16x2_bits(float a, float b) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&v);
}

// split3 of two values at once, the pieces already packed in pairs: the same
// roundings, in paired conversions (the widening back to FP32 is exact)
__device__ __forceinline__ void split3x2(float a, float b, uint32_t& h, uint32_t& m, uint32_t& l) {
    h = bf16x2_bits(a, b);
    const float ra = a - __uint_as_float(h << 16), rb = b - __uint_as_float(h & 0xffff0000u);
    m = bf16x2_bits(ra, rb);
    const float sa = ra - __uint_as_float(m << 16), sb = rb - __uint_as_float(m & 0xffff0000u);
    l = bf16x2_bits(sa, sb);
}

struct UmmaArgs {
    const uint8_t* M;
    long long Ge;
    int Gs;
    const float* pe;
    const float* ps;
    int ld;
    int C;
    long long per;        // groups per CTA (a multiple of UT)
    int nparts;           // partial slots (>= the grid); slots past the grid are zeroed
    double* partials;     // [slot][Gs][C] small-side sums, or null
    float* extra;         // plain form: Ge x C (+)= M ps, or null
    int accumulate;
    const float* sums;    // Schur form: Ge x C, the primary's stream sums
    const int32_t* counts;
    float* table;         // Schur form: u rows (stride ld)
    int bulk_counts;      // counts are 16-byte aligned: copied in bulk with the sums
    uint32_t raw_bytes;   // stage sizes (multiples of 128)
    uint32_t row_bytes;
};

// Shared-memory plan (bytes from the dynamic base): S pieces, two count
// tiles, the U tile, two raw-count stages and two row stages.
struct UmmaSmem {
    uint32_t b1, cnt0, cnt1, u, raw0, raw1, row0, row1, total;
};
__host__ __device__ inline UmmaSmem umma_smem_plan(int KT, uint32_t raw_bytes, uint32_t row_bytes) {
    UmmaSmem s;
    s.b1 = 0;
    s.cnt0 = (uint32_t)(UN1 * KT * 2);
    s.cnt1 = s.cnt0 + (uint32_t)(UT * KT * 2);
    s.u = s.cnt1 + (uint32_t)(UT * KT * 2);
    s.raw0 = s.u + (uint32_t)(UM2 * UT * 2);
    s.raw1 = s.raw0 + raw_bytes;
    s.row0 = s.raw1 + raw_bytes;
    s.row1 = s.row0 + row_bytes;
    s.total = s.row1 + row_bytes;
    return s;
}

// exact float of the byte b of a 32-bit word (2^23 + b as an FP32 bit pattern, minus 2^23)
__device__ __forceinline__ float byte_f32(uint32_t w, uint32_t sel) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, sel)) - 8388608.0f;
}

template <int N>
__device__ __forceinline__ void tmem_ld4(uint32_t taddr, float (&v)[N], int base) {
    uint32_t r0, r1, r2, r3;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(taddr));
    v[base] = __uint_as_float(r0);
    v[base + 1] = __uint_as_float(r1);
    v[base + 2] = __uint_as_float(r2);
    v[base + 3] = __uint_as_float(r3);
}

// Persistent pass: CTA b covers groups [b per, (b + 1) per) tile by tile.
// Two threads per group of the tile (g = tid % 128, half h = tid / 128): each
// converts half of the group's counts and owns 8 of its 16 column slots,
// c = 4h + j and 8 + 4h + j (j < 4), so that each writes whole 8-byte halves
// of the U tile's 16-byte chunks. Per tile i:
//   (a) counts of tile i + 1 -> BF16 count tile; S1; MMA E(i + 1) = counts . S
//   (b) wait E(i); u or the e-side output of tile i; pieces of u / pe -> U; S2;
//       MMA D2 += U' . counts(i)
// with the raw counts fetched three tiles ahead and the rows two tiles ahead
// (bulk copies on per-stage mbarriers), so that copies, E(i + 1) and D2(i)
// overlap the CUDA-core work of tile i.
constexpr int BT = 2 * UT;  // threads per CTA

template <int KT, bool SCHUR>
__global__ void __launch_bounds__(BT, 4) dense_umma_kernel(UmmaArgs a) {
    using TP = TmemPlan<KT>;
    extern __shared__ __align__(1024) unsigned char sm[];
    // 0, 1: raw-count stages; 2, 3: row stages; 4, 5: E buffers; 6: D2
    __shared__ __align__(8) uint64_t bars[7];
    // phases armed (copies or MMA commits issued) and phases waited, per
    // barrier; only the elected thread touches them
    __shared__ uint32_t s_arm[7], s_done[7];
    __shared__ uint32_t tmem_base_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int g = tid & (UT - 1), h = tid / UT;
    const int Gs = a.Gs, C = a.C, ld = a.ld;
    const bool small = a.partials != nullptr;
    const bool need_e = SCHUR || a.extra != nullptr;
    // partial slots past the grid hold zeros
    if (small)
        for (long long slot = (long long)blockIdx.x + gridDim.x; slot < a.nparts; slot += gridDim.x)
            for (int j = tid; j < Gs * C; j += BT) a.partials[slot * Gs * C + j] = 0.0;
    double* const part = small ? a.partials + (long long)blockIdx.x * Gs * C : nullptr;
    const long long g0 = (long long)blockIdx.x * a.per;
    const long long g1 = min(a.Ge, g0 + a.per);
    if (g0 >= g1) {
        if (small)
            for (int j = tid; j < Gs * C; j += BT) part[j] = 0.0;
        return;
    }
    const UmmaSmem L = umma_smem_plan(KT, a.raw_bytes, a.row_bytes);
    constexpr uint32_t CORE_ROW = (uint32_t)(KT / 8) * 128;  // bytes of one 8-group row of count cores
    constexpr uint32_t U_LBO = (uint32_t)(UM2 / 8) * 128;    // bytes between 8-group blocks of the U tile
    const uint32_t sbase = smem_u32(sm);
    const uint32_t sums_bytes = (uint32_t)(((UT * C * 4) + 15) / 16 * 16);
    // this thread's column slots: c = 4h + j (j < 4) and 8 + 4h + (j - 4) (j >= 4)
    auto col_of = [&](int j) { return j < 4 ? 4 * h + j : 8 + 4 * h + (j - 4); };

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_s)),
                     "r"(TP::COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < 7; ++i) {
            mbar_init(&bars[i], 1);
            s_arm[i] = 0;
            s_done[i] = 0;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // U tile zeroed once (rows 48..63 and columns past C stay zero), S pieces
    // (K-major: n = p * 16 + c, k = t)
    for (uint32_t o = tid * 16; o < (uint32_t)(UM2 * UT * 2); o += BT * 16)
        *reinterpret_cast<uint4*>(sm + L.u + o) = make_uint4(0, 0, 0, 0);
    if (need_e) {
        for (int i = tid; i < UN1 * KT; i += BT) {
            const int n = i / KT, t = i - (i / KT) * KT;
            const int p = n / UCP, c = n - p * UCP;
            const float v = (t < Gs && c < C) ? a.ps[(long long)t * ld + c] : 0.0f;
            __nv_bfloat16 hh, mm, ll;
            split3(v, hh, mm, ll);
            const __nv_bfloat16 piece = p == 0 ? hh : (p == 1 ? mm : ll);
            const uint32_t off = (uint32_t)(n / 8) * CORE_ROW + (uint32_t)(t / 8) * 128 + (uint32_t)(n % 8) * 16 +
                                 (uint32_t)(t % 8) * 2;
            *reinterpret_cast<__nv_bfloat16*>(sm + L.b1 + off) = piece;
        }
    }
    fence_async_smem();
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = tmem_base_s;
    const uint32_t t_lane = (uint32_t)((warp & 3) * 32) << 16;
    const int ntiles = (int)((g1 - g0 + UT - 1) / UT);
    auto tile_of = [&](int j) { return g0 + (long long)j * UT; };
    auto full = [&](int j) { return tile_of(j) + UT <= g1; };
    // copy issue (elected thread): a ragged tile completes its stage's phase
    // without copies; its threads read their rows from global memory
    auto issue_raw = [&](int j) {
        uint64_t* bar = &bars[j & 1];
        ++s_arm[j & 1];
        if (!full(j)) {
            mbar_arrive(bar);
            return;
        }
        const uint32_t cb = (uint32_t)(UT * Gs);
        mbar_arrive_tx(bar, cb);
        bulk_copy(sm + ((j & 1) ? L.raw1 : L.raw0), a.M + tile_of(j) * Gs, cb, bar);
    };
    const bool rows_needed = SCHUR || small;
    auto issue_rows = [&](int j) {
        uint64_t* bar = &bars[2 + (j & 1)];
        ++s_arm[2 + (j & 1)];
        if (!full(j) || !rows_needed) {
            mbar_arrive(bar);
            return;
        }
        unsigned char* row = sm + ((j & 1) ? L.row1 : L.row0);
        if (SCHUR) {
            const uint32_t cbytes = a.bulk_counts ? (uint32_t)(UT * 4) : 0u;
            mbar_arrive_tx(bar, (uint32_t)(UT * C * 4) + cbytes);
            bulk_copy(row, a.sums + tile_of(j) * C, (uint32_t)(UT * C * 4), bar);
            if (cbytes) bulk_copy(row + sums_bytes, a.counts + tile_of(j), cbytes, bar);
        } else {
            mbar_arrive_tx(bar, (uint32_t)(UT * ld * 4));
            bulk_copy(row, a.pe + tile_of(j) * ld, (uint32_t)(UT * ld * 4), bar);
        }
    };
    // waits for the next phase of barrier b (phases complete in issue order,
    // so the parity of the next one is the count of phases waited so far)
    auto bar_wait = [&](int b) -> bool {
        const bool r = mbar_wait(&bars[b], s_done[b] & 1u);
        if (r) ++s_done[b];
        return r;
    };
    bool failed = false;
    // counts of tile j -> count tile j & 1 (BF16 core matrices (g/8, t/8), row
    // g % 8); half h converts the core blocks [h KT/16, (h + 1) KT/16)
    auto convert = [&](int j) -> bool {
        const long long tile = tile_of(j);
        const int nt = (int)min((long long)UT, g1 - tile);
        const bool mine = g < nt;
        const unsigned char* src = full(j) ? sm + ((j & 1) ? L.raw1 : L.raw0) + g * Gs : a.M + (tile + g) * Gs;
        const uint32_t cnt_off = (j & 1) ? L.cnt1 : L.cnt0;
#pragma unroll
        for (int tq = 0; tq < KT / 16; ++tq) {
            const int tb = h * (KT / 16) + tq;
            uint32_t w[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int t0 = tb * 8 + 2 * q;
                uint32_t pair = 0;
                if (mine && t0 < Gs) pair = src[t0] | ((t0 + 1 < Gs ? (uint32_t)src[t0 + 1] : 0u) << 8);
                const float x0 = byte_f32(pair, 0x7540u), x1 = byte_f32(pair, 0x7541u);
                w[q] = bf16x2_bits(x0, x1);
            }
            *reinterpret_cast<uint4*>(sm + cnt_off + (uint32_t)(g / 8) * CORE_ROW + (uint32_t)tb * 128 +
                                      (uint32_t)(g % 8) * 16) = make_uint4(w[0], w[1], w[2], w[3]);
        }
        fence_async_smem();
        return true;
    };
    auto issue_e = [&](int j) {
        const uint32_t cnt_off = (j & 1) ? L.cnt1 : L.cnt0;
        const uint32_t id = umma_idesc(UT, UN1, 0, 0);
        const uint32_t ecol = (j & 1) ? TP::E1 : TP::E0;
#pragma unroll
        for (int s = 0; s < KT / 16; ++s)
            umma_bf16(tmem + ecol, umma_desc(sbase + cnt_off + s * 256, 128, CORE_ROW),
                      umma_desc(sbase + L.b1 + s * 256, 128, CORE_ROW), id, s > 0);
        ++s_arm[4 + (j & 1)];
        umma_commit(&bars[4 + (j & 1)]);
    };

    // prologue: copies of tiles 0..1 (raw and rows); counts of tile 0 and its E
    if (tid == 0) {
        for (int j = 0; j < 2 && j < ntiles; ++j) issue_raw(j);
        for (int j = 0; j < 2 && j < ntiles; ++j) issue_rows(j);
    }
    // one thread waits on each mbarrier and the block follows it at a barrier
    // (the waiting thread's observation of the phase, then bar.sync, orders
    // the copies' and the MMAs' results before every thread's reads)
    bool ok = tid != 0 || bar_wait(0);
    if (__syncthreads_or(!ok)) failed = true;
    if (!failed) convert(0);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (!failed && tid == 0) {
        if (need_e) issue_e(0);
        if (ntiles > 2) issue_raw(2);  // raw stage 0 was consumed by the conversion of tile 0
    }

    int d2_waited = -1;  // the last tile whose D2 MMA is known complete
    for (int i = 0; i < ntiles && !failed; ++i) {
        const long long tile = tile_of(i);
        const int nt = (int)min((long long)UT, g1 - tile);
        const bool mine = g < nt;
        // (a) counts of tile i + 1 (its count tile was read by the MMAs of tile i - 1)
        ok = true;
        if (i + 1 < ntiles) {
            if (tid == 0) {
                if (small && i >= 1) ok = bar_wait(6);
                ok = ok && bar_wait((i + 1) & 1);
            }
            if (small && i >= 1) d2_waited = i - 1;
            if (__syncthreads_or(!ok)) {
                failed = true;
                break;
            }
            convert(i + 1);
        }
        // (b) this tile's rows and E(i), waited before the one barrier that
        // also publishes the counts of tile i + 1 converted above
        ok = tid != 0 || bar_wait(2 + (i & 1));
        if (tid == 0 && ok && need_e) ok = bar_wait(4 + (i & 1));
        fence_before_sync();
        if (__syncthreads_or(!ok)) {  // S1
            failed = true;
            break;
        }
        fence_after_sync();
        if (tid == 0 && i + 1 < ntiles) {
            if (need_e) issue_e(i + 1);
            if (i + 3 < ntiles) issue_raw(i + 3);  // raw stage (i + 1) & 1 was just consumed
        }
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) v[j] = 0.0f;
        int n_g = 0;
        const float* srow = reinterpret_cast<const float*>(sm + ((i & 1) ? L.row1 : L.row0));
        if (mine) {
            const bool f = full(i);
            if (SCHUR) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int c = col_of(j);
                    if (c < C) v[j] = f ? srow[g * C + c] : a.sums[(tile + g) * C + c];
                }
                n_g = (f && a.bulk_counts) ? reinterpret_cast<const int32_t*>(sm + ((i & 1) ? L.row1 : L.row0) +
                                                                             sums_bytes)[g]
                                           : a.counts[tile + g];
            } else if (small) {
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int c = col_of(j);
                    if (c < C) v[j] = f ? srow[g * ld + c] : a.pe[(tile + g) * ld + c];
                }
            }
        }
        if (need_e) {
            // E columns of this thread's slots: piece p at p * 16 + c
            float e[24];
            const uint32_t ecol = (i & 1) ? TP::E1 : TP::E0;
#pragma unroll
            for (int p = 0; p < UNP; ++p) {
                tmem_ld4(tmem + t_lane + ecol + p * UCP + 4 * h, e, p * 8);
                tmem_ld4(tmem + t_lane + ecol + p * UCP + 8 + 4 * h, e, p * 8 + 4);
            }
            tmem_wait_ld();
            if (SCHUR) {
                const float rn = n_g > 0 ? 1.0f / (float)n_g : 0.0f;
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    if (col_of(j) < C) v[j] = n_g > 0 ? (v[j] - ((e[16 + j] + e[8 + j]) + e[j])) * rn : 0.0f;
                if (mine) {
                    // this thread's two 16-byte column quads of the padded row
                    // (zeros past C): whole 32-byte sectors are written, so
                    // none has to be read back to merge a partial write
                    float* trow = a.table + (tile + g) * ld + 4 * h;
                    if (4 * h + 4 <= ld) *reinterpret_cast<float4*>(trow) = make_float4(v[0], v[1], v[2], v[3]);
                    if (8 + 4 * h + 4 <= ld)
                        *reinterpret_cast<float4*>(trow + 8) = make_float4(v[4], v[5], v[6], v[7]);
                }
            } else if (mine) {
                float* xr = a.extra + (tile + g) * C;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const int c = col_of(j);
                    if (c < C) {
                        const float ec = (e[16 + j] + e[8 + j]) + e[j];
                        xr[c] = a.accumulate ? xr[c] + ec : ec;
                    }
                }
            }
        }
        if (small) {
            // the U tile was read by D2(i - 1)
            if (i >= 1 && d2_waited < i - 1) {
                ok = tid != 0 || bar_wait(6);
                d2_waited = i - 1;
                if (__syncthreads_or(!ok)) {
                    failed = true;
                    break;
                }
            }
            // U pieces, MN-major: row m = p * 16 + c, core (m/8, g/8), row g % 8;
            // this thread's 4 columns of each 8-column block are the chunk's half h
#pragma unroll
            for (int hb = 0; hb < 2; ++hb) {
                if (hb * 8 >= C) break;
                uint32_t w[UNP][2];
#pragma unroll
                for (int q = 0; q < 2; ++q)
                    split3x2(v[hb * 4 + 2 * q], v[hb * 4 + 2 * q + 1], w[0][q], w[1][q], w[2][q]);
#pragma unroll
                for (int p = 0; p < UNP; ++p) {
                    const uint32_t mb = (uint32_t)(p * 2 + hb);
                    *reinterpret_cast<uint2*>(sm + L.u + mb * 128 + (uint32_t)(g / 8) * U_LBO + (uint32_t)(g % 8) * 16 +
                                              (uint32_t)h * 8) = make_uint2(w[p][0], w[p][1]);
                }
            }
            fence_async_smem();
        }
        fence_before_sync();
        __syncthreads();  // S2
        fence_after_sync();
        if (tid == 0) {
            if (small) {
                const uint32_t id = umma_idesc(UM2, KT, 1, 1);
                const uint32_t cnt_off = (i & 1) ? L.cnt1 : L.cnt0;
#pragma unroll
                for (int s = 0; s < UT / 16; ++s)
                    umma_bf16(tmem + TP::D2, umma_desc(sbase + L.u + s * 2 * U_LBO, U_LBO, 128),
                              umma_desc(sbase + cnt_off + s * 2 * CORE_ROW, CORE_ROW, 128), id,
                              (i > 0 || s > 0) ? 1 : 0);
                ++s_arm[6];
                umma_commit(&bars[6]);
            }
            if (i + 2 < ntiles) issue_rows(i + 2);  // row stage i & 1 was read before S2
        }
    }
    if (failed) {
        if (tid == 0) atomicExch(&g_umma_error, 1);
    } else if (small) {
        const bool okf = tid != 0 || bar_wait(6);
        if (__syncthreads_or(!okf)) {
            failed = true;
            if (tid == 0) atomicExch(&g_umma_error, 1);
        } else {
            fence_after_sync();
            // D2 row m = p * 16 + c sits in TMEM lane p * 32 + c (M = 64 layout):
            // warps 0..2, lanes 0..15 -> shared [m][t] floats over the U tile
            float* d2s = reinterpret_cast<float*>(sm + L.u);
            __syncthreads();  // the U tile is free (D2 complete); reuse it for the readback
            if (warp < 4) {
#pragma unroll
                for (int c0 = 0; c0 < KT; c0 += 16) {
                    float d[16];
                    tmem_ld16(tmem + t_lane + TP::D2 + c0, d, 0);
                    tmem_wait_ld();
                    if (warp < UNP && lane < UCP)
#pragma unroll
                        for (int t = 0; t < 16; ++t) d2s[(warp * UCP + lane) * KT + c0 + t] = d[t];
                }
            }
            __syncthreads();
            for (int j = tid; j < Gs * C; j += BT) {
                const int t = j / C, c = j - t * C;
                part[j] = ((double)d2s[(32 + c) * KT + t] + (double)d2s[(16 + c) * KT + t]) + (double)d2s[c * KT + t];
            }
        }
    }
    // after a wait ran out of time: let every copy and MMA still in flight
    // land (each wait bounded again) before the shared memory and the tensor
    // memory are given back
    if (failed && tid == 0)
        for (int b = 0; b < 7; ++b)
            while (s_done[b] < s_arm[b] && bar_wait(b)) {
            }
    fence_before_sync();
    __syncthreads();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TP::COLS));
}

template <int KT, bool SCHUR>
int launch_umma(UmmaArgs a, cudaStream_t s) {
    const UmmaSmem L = umma_smem_plan(KT, a.raw_bytes, a.row_bytes);
    // the largest shared-memory carveout, so that four CTAs fit on an SM (the
    // default carveout leaves room for one)
    static const cudaError_t attr = [] {
        cudaError_t e = cudaFuncSetAttribute(dense_umma_kernel<KT, SCHUR>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             200 * 1024);
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(dense_umma_kernel<KT, SCHUR>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared);
        return e;
    }();
    if (attr != cudaSuccess) return set_cuda_error(attr, "dense tensor-core pass attr");
    // one wave of persistent CTAs (at most the partial slots), each over a
    // contiguous range of whole tiles. Resident CTAs per SM for this
    // shared-memory size are cached per size, so the calls made during a
    // stream capture make no runtime queries.
    static thread_local uint32_t cached_bytes = 0;
    static thread_local int cached_sms = 0, cached_occ = 0;
    if (cached_bytes != L.total) {
        // CTAs per SM from the SM's shared memory (the occupancy API's answer
        // does not follow the carveout set above), the per-block reserve and
        // the kernel's static shared memory
        int dev = 0, smem_sm = 0, reserved = 0;
        FEGB_CUDA(cudaGetDevice(&dev), "cudaGetDevice");
        FEGB_CUDA(cudaDeviceGetAttribute(&cached_sms, cudaDevAttrMultiProcessorCount, dev), "SM count");
        FEGB_CUDA(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev), "SM smem");
        FEGB_CUDA(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev), "smem reserve");
        cudaFuncAttributes fa{};
        FEGB_CUDA(cudaFuncGetAttributes(&fa, dense_umma_kernel<KT, SCHUR>), "kernel attributes");
        const size_t per_cta = (size_t)L.total + fa.sharedSizeBytes + (size_t)reserved;
        cached_occ = (int)std::max<size_t>(1, (size_t)smem_sm / per_cta);
        cached_bytes = L.total;
    }
    // tensor memory per SM: 512 columns
    const int occ = std::max(1, std::min(cached_occ, 512 / TmemPlan<KT>::COLS));
    const long long tiles = (a.Ge + UT - 1) / UT;
    int grid = (int)std::min<long long>({(long long)a.nparts, (long long)occ * cached_sms, tiles});
    grid = std::max(grid, 1);
    const long long tiles_per = (tiles + grid - 1) / grid;
    a.per = tiles_per * UT;
    dense_umma_kernel<KT, SCHUR><<<grid, BT, L.total, s>>>(a);
    FEGB_LAUNCH_CHECK("dense small-G pair product (tcgen05)");
    return 0;
}

bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

}  // namespace

int launch_dense_pair_umma(const uint8_t* M, long long Ge, int Gs, const float* pe, const float* ps, int ld, int C,
                           double* partials, float* extra, int accumulate, const DenseSchur<float>& sch,
                           cudaStream_t s, bool* launched) {
    *launched = false;
    const bool schur = sch.sums != nullptr;
    if (Ge <= 0 || Gs <= 0 || Gs > 64 || C <= 0 || C > UCP || ld < C || ld % 4 != 0) return 0;
    if (!aligned16(M) || !aligned16(ps) || (pe && !aligned16(pe)) ||
        (schur && (!aligned16(sch.sums) || !aligned16(sch.table))))
        return 0;
    if (!schur && partials && !pe) return 0;
    UmmaArgs a{};
    a.M = M;
    a.Ge = Ge;
    a.Gs = Gs;
    a.pe = pe;
    a.ps = ps;
    a.ld = ld;
    a.C = C;
    a.nparts = dense_chunks(Ge);
    a.partials = partials;
    a.extra = schur ? nullptr : extra;
    a.accumulate = accumulate;
    a.sums = sch.sums;
    a.counts = sch.counts;
    a.table = sch.table;
    a.bulk_counts = schur && aligned16(sch.counts) ? 1 : 0;
    a.raw_bytes = (uint32_t)((UT * Gs + 127) / 128 * 128);
    const uint32_t rb = schur ? (uint32_t)(((UT * C * 4 + 15) / 16) * 16 + UT * 4) : (uint32_t)(UT * ld * 4);
    a.row_bytes = (rb + 127) / 128 * 128;
    *launched = true;
    if (Gs <= 32) return schur ? launch_umma<32, true>(a, s) : launch_umma<32, false>(a, s);
    return schur ? launch_umma<64, true>(a, s) : launch_umma<64, false>(a, s);
}

int dense_umma_error(int* flag, bool reset, cudaStream_t s) {
    void* p = nullptr;
    FEGB_CUDA(cudaGetSymbolAddress(&p, g_umma_error), "tensor-core pass error word");
    int h = 0;
    FEGB_CUDA(cudaMemcpyAsync(&h, p, sizeof(int), cudaMemcpyDeviceToHost, s), "tensor-core pass error read");
    FEGB_CUDA(cudaStreamSynchronize(s), "tensor-core pass error sync");
    if (reset && h) FEGB_CUDA(cudaMemsetAsync(p, 0, sizeof(int), s), "tensor-core pass error reset");
    *flag = h;
    return 0;
}

}  // namespace fegb
