// The fe_gpu .bin dataset read straight into device memory.
//
// The reference loads the file on the host (load_dataset_from_file,
// src/io/fe_data_io.f90:23-389): values widened to FP64 and the FE ids
// interleaved into fe_ids(n_fe, n) before the upload (7.8 s of its 150M-row
// run). The file stores every column contiguously (y, W columns, Z columns,
// one id array per FE dimension, cluster ids, weights, then an optional META
// names block), which is already the device layout: here reader threads pread
// fixed chunks into pinned buffers and copy them asynchronously to their
// final place; FP32 files are widened to FP64 by a kernel on the device.
#include "common.cuh"

#include <fcntl.h>
#include <unistd.h>
#include <sys/stat.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fegb.h"

namespace fegb {
namespace {

constexpr long long HEADER_NEW = 8 + 5 * 4;  // N (int64), K, L, n_fe, has_cluster, has_weights
constexpr long long HEADER_OLD = 8 + 4 * 4;  // N, K, n_fe, has_cluster, has_weights
constexpr size_t LOAD_CHUNK = 32u << 20;     // bytes per pread / copy
constexpr int LOAD_THREADS = 8;

// compute_data_bytes (src/io/fe_data_io.f90:331-349)
long long data_bytes(long long n, int k, int l, int n_fe, bool hc, bool hw, int vb) {
    long long t = n * (1 + (long long)k) * vb;
    if (l > 0) t += n * (long long)l * vb;
    if (hw) t += n * vb;
    t += (long long)n_fe * n * 4;
    if (hc) t += n * 4;
    return t;
}

struct Layout {
    long long n = 0;
    int k = 0, l = 0, n_fe = 0;
    bool hc = false, hw = false;
    int precision = 0;       // 0 FP64, 1 FP32
    long long data_off = 0;  // first value byte
    long long meta_off = 0;  // META block (0 = none)
};

int read_exact(int fd, void* buf, size_t bytes, long long off) {
    char* p = static_cast<char*>(buf);
    while (bytes > 0) {
        ssize_t r = pread(fd, p, bytes, (off_t)off);
        if (r <= 0) return 1;
        p += r;
        bytes -= (size_t)r;
        off += r;
    }
    return 0;
}

// Header detection of src/io/fe_data_io.f90:78-202: the new (28-byte) or old
// (24-byte) header is the one whose implied size matches the file, FP64 or
// FP32 values with or without the trailing precision flag; otherwise the new
// header with a precision flag and trailing metadata.
int parse_header(int fd, long long size, Layout* L) {
    unsigned char h[HEADER_NEW + 4];
    std::memset(h, 0, sizeof(h));
    if (size < HEADER_OLD) return set_error("File too small to contain required header");
    if (read_exact(fd, h, (size_t)std::min<long long>(size, (long long)sizeof(h)), 0))
        return set_error("IO error while reading the header");
    long long n;
    int32_t t[5];
    std::memcpy(&n, h, 8);
    std::memcpy(t, h + 8, 20);
    const int k = t[0];
    if (n <= 0) return set_error("N must be positive");
    if (k < 0) return set_error("K must be non-negative");
    auto totals = [&](long long base, int l, int nfe, bool hc, bool hw, long long* t64, long long* t32) {
        if (l < 0 || nfe < 0) {
            *t64 = *t32 = -1;
            return;
        }
        *t64 = base + data_bytes(n, k, l, nfe, hc, hw, 8);
        *t32 = base + data_bytes(n, k, l, nfe, hc, hw, 4);
    };
    long long n64, n32, o64, o32;
    totals(HEADER_NEW, t[1], t[2], t[3] != 0, t[4] != 0, &n64, &n32);
    totals(HEADER_OLD, 0, t[1], t[2] != 0, t[3] != 0, &o64, &o32);
    bool use_new = size == n64 || size == n32 || size == n64 + 4 || size == n32 + 4;
    const bool use_old = size == o64 || size == o32 || size == o64 + 4 || size == o32 + 4;
    if (!use_new && !use_old) use_new = true;
    long long base;
    L->n = n;
    L->k = k;
    if (use_new) {
        base = HEADER_NEW;
        L->l = t[1];
        L->n_fe = t[2];
        L->hc = t[3] != 0;
        L->hw = t[4] != 0;
        if (L->l < 0) return set_error("L must be non-negative");
    } else {
        base = HEADER_OLD;
        L->l = 0;
        L->n_fe = t[1];
        L->hc = t[2] != 0;
        L->hw = t[3] != 0;
    }
    if (L->n_fe < 0) return set_error("n_fe must be non-negative");
    const long long t64 = base + data_bytes(n, k, L->l, L->n_fe, L->hc, L->hw, 8);
    const long long t32 = base + data_bytes(n, k, L->l, L->n_fe, L->hc, L->hw, 4);
    if (size == t64) {
        L->precision = 0;
        L->data_off = base;
        return 0;
    }
    if (size == t32) {
        L->precision = 1;
        L->data_off = base;
        return 0;
    }
    if (size < base + 4) return set_error("File size does not match header metadata");
    int32_t flag;
    std::memcpy(&flag, h + base, 4);
    long long expected;
    if (flag == 0)
        expected = base + 4 + data_bytes(n, k, L->l, L->n_fe, L->hc, L->hw, 8);
    else if (flag == 1)
        expected = base + 4 + data_bytes(n, k, L->l, L->n_fe, L->hc, L->hw, 4);
    else
        return set_error("Unsupported precision flag value: %d", flag);
    if (size < expected) return set_error("File size does not match header metadata for declared precision");
    L->precision = flag;
    L->data_off = base + 4;
    L->meta_off = size > expected ? expected : 0;
    return 0;
}

__global__ void widen_kernel(const float* __restrict__ src, long long n, double* __restrict__ dst) {
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long st = (long long)gridDim.x * blockDim.x;
    for (; i < n; i += st) dst[i] = (double)src[i];
}

// One section of the file copied to a device destination: vb bytes per
// element on disk; FP32 value sections are widened to FP64.
struct Section {
    long long file_off;
    long long count;  // elements
    int vb;           // bytes per element on disk
    bool widen;       // FP32 -> FP64
    void* dst;
};

struct Job {
    int section;
    long long first;  // first element of the chunk
    long long count;
};

}  // namespace

int load_bin(const char* path, fegb_dataset* out) {
    auto t0 = std::chrono::steady_clock::now();
    std::memset(out, 0, sizeof(*out));
    int fd = open(path, O_RDONLY);
    if (fd < 0) return set_error("Dataset file not found: %s", path);
    struct stat st;
    if (fstat(fd, &st) != 0) {
        close(fd);
        return set_error("cannot stat %s", path);
    }
    Layout L;
    int rc = parse_header(fd, (long long)st.st_size, &L);
    if (rc) {
        close(fd);
        return rc;
    }
    if (L.n > 0x7fffffffLL) {
        close(fd);
        return set_error("n=%lld exceeds the int32 row range", L.n);
    }
    const int vb = L.precision == 1 ? 4 : 8;
    const long long n = L.n;
    const long long nv = n * (1 + (long long)L.k + L.l);
    // device blocks: values (y | W | Z), ids (dimension-major), cluster, weights
    double* vals = nullptr;
    int32_t* ids = nullptr;
    int32_t* cl = nullptr;
    double* wts = nullptr;
    auto cleanup = [&]() {
        if (vals) cudaFree(vals);
        if (ids) cudaFree(ids);
        if (cl) cudaFree(cl);
        if (wts) cudaFree(wts);
        close(fd);
    };
    cudaError_t e = cudaMalloc(&vals, sizeof(double) * (size_t)nv);
    if (e == cudaSuccess && L.n_fe > 0) e = cudaMalloc(&ids, sizeof(int32_t) * (size_t)n * L.n_fe);
    if (e == cudaSuccess && L.hc) e = cudaMalloc(&cl, sizeof(int32_t) * (size_t)n);
    if (e == cudaSuccess && L.hw) e = cudaMalloc(&wts, sizeof(double) * (size_t)n);
    if (e != cudaSuccess) {
        cleanup();
        return set_cuda_error(e, "dataset device allocation");
    }
    std::vector<Section> secs;
    long long off = L.data_off;
    secs.push_back({off, nv, vb, vb == 4, vals});
    off += nv * vb;
    if (L.n_fe > 0) secs.push_back({off, n * L.n_fe, 4, false, ids});
    off += n * L.n_fe * 4LL;
    if (L.hc) secs.push_back({off, n, 4, false, cl});
    off += L.hc ? n * 4 : 0;
    if (L.hw) secs.push_back({off, n, vb, vb == 4, wts});
    std::vector<Job> jobs;
    for (int si = 0; si < (int)secs.size(); ++si) {
        const long long per = (long long)(LOAD_CHUNK / secs[si].vb);
        for (long long f = 0; f < secs[si].count; f += per)
            jobs.push_back({si, f, std::min(per, secs[si].count - f)});
    }
    std::atomic<int> next{0};
    std::mutex mu;
    std::string err;
    auto worker = [&]() {
        cudaStream_t s = nullptr;
        void* pin[2] = {nullptr, nullptr};
        float* stage[2] = {nullptr, nullptr};
        cudaEvent_t done[2] = {nullptr, nullptr};
        auto fail = [&](const std::string& m) {
            std::lock_guard<std::mutex> g(mu);
            if (err.empty()) err = m;
        };
        if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return fail("loader stream");
        bool ok = true;
        for (int b = 0; b < 2 && ok; ++b) {
            ok = cudaHostAlloc(&pin[b], LOAD_CHUNK, cudaHostAllocDefault) == cudaSuccess &&
                 cudaMalloc(&stage[b], LOAD_CHUNK) == cudaSuccess &&
                 cudaEventCreateWithFlags(&done[b], cudaEventDisableTiming) == cudaSuccess;
        }
        if (!ok) fail("loader buffers");
        int b = 0;
        for (int j = next++; ok && j < (int)jobs.size(); j = next++) {
            {
                std::lock_guard<std::mutex> g(mu);
                if (!err.empty()) break;
            }
            const Job& J = jobs[j];
            const Section& S = secs[J.section];
            // the buffer's previous copy must be done before it is refilled
            if (cudaEventSynchronize(done[b]) != cudaSuccess) {
                fail("loader copy");
                break;
            }
            const size_t bytes = (size_t)J.count * S.vb;
            if (read_exact(fd, pin[b], bytes, S.file_off + J.first * S.vb)) {
                fail("IO error while reading data block");
                break;
            }
            cudaError_t ce;
            if (S.widen) {
                ce = cudaMemcpyAsync(stage[b], pin[b], bytes, cudaMemcpyHostToDevice, s);
                if (ce == cudaSuccess) {
                    widen_kernel<<<grid_stride_blocks(J.count, 256), 256, 0, s>>>(
                        stage[b], J.count, static_cast<double*>(S.dst) + J.first);
                    count_launch();
                    ce = cudaPeekAtLastError();
                }
            } else {
                ce = cudaMemcpyAsync(static_cast<char*>(S.dst) + (size_t)J.first * S.vb, pin[b], bytes,
                                     cudaMemcpyHostToDevice, s);
            }
            if (ce == cudaSuccess) ce = cudaEventRecord(done[b], s);
            if (ce != cudaSuccess) {
                fail(std::string("loader copy: ") + cudaGetErrorString(ce));
                break;
            }
            b ^= 1;
        }
        cudaStreamSynchronize(s);
        for (int i = 0; i < 2; ++i) {
            if (pin[i]) cudaFreeHost(pin[i]);
            if (stage[i]) cudaFree(stage[i]);
            if (done[i]) cudaEventDestroy(done[i]);
        }
        cudaStreamDestroy(s);
    };
    const int nt = (int)std::min<size_t>(LOAD_THREADS, std::max<size_t>(1, jobs.size()));
    std::vector<std::thread> pool;
    for (int i = 1; i < nt; ++i) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    if (!err.empty()) {
        cleanup();
        return set_error("%s", err.c_str());
    }
    close(fd);
    out->n = n;
    out->k = L.k;
    out->l = L.l;
    out->n_fe = L.n_fe;
    out->has_cluster = L.hc ? 1 : 0;
    out->has_weights = L.hw ? 1 : 0;
    out->precision_flag = L.precision;
    out->metadata_offset = L.meta_off;
    out->y = vals;
    out->W = L.k > 0 ? vals + n : nullptr;
    out->Z = L.l > 0 ? vals + n * (1 + (long long)L.k) : nullptr;
    out->fe_ids = ids;
    out->cluster = cl;
    out->weights = wts;
    out->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return set_ok();
}

}  // namespace fegb

extern "C" int fegb_load_bin(const char* path, fegb_dataset* out) {
    if (!path || !out) return fegb::set_error("fegb_load_bin: null argument");
    return fegb::load_bin(path, out);
}

extern "C" int fegb_free_dataset(fegb_dataset* ds) {
    if (!ds) return fegb::set_ok();
    if (ds->y) cudaFree(ds->y);
    if (ds->fe_ids) cudaFree(ds->fe_ids);
    if (ds->cluster) cudaFree(ds->cluster);
    if (ds->weights) cudaFree(ds->weights);
    std::memset(ds, 0, sizeof(*ds));
    return fegb::set_ok();
}
