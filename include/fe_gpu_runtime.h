/*
 * fe_gpu_runtime.h -- kernel-level C ABI of libfegb.so.
 *
 * Drop-in for the reference's src/gpu/fe_gpu_runtime.h (lines 14-131): every
 * symbol below keeps the reference's name, argument list, argument meaning and
 * status convention, so the reference's Fortran iso_c_binding interface
 * blocks (src/gpu/fe_gpu_runtime.f90:59-154, src/gpu/fe_gpu_demean.f90:14-59,
 * src/gpu/fe_gpu_linalg.f90:18-90, src/core/fe_cluster_utils.f90:9-23) bind to
 * this library unchanged. Differences in behaviour, all deliberate:
 *   - no cuBLAS, Thrust or CUB: every routine is a kernel of this library;
 *   - no floating-point atomics: group sums, cluster scores, dot products and
 *     cross products use a fixed summation order, so results are identical
 *     from run to run;
 *   - fe_build_cluster_ids, the reference's CPU builder
 *     (src/core/cluster_id_builder.c:271-278), runs on the device and returns
 *     the same ids.
 * Status: 0 on success, otherwise a CUDA error code or 1; the message is kept
 * per host thread and read with fe_gpu_runtime_get_last_error.
 * All calls are synchronous with respect to the host, as in the reference.
 */
#ifndef FE_GPU_RUNTIME_H
#define FE_GPU_RUNTIME_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#ifndef FE_GPU_NAME_LEN
#define FE_GPU_NAME_LEN 256
#endif

/* src/gpu/fe_gpu_runtime.h:14-21 */
typedef struct {
    int device_id;
    size_t total_global_mem;
    int multiprocessor_count;
    int major;
    int minor;
    char name[FE_GPU_NAME_LEN];
} fe_gpu_device_info;

/* runtime: src/gpu/fe_gpu_runtime.h:23-33 */
int fe_gpu_runtime_is_available(void);                 /* 0 when a CUDA device is present */
int fe_gpu_runtime_init(int device_id, fe_gpu_device_info* info);
int fe_gpu_runtime_shutdown(void);
int fe_gpu_runtime_malloc(void** ptr, size_t bytes);
int fe_gpu_runtime_free(void* ptr);
int fe_gpu_runtime_memcpy_htod(void* dst, const void* src, size_t bytes);
int fe_gpu_runtime_memcpy_dtoh(void* dst, const void* src, size_t bytes);
int fe_gpu_runtime_memcpy_dtod(void* dst, const void* src, size_t bytes);
int fe_gpu_runtime_memset(void* ptr, int value, size_t bytes);
int fe_gpu_runtime_get_last_error(char* buffer, size_t length);
int fe_gpu_runtime_clear_error(void);

/* linear algebra: src/gpu/fe_gpu_runtime.h:35-62 (column-major, FP64) */
int fe_gpu_linalg_init(void);
int fe_gpu_linalg_shutdown(void);
/* Q (upper triangle, n_cols x n_cols, ld n_cols) = alpha W^T W + beta Q */
int fe_gpu_syrk(int n_rows, int n_cols, double alpha, const double* W, int ldW, double beta, double* Q);
/* Same result as fe_gpu_syrk without allocating device memory (no
 * counterpart in the reference). For callers that cannot let a library
 * allocate while they run -- a host that owns every device buffer through its
 * own allocator and budget, or a section that must not touch the allocator.
 * Its partial sums live in a fixed 642 KB device array held by every GPU that
 * loads the library; n_cols is limited to 32 (larger requests return a
 * nonzero status), and ldW below max(1, n_rows) is rejected as in
 * fe_gpu_syrk. The first call on each device (with that device current)
 * looks up the array's address and records the device's context; a call in a
 * new context (after cudaDeviceReset) looks it up again. Make the first call,
 * and the first after a reset, before any stream capture. All calls share the
 * array: calls that overlap on the GPU race. */
int fe_gpu_syrk_noalloc(int n_rows, int n_cols, double alpha, const double* W, int ldW, double beta, double* Q);
/* b = alpha W^T y + beta b */
int fe_gpu_gemv(int n_rows, int n_cols, double alpha, const double* W, int ldW, const double* y, double beta,
                double* b);
/* residual = y - W beta (left untouched when n_cols == 0, as in the reference) */
int fe_gpu_residual(int n_rows, int n_cols, const double* W, int ldW, const double* beta, const double* y,
                    double* residual);
/* *result (host) = x . y */
int fe_gpu_dot(int n_rows, const double* x, const double* y, double* result);
/* C = alpha op(A) op(B) + beta C; trans 'N'/'n' = no transpose, anything else = transpose */
int fe_gpu_gemm(char transA, char transB, int m, int n, int k, double alpha, const double* A, int ldA,
                const double* B, int ldB, double beta, double* C, int ldC);

/* clustering: src/gpu/fe_gpu_runtime.h:63-75 */
/* scores[c + j*n_clusters] += sum over rows i with cluster_ids[i] = c+1 of residual[i] * W[i + j*ldW] */
int fe_gpu_cluster_scores(const double* residual, const double* W, const int* cluster_ids, int n_rows, int n_cols,
                          int ldW, int n_clusters, double* scores);
/* meat (upper, n_cols x n_cols) = scores^T scores */
int fe_gpu_cluster_meat(int n_clusters, int n_cols, const double* scores, int ldScores, double* meat);

/* demeaning: src/gpu/fe_gpu_runtime.h:77-112. Group tables are row-major by
 * group (g * n_cols + j); ids are 1-based, ids <= 0 are skipped. */
int fe_gpu_fe_accumulate(const double* y, const double* W, const double* Z, const int* fe_ids, size_t n_obs,
                         int n_groups, int n_reg, int n_inst, size_t leading_dim, double* group_sum_y,
                         double* group_sum_W, double* group_sum_Z, int* group_counts);
int fe_gpu_fe_compute_means(double* group_sum_y, double* group_sum_W, double* group_sum_Z, const int* group_counts,
                            int n_groups, int n_reg, int n_inst);
int fe_gpu_fe_subtract(double* y, double* W, double* Z, const int* fe_ids, size_t n_obs, int n_reg, int n_inst,
                       size_t leading_dim, const double* group_mean_y, const double* group_mean_W,
                       const double* group_mean_Z, double relaxation);
/* mixed = prev + relaxation (mean - prev); prev = mean = mixed */
int fe_gpu_mix_means(double* mean, double* prev, size_t n, double relaxation);
int fe_gpu_axpy(int n, double alpha, const double* x, double* y);

/* utilities: src/gpu/fe_gpu_runtime.h:114-131 */
int fe_gpu_absmax(const double* data, long long n, double* out);
/* indices: host array of 1-based source columns */
int fe_gpu_copy_columns(const double* src, int ld_src, const int* indices, int n_indices, int n_rows, double* dst,
                        int ld_dst, int dest_offset);
/* fe_ptrs/strides: host arrays; out_ids: device; *out_n_clusters: host */
int fe_gpu_build_multi_cluster_ids(const void* const* fe_ptrs, const unsigned long long* strides, int n_dims,
                                   long long n_obs, int* out_ids, int* out_n_clusters);

/* src/core/cluster_id_builder.c:271-278 -- host arrays in, host ids out.
 * fe_ids: n_fe x n_obs with the dimension index fastest (ld_fe = n_fe).
 * Returns 0, or the reference's codes: 1 null argument, 2 bad ld/n, 3 bad
 * subset length, 4 bad dimension index, 6 allocation failure. */
int fe_build_cluster_ids(const int32_t* fe_ids, int ld_fe, long long n_obs, const int32_t* subset_dims,
                         const int32_t* subset_sizes, int subset_len, int32_t* out_ids, int32_t* out_n_clusters);

#ifdef __cplusplus
}
#endif

#endif /* FE_GPU_RUNTIME_H */
