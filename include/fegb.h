/*
 * fegb.h -- whole-fit C ABI of the GB300 estimation library (libfegb.so).
 *
 * These entry points replace, as one call, the estimation driver that the
 * reference runs on top of its kernel-level ABI:
 *   fegb_estimate_host    <- fe_gpu_estimate(cfg, header, host, group_sizes, result)
 *                            (src/core/fe_pipeline.f90:516-1896) including the
 *                            upload of src/gpu/fe_gpu_data.f90:41-120
 *   fegb_estimate_device  <- the same with the dataset already resident on the
 *                            device (fe_gpu_dataset, src/gpu/fe_gpu_data.f90:23-32)
 *   fegb_within_transform <- fe_gpu_within_transform (src/gpu/fe_gpu_demean.f90:63-311)
 *   fegb_cluster_ids      <- fe_build_cluster_ids (src/core/cluster_id_builder.c:271-278)
 *                            and fe_gpu_build_multi_cluster_ids
 *                            (src/gpu/fe_gpu_runtime.cu:700-886), bit-identical ids
 *   fegb_compact_ids      <- relabel_ids (tools/dataframe_to_fe_binary.py:87-94)
 *   fegb_group_sizes      <- compute_fe_group_sizes (src/core/fe_grouping.f90:11-37)
 *
 * Conventions follow the kernel-level ABI in fe_gpu_runtime.h: every call
 * returns 0 on success or a nonzero status and leaves a message readable with
 * fe_gpu_runtime_get_last_error(); matrices are column-major FP64 with leading
 * dimension n; FE and cluster ids are int32 and 1-based. Host FE ids use the
 * reference host layout fe_ids(n_fe, n): dimension index fastest.
 */
#ifndef FEGB_H
#define FEGB_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FEGB_PREC_FP64 0   /* plain form: FP64 storage and arithmetic throughout */
#define FEGB_PREC_MIXED 1  /* FP32 correction sweeps inside an FP64 refinement loop */

#define FEGB_DEMEAN_AP 0   /* symmetric over-relaxed alternating projections */
#define FEGB_DEMEAN_CG 1   /* conjugate gradients on the FE normal equations (--demean-cg) */

#define FEGB_SE_GPU 0      /* conventions of the reference GPU estimator */
#define FEGB_SE_CPU 1      /* conventions of the reference CPU estimator */

typedef struct fegb_config {
    double fe_tol;            /* stop when the max group-mean update is below this (default 1e-6) */
    int fe_max_iter;          /* iteration cap (default 500) */
    int precision;            /* FEGB_PREC_* */
    int demean_method;        /* FEGB_DEMEAN_* */
    int se_convention;        /* FEGB_SE_* */
    int drop_singletons;      /* 1: drop rows in singleton groups, iterated (off by default) */
    int n_cluster_dims;       /* entries in cluster_dims */
    const int* cluster_dims;  /* 1-based FE dimensions for clustered SEs (at most 3 used) */
    int n_iv_regressors;      /* entries in iv_regressors */
    const int* iv_regressors; /* 1-based endogenous regressor columns */
    int n_iv_instruments;     /* entries in iv_instruments (0 = all instrument columns) */
    const int* iv_instruments;/* 1-based instrument columns */
    int verbose;
    void* stream;             /* cudaStream_t to run on; NULL = the library's own stream */
    int profile;              /* 1: time every sweep launch with CUDA events (fills prof_* in the result) */
} fegb_config;

typedef struct fegb_result {
    int converged;
    int fe_iterations;        /* iterations of the within-transform */
    int solver_info;          /* 0 ok; Cholesky minor that failed; -1 all columns dropped */
    int rank;
    int dof_model;
    int dof_fes;
    long long dof_resid;
    int is_iv;
    int n_instruments;
    int n_cluster_dims_used;
    int psd_fix_applied;
    int min_single_cluster;
    long long n_obs_used;     /* rows after singleton removal */
    long long n_singletons;   /* rows dropped as singletons */
    double max_update;        /* final convergence measure */
    double rss;
    double tss_total;
    double tss_within;
    double r2;
    double r2_adj;
    double r2_within;
    double f_stat;
    /* instrumentation */
    int projections;          /* FE projections executed (all precisions) */
    int outer_iterations;     /* FP64 refinement passes (mixed form) */
    double demean_bytes;      /* algorithmic bytes of all sweep launches (per-family formulas below) */
    double time_h2d;          /* seconds */
    double time_prep;
    double time_demean;
    double time_regression;
    double time_se;
    double time_total;
    /* sweep-kernel timing when cfg.profile = 1, by kernel family:
     * data sweeps (rows read, and written back in storage order):
     *   [0] segment FP64, [1] segment FP32, [2] small-G FP64, [3] small-G FP32
     *   algorithmic bytes n (4 + 2 C s) per launch;
     * CG operator sweeps (no row data; ids and gathered FE table rows):
     *   [4] segment FP64, [5] segment FP32, [6] small-G FP64, [7] small-G FP32
     *   algorithmic bytes n (4 D + (D-1) C s) per launch, D = FE dimensions */
    int prof_launches[8];
    double prof_seconds[8];   /* summed CUDA-event durations of those launches */
    double prof_bytes[8];     /* summed algorithmic bytes of those launches */
} fegb_result;

/* Default configuration (tolerance 1e-6, 500 iterations, FP64, AP, GPU conventions). */
void fegb_config_init(fegb_config* cfg);

/* Whole fit from host arrays: y[n], W[n*k] and Z[n*l] column-major,
 * fe_ids[n_fe*n] in the reference host layout (dimension fastest).
 * group_sizes may be NULL (computed as the max id per dimension).
 * beta and se receive k values. */
int fegb_estimate_host(const fegb_config* cfg, long long n, int k, int l, int n_fe, const double* y,
                       const double* W, const double* Z, const int* fe_ids, const int* group_sizes, double* beta,
                       double* se, fegb_result* result);

/* Whole fit from device arrays: d_y[n], d_W[n*k], d_Z[n*l] (column-major,
 * leading dimension n) and d_fe_ids[d] = device pointer to n 1-based ids of
 * dimension d. Device inputs are not modified. beta and se are host arrays. */
int fegb_estimate_device(const fegb_config* cfg, long long n, int k, int l, int n_fe, const double* d_y,
                         const double* d_W, const double* d_Z, const int* const* d_fe_ids, const int* group_sizes,
                         double* beta, double* se, fegb_result* result);

/* Within-transform of device columns in place: d_y[n], d_W[n*k], d_Z[n*l]
 * (column-major, leading dimension n) against the FE ids d_fe_ids[d].
 * *converged and *iterations are written on the host. */
int fegb_within_transform(const fegb_config* cfg, long long n, int k, int l, int n_fe, double* d_y, double* d_W,
                          double* d_Z, const int* const* d_fe_ids, const int* group_sizes, int* converged,
                          int* iterations, double* max_update);

/* Multi-way cluster-intersection ids on the device, identical to the
 * reference builder: d_fe_ids[j] (device, 1-based) for the subset dims,
 * sizes[j] their group counts. d_out_ids (device, n) receives 1-based ids,
 * *n_clusters the count. */
int fegb_cluster_ids(const int* const* d_fe_ids, const int* sizes, int n_dims, long long n, int* d_out_ids,
                     int* n_clusters);

/* 1-based dense relabelling of raw device codes (rank among sorted distinct values). */
int fegb_compact_ids(const int* d_raw, long long n, int* d_out, int* n_levels);

/* G_d = max id per dimension over device id arrays; status 1 if an id < 1. */
int fegb_group_sizes(const int* const* d_fe_ids, int n_fe, long long n, int* sizes);

/* Number of kernel launches issued by this library since it was loaded. */
long long fegb_kernel_launches(void);

/* Launch-shape knobs (process-wide integers), chosen per problem shape by the
 * autotuner (fe_gpu_gb300/autotune.py, table fe_gpu_gb300/tuning_gb300.json)
 * and set by the host before a fit. Keys:
 *   "dense_form"                -1 default, 0 CUDA-core, 1 tensor-core form of
 *                               the CG operator's count-matrix passes
 *   "cg_cols_per_pass"          0: all columns of a table row in one pass of
 *                               the CG operator sweep; 4 or 8: at most that many
 *   "split_gram_pairs_per_col"  Gram products with at least this many output
 *                               pairs per input column use the split-FP32 form
 *   "cg_graph"                  1: the CG loop runs as a CUDA graph; 0: host loop
 *   "batch_estimator"           1: fegb_estimate_batch estimates each column
 *                               class in one batched pass; 0: spec by spec
 *   "cg_short_groups"           1: a CG operator sweep whose groups all have
 *                               few positions runs one thread per group; 0:
 *                               the chunked sweep for every stream
 * No knob changes what is computed beyond rounding; unknown keys and values
 * out of range return a nonzero status. */
int fegb_set_tuning(const char* key, int value);
int fegb_get_tuning(const char* key, int* value);
/* Every knob back to its default. */
int fegb_reset_tuning(void);

/* Memory of the current device's default stream-ordered pool, the pool this
 * library's temporaries come from: bytes in use now, the high-water mark of
 * bytes in use, and bytes reserved from the device. reset_high != 0 first
 * resets the high-water mark to the bytes in use now. Any output may be null.
 * A diagnostic for hosts that budget device memory. */
int fegb_pool_usage(int reset_high, unsigned long long* used, unsigned long long* used_high,
                    unsigned long long* reserved);

/* Self-test of one dense count-matrix pass of the CG operator (FP32 storage,
 * uint8 counts), on host arrays. counts: Ge x Gs row-major (rows of each pair
 * of a group g of a many-group dimension and a group t of a small dimension);
 * pe: Ge x ld and ps: Gs x ld rows (first C columns used). Outputs:
 *   out_small[t*C+c] = -sum_g counts[g][t] pe[g][c]        (null: not formed)
 *   out_extra[g*C+c] (+)= sum_t counts[g][t] ps[t][c]      (null: not formed;
 *                       accumulate = 1 adds to the values passed in)
 * Schur form (sums non-null, Ge x C; group_counts Ge; pe unused; out_extra
 * null): out_table[g*ld+c] = (sums[g][c] - sum_t counts[g][t] ps[t][c]) /
 * group_counts[g] and out_small uses those rows as pe; for odd Ge the group
 * counts are placed one element past a 16-byte boundary on the device (the
 * pass then loads them with plain loads instead of bulk copies).
 * tensor_cores = 1: the tensor-core (tcgen05, BF16 pieces) form where the
 * shapes allow it (C <= 16, Gs <= 64), else the FP32 form; 0: the FP32 form. */
int fegb_test_dense_pair(const unsigned char* counts, long long Ge, int Gs, const float* pe, const float* ps, int ld,
                         int C, const float* sums, const int* group_counts, int accumulate, int tensor_cores,
                         double* out_small, float* out_extra, float* out_table);

/* Self-test of the FP64 group-sum sweeps behind the within-transform's group
 * means, on host arrays: X is n x C row-major, gid the 0-based group of each
 * row (non-decreasing for the segment form, small_g = 0; any order for the
 * small-G form, small_g = 1, which needs G x C to fit its shared-memory
 * tables). out_sums[g*C+c] = sum of X[i][c] over the rows of group g. */
int fegb_test_group_sums(const double* X, long long n, int C, const int* gid, int G, int small_g, double* out_sums);

/* Self-test of the Gram products behind the normal equations and the
 * single-row cluster meats, on host arrays: X is n x a row-major; out (a x a,
 * column-major, both triangles) = X'X. split = 1: the split-FP32
 * (double-single) forms (rows kernel up to 10 columns, register-blocked
 * kernel above); 0: the FP64 form. */
int fegb_test_gram(const double* X, long long n, int a, int split, double* out);

/* FE reconstruction of --save-fe (reconstruct_and_save_fixed_effects,
 * src/core/fe_pipeline.f90:1619-1733): forward Gauss-Seidel sweeps of the
 * residual y - W beta (beta: host, k values), dimension by dimension, each
 * dimension's group means centred and accumulated, until the largest update
 * is below cfg.fe_tol (at most cfg.fe_max_iter sweeps). fe_values and
 * fe_counts (host) receive sum(G_d) entries, dimension by dimension (group g of
 * dimension d at offset sum_{e<d} G_e + g - 1); groups with count 0 have value 0. */
int fegb_reconstruct_fe(const fegb_config* cfg, long long n, int k, int n_fe, const double* d_y, const double* d_W,
                        const double* beta, const int* const* d_fe_ids, const int* group_sizes, double* fe_values,
                        long long* fe_counts, int* iterations, double* max_update);

/* ---- the .bin dataset straight to device memory ----
 * Replaces the host loader load_dataset_from_file (src/io/fe_data_io.f90:23-389)
 * plus the upload: the header is detected as the reference does (new/old
 * header, FP64/FP32 values, optional precision flag and META block), every
 * column is read in chunks into pinned buffers by a pool of host threads and
 * copied to its place on the device; FP32 values are widened to FP64 there.
 * Device buffers are owned by the caller: release them with fegb_free_dataset.
 * The META names block, when present, starts at metadata_offset. */
typedef struct fegb_dataset {
    long long n;
    int k, l, n_fe;
    int has_cluster, has_weights;
    int precision_flag;         /* values on disk: 0 FP64, 1 FP32 */
    long long metadata_offset;  /* byte offset of the META block, 0 when absent */
    double* y;                  /* device, n */
    double* W;                  /* device, n x k column-major (ld n); NULL when k = 0 */
    double* Z;                  /* device, n x l column-major (ld n); NULL when l = 0 */
    int* fe_ids;                /* device, dimension d at fe_ids + d * n (1-based ids) */
    int* cluster;               /* device, n; NULL unless has_cluster */
    double* weights;            /* device, n; NULL unless has_weights */
    double seconds;             /* wall time of the load */
} fegb_dataset;

int fegb_load_bin(const char* path, fegb_dataset* out);
int fegb_free_dataset(fegb_dataset* ds);

/* ---- batched specifications ----
 * One independent regression of a batch: its own rows, columns, FE ids,
 * cluster dimensions and IV columns (device arrays in the layout of
 * fegb_estimate_device). */
typedef struct fegb_spec {
    long long n;               /* rows (> 0) */
    int k, l, n_fe;            /* regressors, instruments, FE dimensions (1..8) */
    const double* y;           /* device, n */
    const double* W;           /* device, n x k column-major (ld n) */
    const double* Z;           /* device, n x l column-major (ld n); may be NULL when l = 0 */
    const int* const* fe_ids;  /* host array of n_fe device pointers to n 1-based ids */
    int n_cluster_dims;
    const int* cluster_dims;   /* 1-based FE dimensions of this spec */
    int n_iv_regressors;
    const int* iv_regressors;  /* 1-based endogenous columns of W */
    int n_iv_instruments;
    const int* iv_instruments; /* 1-based columns of Z (0 entries = all) */
} fegb_spec;

/* Fits n_specs independent specifications with one within-transform per
 * column-count class: the specifications of a class are stacked into one
 * problem whose FE groups are disjoint by specification and demeaned
 * together (the stacked system is block diagonal, so each specification gets
 * exactly its own projection); each is then estimated on its own rows.
 * Tolerance, precision, method and SE convention come from cfg (singleton
 * dropping is not supported here); cluster dimensions and IV columns from
 * each spec. beta and se are host arrays of sum(k) values in spec order;
 * results[i] describes spec i (fe_iterations, converged, max_update and
 * time_demean are those of its class's shared within-transform; with
 * cfg.profile the class's sweep timings appear once, in the prof_* fields of
 * the class's first spec). */
int fegb_estimate_batch(const fegb_config* cfg, int n_specs, const fegb_spec* specs, double* beta, double* se,
                        fegb_result* results);

/* ---- formula design-matrix expansion (src/src_main.f90:595-1440) ----
 * Every expanded regressor or instrument is a product of factors taken left
 * to right; a factor is a raw source column or the dummy of one of its levels
 * (1.0 where nint(x) == level, else 0.0). */
#define FEGB_DESIGN_MAX_FACTORS 8
typedef struct fegb_design_factor {
    int src;       /* index into the list of source columns */
    int level;     /* level of the dummy (used when is_dummy = 1) */
    int is_dummy;  /* 1: factor = (nint(x) == level); 0: factor = x */
} fegb_design_factor;

typedef struct fegb_design_column {
    int n_factors; /* 1..FEGB_DESIGN_MAX_FACTORS */
    fegb_design_factor factors[FEGB_DESIGN_MAX_FACTORS];
} fegb_design_column;

/* Levels of a categorical device column (collect_levels_for_column,
 * src/src_main.f90:1390-1435): the first max_levels distinct values lying
 * within 1e-6 of an integer, in order of first appearance, written sorted
 * ascending to the host array levels[max_levels]; *n_levels on the host. */
int fegb_design_levels(const double* d_col, long long n, int max_levels, int* levels, int* n_levels, void* stream);

/* Expanded columns on the device: column j of d_out (at d_out + j*ld_out,
 * n values) = product of cols[j].factors over the device source columns
 * d_src[0..n_src) (host array of device pointers, n values each). */
int fegb_build_design(const double* const* d_src, int n_src, long long n, const fegb_design_column* cols, int n_cols,
                      double* d_out, long long ld_out, void* stream);

/* Iterated singleton removal: d_keep (device, n bytes) gets 1 for kept rows. */
int fegb_drop_singletons(const int* const* d_fe_ids, const int* sizes, int n_fe, long long n, unsigned char* d_keep,
                         long long* n_dropped);

#ifdef __cplusplus
}
#endif

#endif /* FEGB_H */
