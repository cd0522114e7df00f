/*
 * fe_oracle.h -- TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the fe_gpu estimation path, used as the correctness
 * checker for the CUDA library (tests/, smoke() and bench.py's CPU-baseline leg
 * are the only callers). Nothing in the product path links or calls this code.
 *
 * Two estimators are restated:
 *   orc_cpu_estimate  -- the reference's all-CPU estimator
 *                        (src/core/fe_pipeline.f90:71-513, fe_cpu_estimate).
 *   orc_gpu_estimate  -- the reference GPU estimator's conventions, run on the
 *                        CPU in FP64 (src/core/fe_pipeline.f90:516-1896 and
 *                        src/gpu/fe_gpu_demean.f90:63-311).
 *
 * Pinning: the restatement is checked against the reference's own known-answer
 * tests (tests/test_gpu_regression.f90, tests/test_gpu_demean.f90), against
 * the reference's compiled multi-way cluster-id builder
 * (src/core/cluster_id_builder.c, built into oracle/_ref/ by
 * oracle/build_ref.sh where the reference tree is present), and against
 * closed-form identities (noise-free panels, FWL).
 *
 * Array conventions (same as the reference host arrays):
 *   y       : n doubles
 *   W       : n x k doubles, column-major, leading dimension n
 *   Z       : n x l doubles, column-major, leading dimension n
 *   fe_ids  : n_fe x n int32, dimension index fastest (Fortran fe_ids(d, i)),
 *             1-based group ids
 */
#ifndef FE_ORACLE_H
#define FE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    double fe_tol;            /* default 1e-6 (src/core/fe_config.f90:55) */
    int fe_max_iter;          /* default 500 */
    int n_cluster_dims;       /* number of entries in cluster_dims */
    const int* cluster_dims;  /* 1-based FE dimensions to cluster on */
    int n_iv_regressors;      /* endogenous regressor indices (1-based) */
    const int* iv_regressors;
    int n_iv_instruments;     /* selected instrument columns (1-based); 0 = all */
    const int* iv_instruments;
    int demean_scheme;        /* 0: forward Gauss-Seidel (CPU path), 1: symmetric relaxed (GPU path) */
} orc_config;

typedef struct {
    int converged;
    int fe_iterations;
    int solver_info;
    int rank;
    int dof_model;
    int dof_fes;
    long long dof_resid;
    int is_iv;
    int n_instruments;
    int n_cluster_dims_used;
    int psd_fix_applied;
    int min_single_cluster;
    double max_update;
    double rss;
    double tss_total;
    double tss_within;
    double r2;
    double r2_adj;
    double r2_within;
    double f_stat;
} orc_result;

/* fe_grouping.f90:11-37: G_d = max id; returns 1 if any id < 1. */
int orc_group_sizes(const int32_t* fe_ids, int n_fe, long long n, int32_t* out_sizes);

/* tools/dataframe_to_fe_binary.py:87-94: 1-based rank among sorted distinct codes. */
int orc_compact_ids(const int32_t* raw, long long n, int32_t* out, int32_t* out_levels);

/* Iterated singleton removal (no counterpart in the reference; parity unpinned).
 * keep[i] = 1 for surviving rows; returns the number of dropped rows. */
long long orc_drop_singletons(const int32_t* fe_ids, int n_fe, long long n, const int32_t* group_sizes,
                              uint8_t* keep);

/* cluster_id_builder.c:271-314: intersection ids over subset_dims (1-based dims),
 * ranks of the mixed-radix key when the key span fits 2^62, otherwise
 * first-appearance ids. Returns 0 on success. */
int orc_cluster_ids(const int32_t* fe_ids, int ld_fe, long long n, const int32_t* subset_dims,
                    const int32_t* subset_sizes, int subset_len, int32_t* out_ids, int32_t* out_n_clusters);

/* Plain forward Gauss-Seidel demeaning of y and W in place
 * (fe_pipeline.f90:135-152, 225-277). Returns iterations; *converged, *max_update out. */
int orc_demean_forward(double* y, double* W, int k, long long n, int n_fe, const int32_t* fe_ids,
                       const int32_t* group_sizes, double tol, int max_iter, int* converged, double* max_update);

/* Symmetric over-relaxed alternating projections of y, W and Z in place
 * (fe_gpu_demean.f90:63-311). Returns iterations. */
int orc_demean_symmetric(double* y, double* W, int k, double* Z, int l, long long n, int n_fe,
                         const int32_t* fe_ids, const int32_t* group_sizes, double tol, int max_iter,
                         int* converged, double* max_update);

/* fe_pipeline.f90:71-513 */
/* FE reconstruction of --save-fe (src/core/fe_pipeline.f90:1619-1733),
 * restated loop for loop: residual = y - sum_j W_j beta_j; per iteration and
 * FE dimension d = 1..n_fe: group sums, means, centring on the count-weighted
 * mean, fe_values += means, residual -= means; stop when max |mean| < tol.
 * fe_ids: n_fe x n, dimension fastest. values/counts: sum(G_d) entries,
 * dimension by dimension. *iterations follows the reference's DO loop
 * (max_iter + 1 when the tolerance was not reached). */
int orc_reconstruct_fe(long long n, int k, int n_fe, const double* y, const double* W, const double* beta,
                       const int32_t* fe_ids, const int32_t* sizes, double tol, int max_iter, double* values,
                       long long* counts, int* iterations, double* max_update);

int orc_cpu_estimate(const orc_config* cfg, long long n, int k, int n_fe, const double* y, const double* W,
                     const int32_t* fe_ids, const int32_t* group_sizes, double* beta, double* se,
                     orc_result* res);

/* fe_pipeline.f90:516-1896 (GPU-path conventions, computed on the CPU in FP64).
 * If demeaned_y/demeaned_W/demeaned_Z are non-NULL the caller supplies already
 * demeaned columns and the within-transform is skipped (iterations reported 0). */
int orc_gpu_estimate(const orc_config* cfg, long long n, int k, int l, int n_fe, const double* y,
                     const double* W, const double* Z, const int32_t* fe_ids, const int32_t* group_sizes,
                     double* beta, double* se, orc_result* res);

/* fe_solver.f90:41-74: Cholesky solve + inverse of an n x n SPD matrix
 * (column-major). Q is overwritten; returns LAPACK-style info. */
int orc_chol_solve_invert(int nn, double* Q, const double* b, double* beta, double* Q_inv);

/* Symmetric eigen-decomposition by cyclic Jacobi (stands in for LAPACK dsyev,
 * fe_pipeline.f90:1844-1894). A is n x n column-major (overwritten);
 * eigenvalues ascending in w, eigenvectors in V columns. */
int orc_sym_eig(int nn, double* A, double* w, double* V);

/* PSD fix: clamp negative eigenvalues to zero (fe_pipeline.f90:1844-1894).
 * Returns 1 if any eigenvalue was clamped. */
int orc_psd_fix(int nn, double* A);

#ifdef __cplusplus
}
#endif

#endif
