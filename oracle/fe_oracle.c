/*
 * fe_oracle.c -- TEST INFRASTRUCTURE ONLY (see fe_oracle.h).
 *
 * A CPU restatement of the fe_gpu estimation path in plain C + OpenMP. It is
 * the checker for the CUDA library and the timed CPU baseline; it is never
 * linked into, or called from, the product path.
 */
#include "fe_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_CLUSTER_DIMS 3 /* fe_pipeline.f90:20 */

static double* dalloc(size_t n) { return (double*)calloc(n ? n : 1, sizeof(double)); }

/* ------------------------------------------------------------------------ */
/* Integer prep                                                              */
/* ------------------------------------------------------------------------ */

/* fe_grouping.f90:11-37 */
int orc_group_sizes(const int32_t* fe_ids, int n_fe, long long n, int32_t* out_sizes) {
    for (int d = 0; d < n_fe; ++d) {
        int32_t mx = 0;
        for (long long i = 0; i < n; ++i) {
            int32_t v = fe_ids[(size_t)i * n_fe + d];
            if (v < 1) return 1;
            if (v > mx) mx = v;
        }
        out_sizes[d] = mx > 0 ? mx : 0;
    }
    return 0;
}

static int cmp_i32(const void* a, const void* b) {
    int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

/* tools/dataframe_to_fe_binary.py:87-94 (pd.factorize(sort=True) + 1) */
int orc_compact_ids(const int32_t* raw, long long n, int32_t* out, int32_t* out_levels) {
    if (n <= 0) {
        *out_levels = 0;
        return 0;
    }
    int32_t* u = (int32_t*)malloc((size_t)n * sizeof(int32_t));
    if (!u) return 6;
    memcpy(u, raw, (size_t)n * sizeof(int32_t));
    qsort(u, (size_t)n, sizeof(int32_t), cmp_i32);
    long long m = 0;
    for (long long i = 0; i < n; ++i)
        if (i == 0 || u[i] != u[m - 1]) u[m++] = u[i];
    for (long long i = 0; i < n; ++i) {
        long long lo = 0, hi = m - 1;
        while (lo < hi) {
            long long mid = (lo + hi) / 2;
            if (u[mid] < raw[i]) lo = mid + 1; else hi = mid;
        }
        out[i] = (int32_t)(lo + 1);
    }
    *out_levels = (int32_t)m;
    free(u);
    return 0;
}

/* Iterated singleton removal: drop every row whose group in some dimension has
 * exactly one surviving row, until no such row remains. */
long long orc_drop_singletons(const int32_t* fe_ids, int n_fe, long long n, const int32_t* group_sizes,
                              uint8_t* keep) {
    for (long long i = 0; i < n; ++i) keep[i] = 1;
    long long dropped = 0;
    int changed = 1;
    while (changed) {
        changed = 0;
        for (int d = 0; d < n_fe; ++d) {
            int32_t G = group_sizes[d];
            long long* cnt = (long long*)calloc((size_t)G + 1, sizeof(long long));
            for (long long i = 0; i < n; ++i)
                if (keep[i]) cnt[fe_ids[(size_t)i * n_fe + d]]++;
            for (long long i = 0; i < n; ++i) {
                if (keep[i] && cnt[fe_ids[(size_t)i * n_fe + d]] == 1) {
                    keep[i] = 0;
                    ++dropped;
                    changed = 1;
                }
            }
            free(cnt);
        }
    }
    return dropped;
}

/* cluster_id_builder.c:271-314 restated. Sort-encoded path: key = sum_j
 * mult_j*(v_j-1) with mult_j = prod_{i<j} size_i; ids are the 1-based ranks of
 * the distinct keys in increasing order (cluster_id_builder.c:146-194). When the
 * key span exceeds 2^62 (or a size is 0) ids are handed out in order of first
 * appearance (cluster_id_builder.c:202-257). */
typedef struct {
    uint64_t key;
    int64_t idx;
} orc_keyidx;

static int cmp_keyidx(const void* a, const void* b) {
    const orc_keyidx* x = (const orc_keyidx*)a;
    const orc_keyidx* y = (const orc_keyidx*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

typedef struct {
    int32_t v[4];
    int64_t idx;
} orc_tuple;

static int g_tuple_len;
static int cmp_tuple(const void* a, const void* b) {
    const orc_tuple* x = (const orc_tuple*)a;
    const orc_tuple* y = (const orc_tuple*)b;
    for (int j = 0; j < g_tuple_len; ++j)
        if (x->v[j] != y->v[j]) return x->v[j] < y->v[j] ? -1 : 1;
    return (x->idx > y->idx) - (x->idx < y->idx);
}

static int cmp_i64pair(const void* a, const void* b) {
    const int64_t* x = (const int64_t*)a;
    const int64_t* y = (const int64_t*)b;
    return (x[0] > y[0]) - (x[0] < y[0]);
}

int orc_cluster_ids(const int32_t* fe_ids, int ld_fe, long long n, const int32_t* subset_dims,
                    const int32_t* subset_sizes, int subset_len, int32_t* out_ids, int32_t* out_n_clusters) {
    if (!fe_ids || !subset_dims || !subset_sizes || !out_ids || !out_n_clusters) return 1;
    if (ld_fe <= 0 || n <= 0) return 2;
    if (subset_len <= 0 || subset_len > 4) return 3;

    int sort_ok = 1;
    uint64_t span = 1;
    for (int j = 0; j < subset_len; ++j) {
        uint64_t s = (uint64_t)subset_sizes[j];
        if (s == 0 || s > UINT64_MAX / span) {
            sort_ok = 0;
            break;
        }
        span *= s;
        if (span > (1ULL << 62)) {
            sort_ok = 0;
            break;
        }
    }
    if (sort_ok) {
        uint64_t mult[4];
        uint64_t stride = 1;
        for (int j = 0; j < subset_len; ++j) {
            mult[j] = stride;
            stride *= (uint64_t)subset_sizes[j];
        }
        orc_keyidx* ki = (orc_keyidx*)malloc((size_t)n * sizeof(orc_keyidx));
        if (!ki) return 6;
        for (long long i = 0; i < n; ++i) {
            uint64_t key = 0;
            for (int j = 0; j < subset_len; ++j) {
                int dim = subset_dims[j];
                if (dim < 1 || dim > ld_fe) continue;
                int32_t v = fe_ids[(size_t)i * ld_fe + (dim - 1)];
                key += mult[j] * (uint64_t)(int64_t)(v - 1);
            }
            ki[i].key = key;
            ki[i].idx = i;
        }
        qsort(ki, (size_t)n, sizeof(orc_keyidx), cmp_keyidx);
        int32_t cur = 0;
        for (long long i = 0; i < n; ++i) {
            if (i == 0 || ki[i].key != ki[i - 1].key) {
                if (cur == INT32_MAX) {
                    free(ki);
                    return 5;
                }
                ++cur;
            }
            out_ids[ki[i].idx] = cur;
        }
        *out_n_clusters = cur;
        free(ki);
        return 0;
    }

    /* first-appearance ids */
    for (int j = 0; j < subset_len; ++j)
        if (subset_dims[j] < 1 || subset_dims[j] > ld_fe) return 4;
    orc_tuple* t = (orc_tuple*)malloc((size_t)n * sizeof(orc_tuple));
    if (!t) return 6;
    for (long long i = 0; i < n; ++i) {
        memset(t[i].v, 0, sizeof(t[i].v));
        for (int j = 0; j < subset_len; ++j) t[i].v[j] = fe_ids[(size_t)i * ld_fe + (subset_dims[j] - 1)];
        t[i].idx = i;
    }
    g_tuple_len = subset_len;
    qsort(t, (size_t)n, sizeof(orc_tuple), cmp_tuple);
    /* distinct tuples with their first index */
    int64_t* first = (int64_t*)malloc((size_t)n * 2 * sizeof(int64_t));
    int64_t m = 0;
    for (long long i = 0; i < n; ++i) {
        /* rows of one tuple are sorted by index, so the first row seen is the first appearance */
        if (i == 0 || memcmp(t[i].v, t[i - 1].v, sizeof(int32_t) * subset_len) != 0) {
            first[2 * m] = t[i].idx;
            first[2 * m + 1] = m;
            ++m;
        }
    }
    /* group index of each sorted row */
    int64_t* grp = (int64_t*)malloc((size_t)n * sizeof(int64_t));
    int64_t gcur = -1;
    for (long long i = 0; i < n; ++i) {
        if (i == 0 || memcmp(t[i].v, t[i - 1].v, sizeof(int32_t) * subset_len) != 0) ++gcur;
        grp[i] = gcur;
    }
    qsort(first, (size_t)m, 2 * sizeof(int64_t), cmp_i64pair);
    int32_t* id_of_group = (int32_t*)malloc((size_t)m * sizeof(int32_t));
    for (int64_t r = 0; r < m; ++r) id_of_group[first[2 * r + 1]] = (int32_t)(r + 1);
    for (long long i = 0; i < n; ++i) out_ids[t[i].idx] = id_of_group[grp[i]];
    *out_n_clusters = (int32_t)m;
    free(t);
    free(first);
    free(grp);
    free(id_of_group);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Demeaning                                                                 */
/* ------------------------------------------------------------------------ */

/* fe_pipeline.f90:225-277 (cpu_demean_single) for one FE dimension. */
static void demean_single_forward(double* y, double* W, int k, long long n, const int32_t* fe_ids, int n_fe, int d,
                                  int32_t G, double* max_change) {
    if (G <= 0) return;
    double* sum_y = dalloc((size_t)G + 1);
    double* sum_W = dalloc(((size_t)G + 1) * (size_t)(k > 0 ? k : 1));
    long long* cnt = (long long*)calloc((size_t)G + 1, sizeof(long long));
#pragma omp parallel
    {
        double* ly = dalloc((size_t)G + 1);
        double* lW = dalloc(((size_t)G + 1) * (size_t)(k > 0 ? k : 1));
        long long* lc = (long long*)calloc((size_t)G + 1, sizeof(long long));
#pragma omp for schedule(static)
        for (long long i = 0; i < n; ++i) {
            int32_t g = fe_ids[(size_t)i * n_fe + d];
            if (g < 1 || g > G) continue;
            ly[g] += y[i];
            lc[g] += 1;
            for (int j = 0; j < k; ++j) lW[(size_t)g * k + j] += W[(size_t)j * n + i];
        }
#pragma omp critical
        {
            for (int32_t g = 1; g <= G; ++g) {
                sum_y[g] += ly[g];
                cnt[g] += lc[g];
                for (int j = 0; j < k; ++j) sum_W[(size_t)g * k + j] += lW[(size_t)g * k + j];
            }
        }
        free(ly);
        free(lW);
        free(lc);
    }
    for (int32_t g = 1; g <= G; ++g) {
        if (cnt[g] > 0) {
            sum_y[g] = sum_y[g] / (double)cnt[g];
            for (int j = 0; j < k; ++j) sum_W[(size_t)g * k + j] /= (double)cnt[g];
        } else {
            sum_y[g] = 0.0;
            for (int j = 0; j < k; ++j) sum_W[(size_t)g * k + j] = 0.0;
        }
    }
    double mc = *max_change;
#pragma omp parallel for schedule(static) reduction(max : mc)
    for (long long i = 0; i < n; ++i) {
        int32_t g = fe_ids[(size_t)i * n_fe + d];
        if (g < 1 || g > G) continue;
        y[i] -= sum_y[g];
        double a = fabs(sum_y[g]);
        if (a > mc) mc = a;
        for (int j = 0; j < k; ++j) {
            W[(size_t)j * n + i] -= sum_W[(size_t)g * k + j];
            a = fabs(sum_W[(size_t)g * k + j]);
            if (a > mc) mc = a;
        }
    }
    *max_change = mc;
    free(sum_y);
    free(sum_W);
    free(cnt);
}

/* fe_pipeline.f90:135-152 */
int orc_demean_forward(double* y, double* W, int k, long long n, int n_fe, const int32_t* fe_ids,
                       const int32_t* group_sizes, double tol, int max_iter, int* converged, double* max_update) {
    double mu = 0.0;
    int iter;
    if (n_fe <= 0) {
        *converged = 1;
        *max_update = 0.0;
        return 0;
    }
    for (iter = 1; iter <= max_iter; ++iter) {
        mu = 0.0;
        for (int d = 0; d < n_fe; ++d) demean_single_forward(y, W, k, n, fe_ids, n_fe, d, group_sizes[d], &mu);
        if (mu < tol) break;
    }
    /* A Fortran DO loop that runs to completion leaves the index at max+1. */
    *converged = mu < tol;
    *max_update = mu;
    return iter;
}

/* One projection of the GPU scheme for dimension d: group sums and counts
 * (fe_gpu_runtime.cu:72-111), means by reciprocal (:183-211), over-relaxed
 * mixing with the previous mixed mean (:361-372), subtraction (:213-253). */
static void sym_project(double* y, double* W, int k, double* Z, int l, long long n, int n_fe, const int32_t* fe_ids,
                        int d, int32_t G, double relax, double* prev, double* mean, double* change_dim) {
    const int C = 1 + k + l;
    long long* cnt = (long long*)calloc((size_t)G, sizeof(long long));
    memset(mean, 0, (size_t)G * C * sizeof(double));
#pragma omp parallel
    {
        double* lm = dalloc((size_t)G * C);
        long long* lc = (long long*)calloc((size_t)G, sizeof(long long));
#pragma omp for schedule(static)
        for (long long i = 0; i < n; ++i) {
            int32_t g = fe_ids[(size_t)i * n_fe + d] - 1;
            if (g < 0 || g >= G) continue;
            double* row = lm + (size_t)g * C;
            row[0] += y[i];
            for (int j = 0; j < k; ++j) row[1 + j] += W[(size_t)j * n + i];
            for (int j = 0; j < l; ++j) row[1 + k + j] += Z[(size_t)j * n + i];
            lc[g] += 1;
        }
#pragma omp critical
        {
            for (size_t t = 0; t < (size_t)G * C; ++t) mean[t] += lm[t];
            for (int32_t g = 0; g < G; ++g) cnt[g] += lc[g];
        }
        free(lm);
        free(lc);
    }
    double ch_y = 0.0, ch_w = 0.0, ch_z = 0.0;
    for (int32_t g = 0; g < G; ++g) {
        double inv = cnt[g] > 0 ? 1.0 / (double)cnt[g] : 0.0;
        for (int c = 0; c < C; ++c) {
            size_t t = (size_t)g * C + c;
            double m = mean[t] * inv;
            double p = prev[t];
            double mixed = p + relax * (m - p);
            prev[t] = mixed;
            mean[t] = mixed;
            double a = fabs(mixed);
            if (c == 0) {
                if (a > ch_y) ch_y = a;
            } else if (c <= k) {
                if (a > ch_w) ch_w = a;
            } else {
                if (a > ch_z) ch_z = a;
            }
        }
    }
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < n; ++i) {
        int32_t g = fe_ids[(size_t)i * n_fe + d] - 1;
        if (g < 0 || g >= G) continue;
        const double* row = mean + (size_t)g * C;
        y[i] -= row[0];
        for (int j = 0; j < k; ++j) W[(size_t)j * n + i] -= row[1 + j];
        for (int j = 0; j < l; ++j) Z[(size_t)j * n + i] -= row[1 + k + j];
    }
    double cd = ch_y;
    if (k > 0 && ch_w > cd) cd = ch_w;
    if (l > 0 && ch_z > cd) cd = ch_z;
    *change_dim = cd;
    free(cnt);
}

/* fe_gpu_demean.f90:63-311 */
int orc_demean_symmetric(double* y, double* W, int k, double* Z, int l, long long n, int n_fe,
                         const int32_t* fe_ids, const int32_t* group_sizes, double tol, int max_iter,
                         int* converged, double* max_update) {
    const int C = 1 + k + l;
    int iterations = 0;
    int hit = 0;
    double mu = 0.0;
    *converged = 1;
    if (n_fe == 0 || n == 0) {
        *max_update = 0.0;
        return 0;
    }
    double* relax = dalloc(n_fe);
    double* prev_change = dalloc(n_fe);
    double** prev = (double**)calloc(n_fe, sizeof(double*));
    double** mean = (double**)calloc(n_fe, sizeof(double*));
    int* order = (int*)calloc(n_fe, sizeof(int));
    for (int d = 0; d < n_fe; ++d) {
        relax[d] = 1.5;
        prev_change[d] = DBL_MAX;
        prev[d] = dalloc((size_t)group_sizes[d] * C);
        mean[d] = dalloc((size_t)group_sizes[d] * C);
        order[d] = d;
    }
    /* exchange sort by ascending group count (fe_gpu_demean.f90:104-114) */
    for (int a = 0; a < n_fe - 1; ++a)
        for (int b = a + 1; b < n_fe; ++b)
            if (group_sizes[order[b]] < group_sizes[order[a]]) {
                int t = order[a];
                order[a] = order[b];
                order[b] = t;
            }
    for (int iter = 1; iter <= max_iter; ++iter) {
        mu = 0.0;
        for (int sweep = 0; sweep < 2; ++sweep) {
            for (int pass = 0; pass < 2; ++pass) {
                for (int s = 0; s < n_fe; ++s) {
                    int d = pass == 0 ? order[s] : order[n_fe - 1 - s];
                    double cd = 0.0;
                    if (group_sizes[d] <= 0) continue;
                    sym_project(y, W, k, Z, l, n, n_fe, fe_ids, d, group_sizes[d], relax[d], prev[d], mean[d], &cd);
                    if (cd > mu) mu = cd;
                    if (cd > prev_change[d] * 1.05) {
                        relax[d] = fmax(0.4, relax[d] * 0.5);
                    } else if (cd < prev_change[d] * 0.8) {
                        relax[d] = fmin(2.0, relax[d] * 1.10);
                    }
                    prev_change[d] = cd;
                }
            }
        }
        iterations = iter;
        if (mu < tol) {
            hit = 1;
            break;
        }
    }
    *converged = hit;
    *max_update = mu;
    for (int d = 0; d < n_fe; ++d) {
        free(prev[d]);
        free(mean[d]);
    }
    free(prev);
    free(mean);
    free(relax);
    free(prev_change);
    free(order);
    return iterations;
}

/* ------------------------------------------------------------------------ */
/* Small dense linear algebra (column-major)                                 */
/* ------------------------------------------------------------------------ */

#define A_(M, i, j, ld) (M)[(size_t)(j) * (ld) + (i)]

/* dgesv + dgetri: LU with partial pivoting, solve, then inverse. */
static int lu_solve_invert(int nn, double* A, double* b, double* inv) {
    int* piv = (int*)malloc(sizeof(int) * (nn > 0 ? nn : 1));
    for (int j = 0; j < nn; ++j) {
        int p = j;
        double best = fabs(A_(A, j, j, nn));
        for (int i = j + 1; i < nn; ++i)
            if (fabs(A_(A, i, j, nn)) > best) {
                best = fabs(A_(A, i, j, nn));
                p = i;
            }
        piv[j] = p;
        if (A_(A, p, j, nn) == 0.0) {
            free(piv);
            return j + 1;
        }
        if (p != j)
            for (int c = 0; c < nn; ++c) {
                double t = A_(A, j, c, nn);
                A_(A, j, c, nn) = A_(A, p, c, nn);
                A_(A, p, c, nn) = t;
            }
        for (int i = j + 1; i < nn; ++i) {
            A_(A, i, j, nn) /= A_(A, j, j, nn);
            double f = A_(A, i, j, nn);
            for (int c = j + 1; c < nn; ++c) A_(A, i, c, nn) -= f * A_(A, j, c, nn);
        }
    }
    /* solve */
    for (int j = 0; j < nn; ++j)
        if (piv[j] != j) {
            double t = b[j];
            b[j] = b[piv[j]];
            b[piv[j]] = t;
        }
    for (int i = 0; i < nn; ++i)
        for (int c = 0; c < i; ++c) b[i] -= A_(A, i, c, nn) * b[c];
    for (int i = nn - 1; i >= 0; --i) {
        for (int c = i + 1; c < nn; ++c) b[i] -= A_(A, i, c, nn) * b[c];
        b[i] /= A_(A, i, i, nn);
    }
    /* inverse: solve A X = I column by column */
    for (int col = 0; col < nn; ++col) {
        double* x = inv + (size_t)col * nn;
        for (int i = 0; i < nn; ++i) x[i] = (i == col) ? 1.0 : 0.0;
        for (int j = 0; j < nn; ++j)
            if (piv[j] != j) {
                double t = x[j];
                x[j] = x[piv[j]];
                x[piv[j]] = t;
            }
        for (int i = 0; i < nn; ++i)
            for (int c = 0; c < i; ++c) x[i] -= A_(A, i, c, nn) * x[c];
        for (int i = nn - 1; i >= 0; --i) {
            for (int c = i + 1; c < nn; ++c) x[i] -= A_(A, i, c, nn) * x[c];
            x[i] /= A_(A, i, i, nn);
        }
    }
    free(piv);
    return 0;
}

/* fe_solver.f90:41-74 (dpotrf 'U', dpotrs, dpotri, mirror upper to lower) */
int orc_chol_solve_invert(int nn, double* Q, const double* b, double* beta, double* Q_inv) {
    /* Q = U^T U, U stored in the upper triangle */
    for (int j = 0; j < nn; ++j) {
        double s = A_(Q, j, j, nn);
        for (int p = 0; p < j; ++p) s -= A_(Q, p, j, nn) * A_(Q, p, j, nn);
        if (!(s > 0.0)) return j + 1;
        double ujj = sqrt(s);
        A_(Q, j, j, nn) = ujj;
        for (int c = j + 1; c < nn; ++c) {
            double t = A_(Q, j, c, nn);
            for (int p = 0; p < j; ++p) t -= A_(Q, p, j, nn) * A_(Q, p, c, nn);
            A_(Q, j, c, nn) = t / ujj;
        }
    }
    for (int i = 0; i < nn; ++i) beta[i] = b[i];
    /* U^T z = b */
    for (int i = 0; i < nn; ++i) {
        for (int p = 0; p < i; ++p) beta[i] -= A_(Q, p, i, nn) * beta[p];
        beta[i] /= A_(Q, i, i, nn);
    }
    /* U x = z */
    for (int i = nn - 1; i >= 0; --i) {
        for (int p = i + 1; p < nn; ++p) beta[i] -= A_(Q, i, p, nn) * beta[p];
        beta[i] /= A_(Q, i, i, nn);
    }
    /* inverse: U^{-1} then U^{-1} U^{-T} */
    double* Ui = dalloc((size_t)nn * nn);
    for (int j = 0; j < nn; ++j) {
        A_(Ui, j, j, nn) = 1.0 / A_(Q, j, j, nn);
        for (int i = j - 1; i >= 0; --i) {
            double s = 0.0;
            for (int p = i + 1; p <= j; ++p) s += A_(Q, i, p, nn) * A_(Ui, p, j, nn);
            A_(Ui, i, j, nn) = -s / A_(Q, i, i, nn);
        }
    }
    for (int i = 0; i < nn; ++i)
        for (int j = i; j < nn; ++j) {
            double s = 0.0;
            for (int p = j; p < nn; ++p) s += A_(Ui, i, p, nn) * A_(Ui, j, p, nn);
            A_(Q_inv, i, j, nn) = s;
            A_(Q_inv, j, i, nn) = s;
        }
    free(Ui);
    return 0;
}

/* Cyclic Jacobi eigen-decomposition for a symmetric matrix. */
int orc_sym_eig(int nn, double* A, double* w, double* V) {
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < nn; ++j) A_(V, i, j, nn) = (i == j) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int j = 0; j < nn; ++j)
            for (int i = 0; i < nn; ++i) {
                double a = A_(A, i, j, nn) * A_(A, i, j, nn);
                tot += a;
                if (i != j) off += a;
            }
        if (off <= 1e-30 * (tot > 0 ? tot : 1.0) || off == 0.0) break;
        for (int p = 0; p < nn - 1; ++p)
            for (int q = p + 1; q < nn; ++q) {
                double apq = A_(A, p, q, nn);
                if (apq == 0.0) continue;
                double app = A_(A, p, p, nn), aqq = A_(A, q, q, nn);
                double theta = (aqq - app) / (2.0 * apq);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int r = 0; r < nn; ++r) {
                    double arp = A_(A, r, p, nn), arq = A_(A, r, q, nn);
                    A_(A, r, p, nn) = c * arp - s * arq;
                    A_(A, r, q, nn) = s * arp + c * arq;
                }
                for (int r = 0; r < nn; ++r) {
                    double apr = A_(A, p, r, nn), aqr = A_(A, q, r, nn);
                    A_(A, p, r, nn) = c * apr - s * aqr;
                    A_(A, q, r, nn) = s * apr + c * aqr;
                }
                for (int r = 0; r < nn; ++r) {
                    double vrp = A_(V, r, p, nn), vrq = A_(V, r, q, nn);
                    A_(V, r, p, nn) = c * vrp - s * vrq;
                    A_(V, r, q, nn) = s * vrp + c * vrq;
                }
            }
    }
    for (int i = 0; i < nn; ++i) w[i] = A_(A, i, i, nn);
    /* ascending order */
    for (int i = 0; i < nn; ++i) {
        int m = i;
        for (int j = i + 1; j < nn; ++j)
            if (w[j] < w[m]) m = j;
        if (m != i) {
            double t = w[i];
            w[i] = w[m];
            w[m] = t;
            for (int r = 0; r < nn; ++r) {
                double v = A_(V, r, i, nn);
                A_(V, r, i, nn) = A_(V, r, m, nn);
                A_(V, r, m, nn) = v;
            }
        }
    }
    return 0;
}

/* fe_pipeline.f90:1844-1894: V diag(max(lambda,0)) V^T */
int orc_psd_fix(int nn, double* A) {
    double* S = dalloc((size_t)nn * nn);
    double* V = dalloc((size_t)nn * nn);
    double* w = dalloc(nn);
    memcpy(S, A, sizeof(double) * (size_t)nn * nn);
    orc_sym_eig(nn, S, w, V);
    int applied = 0;
    for (int j = 0; j < nn; ++j) {
        double lam = w[j];
        if (lam < 0.0) {
            lam = 0.0;
            applied = 1;
        }
        double s = lam > 0.0 ? sqrt(lam) : 0.0;
        for (int i = 0; i < nn; ++i) A_(V, i, j, nn) *= s;
    }
    for (int i = 0; i < nn; ++i)
        for (int j = 0; j < nn; ++j) {
            double t = 0.0;
            for (int p = 0; p < nn; ++p) t += A_(V, i, p, nn) * A_(V, j, p, nn);
            A_(A, i, j, nn) = t;
        }
    free(S);
    free(V);
    free(w);
    return applied;
}

/* ------------------------------------------------------------------------ */
/* Estimators                                                                */
/* ------------------------------------------------------------------------ */

/* fe_pipeline.f90:1935-1955 */
static double compute_tss(const double* v, long long n) {
    if (n <= 0) return 0.0;
    double s = 0.0;
    for (long long i = 0; i < n; ++i) s += v[i];
    double m = s / (double)n;
    double t = 0.0;
    for (long long i = 0; i < n; ++i) t += (v[i] - m) * (v[i] - m);
    return t;
}

static int fe_dof(const int32_t* G, int n_fe) {
    int t = 0;
    for (int d = 0; d < n_fe; ++d) t += G[d] - 1 > 0 ? G[d] - 1 : 0;
    return t;
}

/* fe_pipeline.f90:1963-2008 */
static void finalize_stats(orc_result* r, long long n_obs) {
    const double EPS = 1e-12;
    double n = (double)(n_obs > 1 ? n_obs : 1);
    double df_model = (double)(r->dof_model > 0 ? r->dof_model : 0);
    double df_resid = (double)(r->dof_resid > 1 ? r->dof_resid : 1);
    double dev = r->rss;
    double dev0 = r->tss_total > EPS ? r->tss_total : EPS;
    if (dev0 > EPS) {
        r->r2 = 1.0 - dev / dev0;
        r->r2 = fmax(0.0, fmin(1.0, r->r2));
    } else {
        r->r2 = 0.0;
    }
    if (r->tss_within > EPS) {
        r->r2_within = 1.0 - dev / r->tss_within;
        r->r2_within = fmax(0.0, fmin(1.0, r->r2_within));
    } else {
        r->r2_within = r->r2;
    }
    double fe_flag = 1.0;
    double k_total = (double)(r->dof_model + r->dof_fes + 1);
    double denom = fmax(n - k_total, 1.0);
    if (n > 1.0 && dev0 > EPS) {
        r->r2_adj = 1.0 - (dev * (n - fe_flag)) / (dev0 * denom);
        r->r2_adj = fmax(0.0, fmin(1.0, r->r2_adj));
    } else {
        r->r2_adj = r->r2;
    }
    double ssr = fmax(0.0, dev0 - dev);
    if (df_model > 0.0 && df_resid > 0.0 && dev > EPS)
        r->f_stat = (ssr / df_model) / (dev / df_resid);
    else
        r->f_stat = 0.0;
}

/* cross products of two column blocks: out (a x b) = A^T B over n rows */
static void crossprod(const double* A, int a, const double* B, int b, long long n, double* out) {
#pragma omp parallel for collapse(2) schedule(static)
    for (int i = 0; i < a; ++i)
        for (int j = 0; j < b; ++j) {
            double s = 0.0;
            const double* x = A + (size_t)i * n;
            const double* y = B + (size_t)j * n;
            for (long long r = 0; r < n; ++r) s += x[r] * y[r];
            out[(size_t)j * a + i] = s;
        }
}

/* scores S (n_clusters x k) for ids (1-based) and meat = S^T S */
static void cluster_meat(const int32_t* ids, int32_t n_clusters, const double* resid, const double* X, int k,
                         long long n, double* meat) {
    double* S = dalloc((size_t)n_clusters * k);
#pragma omp parallel
    {
        double* L = dalloc((size_t)n_clusters * k);
#pragma omp for schedule(static)
        for (long long i = 0; i < n; ++i) {
            int32_t c = ids[i];
            if (c < 1 || c > n_clusters) continue;
            for (int j = 0; j < k; ++j) L[(size_t)j * n_clusters + (c - 1)] += resid[i] * X[(size_t)j * n + i];
        }
#pragma omp critical
        for (size_t t = 0; t < (size_t)n_clusters * k; ++t) S[t] += L[t];
        free(L);
    }
    for (int a = 0; a < k; ++a)
        for (int b = 0; b < k; ++b) {
            double s = 0.0;
            for (int32_t c = 0; c < n_clusters; ++c) s += S[(size_t)a * n_clusters + c] * S[(size_t)b * n_clusters + c];
            meat[(size_t)b * k + a] = s;
        }
    free(S);
}

/* out = A * B * A for k x k matrices */
static void sandwich(int k, const double* A, const double* B, double* out) {
    double* T = dalloc((size_t)k * k);
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            double s = 0.0;
            for (int p = 0; p < k; ++p) s += B[(size_t)p * k + i] * A[(size_t)j * k + p];
            T[(size_t)j * k + i] = s; /* T = B A */
        }
    for (int i = 0; i < k; ++i)
        for (int j = 0; j < k; ++j) {
            double s = 0.0;
            for (int p = 0; p < k; ++p) s += A[(size_t)p * k + i] * T[(size_t)j * k + p];
            out[(size_t)j * k + i] = s;
        }
    free(T);
}

/* fe_pipeline.f90:71-513 */
int orc_cpu_estimate(const orc_config* cfg, long long n, int k, int n_fe, const double* y_in, const double* W_in,
                     const int32_t* fe_ids, const int32_t* group_sizes, double* beta, double* se,
                     orc_result* res) {
    memset(res, 0, sizeof(*res));
    for (int j = 0; j < k; ++j) {
        beta[j] = 0.0;
        se[j] = 0.0;
    }
    /* initialize_cpu_cluster_dims (fe_pipeline.f90:305-346) */
    int cdims[ORC_MAX_CLUSTER_DIMS];
    int n_cd = 0;
    for (int i = 0; i < cfg->n_cluster_dims && n_cd < ORC_MAX_CLUSTER_DIMS; ++i) {
        int v = cfg->cluster_dims[i];
        if (v < 1 || v > n_fe) continue;
        int dup = 0;
        for (int t = 0; t < n_cd; ++t) dup |= cdims[t] == v;
        if (!dup) cdims[n_cd++] = v;
    }
    double* y = dalloc((size_t)n);
    double* W = dalloc((size_t)n * (k > 0 ? k : 1));
    memcpy(y, y_in, sizeof(double) * (size_t)n);
    if (k > 0) memcpy(W, W_in, sizeof(double) * (size_t)n * k);
    res->tss_total = compute_tss(y, n);

    int conv = 1;
    double mu = 0.0;
    if (n_fe > 0) {
        res->fe_iterations = orc_demean_forward(y, W, k, n, n_fe, fe_ids, group_sizes, cfg->fe_tol, cfg->fe_max_iter,
                                                &conv, &mu);
    }
    res->converged = conv;
    res->max_update = mu;
    {
        double t = 0.0;
        for (long long i = 0; i < n; ++i) t += y[i] * y[i];
        res->tss_within = t;
    }
    res->dof_fes = fe_dof(group_sizes, n_fe);

    if (k > 0) {
        double* WW = dalloc((size_t)k * k);
        double* Wy = dalloc(k);
        double* Qi = dalloc((size_t)k * k);
        crossprod(W, k, W, k, n, WW);
        crossprod(W, k, y, 1, n, Wy);
        int info = lu_solve_invert(k, WW, Wy, Qi);
        res->solver_info = info;
        if (info != 0) {
            free(WW);
            free(Wy);
            free(Qi);
            free(y);
            free(W);
            return 0;
        }
        for (int j = 0; j < k; ++j) beta[j] = Wy[j];
        res->rank = k;
        res->dof_model = k;
        double* r = dalloc((size_t)n);
        double rss = 0.0;
        for (long long i = 0; i < n; ++i) {
            double v = y[i];
            for (int j = 0; j < k; ++j) v -= W[(size_t)j * n + i] * beta[j];
            r[i] = v;
            rss += v * v;
        }
        double sigma2 = rss / fmax(1.0, (double)(n - k));
        res->rss = rss;
        res->dof_resid = n - k;
        int cluster_ok = 0;
        if (n_cd > 0) {
            /* compute_clustered_se_cpu (fe_pipeline.f90:348-483) */
            double* acc = dalloc((size_t)k * k);
            double* meat = dalloc((size_t)k * k);
            double* cov = dalloc((size_t)k * k);
            int32_t* ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
            int min_single = INT32_MAX;
            cluster_ok = 1;
            for (int mask = 1; mask < (1 << n_cd); ++mask) {
                int32_t sd[ORC_MAX_CLUSTER_DIMS], ss[ORC_MAX_CLUSTER_DIMS];
                int m = 0;
                for (int j = 0; j < n_cd; ++j)
                    if (mask & (1 << j)) {
                        sd[m] = cdims[j];
                        ss[m] = group_sizes[cdims[j] - 1];
                        ++m;
                    }
                int32_t nc = 0;
                int st = orc_cluster_ids(fe_ids, n_fe, n, sd, ss, m, ids, &nc);
                if (st != 0 || nc <= 0) {
                    cluster_ok = 0;
                    break;
                }
                if (m == 1 && nc < min_single) min_single = nc;
                cluster_meat(ids, nc, r, W, k, n, meat);
                sandwich(k, Qi, meat, cov);
                double wgt = (m % 2 == 1) ? 1.0 : -1.0;
                for (size_t t = 0; t < (size_t)k * k; ++t) acc[t] += wgt * cov[t];
            }
            if (cluster_ok) {
                if (min_single < INT32_MAX) res->dof_resid = (min_single - 1 > 1) ? min_single - 1 : 1;
                double denom = (double)((n - k) > 1 ? (n - k) : 1);
                double scalar = (double)((n - 1) > 1 ? (n - 1) : 1) / denom;
                if (min_single > 1 && min_single < INT32_MAX)
                    scalar = scalar * (double)min_single / (double)(min_single - 1);
                for (int i = 0; i < k; ++i)
                    for (int j = 0; j < k; ++j) cov[(size_t)j * k + i] = 0.5 * (acc[(size_t)j * k + i] + acc[(size_t)i * k + j]);
                for (int j = 0; j < k; ++j) se[j] = sqrt(fmax(0.0, cov[(size_t)j * k + j] * scalar));
                res->n_cluster_dims_used = n_cd;
                res->min_single_cluster = min_single;
            }
            free(acc);
            free(meat);
            free(cov);
            free(ids);
        }
        if (!cluster_ok) {
            for (int j = 0; j < k; ++j) se[j] = sqrt(fmax(0.0, sigma2 * Qi[(size_t)j * k + j]));
        }
        free(r);
        free(WW);
        free(Wy);
        free(Qi);
    }
    finalize_stats(res, n);
    free(y);
    free(W);
    return 0;
}

/* fe_pipeline.f90:516-1896 (GPU-path conventions) */
int orc_gpu_estimate(const orc_config* cfg, long long n, int k, int l, int n_fe, const double* y_in,
                     const double* W_in, const double* Z_in, const int32_t* fe_ids, const int32_t* group_sizes,
                     double* beta, double* se, orc_result* res) {
    memset(res, 0, sizeof(*res));
    for (int j = 0; j < k; ++j) {
        beta[j] = 0.0;
        se[j] = 0.0;
    }
    /* initialize_cluster_dims (fe_pipeline.f90:1553-1599): valid, unique, at most 3 */
    int cdims[ORC_MAX_CLUSTER_DIMS];
    int n_cd = 0;
    for (int i = 0; i < cfg->n_cluster_dims; ++i) {
        int v = cfg->cluster_dims[i];
        if (v < 1 || v > n_fe) continue;
        int dup = 0;
        for (int t = 0; t < n_cd; ++t) dup |= cdims[t] == v;
        if (dup) continue;
        if (n_cd == ORC_MAX_CLUSTER_DIMS) break;
        cdims[n_cd++] = v;
    }
    res->tss_total = compute_tss(y_in, n);
    res->dof_fes = fe_dof(group_sizes, n_fe);
    int nested = 0;
    for (int i = 0; i < n_cd; ++i) nested += group_sizes[cdims[i] - 1] - 1 > 0 ? group_sizes[cdims[i] - 1] - 1 : 0;

    double* y = dalloc((size_t)n);
    double* W = dalloc((size_t)n * (k > 0 ? k : 1));
    double* Z = dalloc((size_t)n * (l > 0 ? l : 1));
    memcpy(y, y_in, sizeof(double) * (size_t)n);
    if (k > 0) memcpy(W, W_in, sizeof(double) * (size_t)n * k);
    if (l > 0) memcpy(Z, Z_in, sizeof(double) * (size_t)n * l);

    int conv = 1;
    double mu = 0.0;
    res->fe_iterations =
        orc_demean_symmetric(y, W, k, Z, l, n, n_fe, fe_ids, group_sizes, cfg->fe_tol, cfg->fe_max_iter, &conv, &mu);
    res->converged = conv;
    res->max_update = mu;
    if (k <= 0) {
        free(y);
        free(W);
        free(Z);
        return 0;
    }
    {
        double t = 0.0;
        for (long long i = 0; i < n; ++i) t += y[i] * y[i];
        res->tss_within = t;
    }
    double* Q = dalloc((size_t)k * k);
    double* b = dalloc(k);
    crossprod(W, k, W, k, n, Q);
    crossprod(W, k, y, 1, n, b);
    double* vdiag = dalloc(k);
    for (int j = 0; j < k; ++j) vdiag[j] = Q[(size_t)j * k + j];

    /* endogenous flags and instrument selection (fe_pipeline.f90:672-746) */
    int* is_endog = (int*)calloc(k, sizeof(int));
    for (int i = 0; i < cfg->n_iv_regressors; ++i) {
        int v = cfg->iv_regressors[i];
        if (v >= 1 && v <= k) is_endog[v - 1] = 1;
    }
    int n_endog = 0;
    for (int j = 0; j < k; ++j) n_endog += is_endog[j];
    int n_exog = k - n_endog;
    int* sel = (int*)calloc(l > 0 ? l : 1, sizeof(int));
    int n_sel = 0;
    if (l > 0) {
        for (int i = 0; i < cfg->n_iv_instruments; ++i) {
            int v = cfg->iv_instruments[i];
            if (v < 1 || v > l) continue;
            sel[n_sel++] = v;
        }
        if (n_sel == 0)
            for (int i = 0; i < l; ++i) sel[n_sel++] = i + 1;
    }
    int n_aug = n_exog + n_sel;
    int use_iv = n_endog > 0;
    if (use_iv && n_sel < n_endog) use_iv = 0;
    res->is_iv = use_iv;
    res->n_instruments = use_iv ? n_aug : 0;

    double* Xhat = NULL; /* projected regressors for the IV scores */
    int info = 0;
    if (use_iv) {
        /* build_iv_normal_equations (fe_pipeline.f90:947-1032) */
        double* Za = dalloc((size_t)n * n_aug);
        int c = 0;
        for (int j = 0; j < k; ++j)
            if (!is_endog[j]) memcpy(Za + (size_t)(c++) * n, W + (size_t)j * n, sizeof(double) * (size_t)n);
        for (int i = 0; i < n_sel; ++i) memcpy(Za + (size_t)(c++) * n, Z + (size_t)(sel[i] - 1) * n, sizeof(double) * (size_t)n);
        double* Qzz = dalloc((size_t)n_aug * n_aug);
        double* Qzy = dalloc(n_aug);
        double* Qzx = dalloc((size_t)n_aug * k);
        double* Qinv = dalloc((size_t)n_aug * n_aug);
        double* rhs = dalloc(n_aug);
        double* proj = dalloc((size_t)n_aug * k);
        crossprod(Za, n_aug, Za, n_aug, n, Qzz);
        crossprod(Za, n_aug, y, 1, n, Qzy);
        crossprod(Za, n_aug, W, k, n, Qzx);
        info = orc_chol_solve_invert(n_aug, Qzz, Qzy, rhs, Qinv);
        if (info == 0) {
            for (int a = 0; a < n_aug; ++a)
                for (int j = 0; j < k; ++j) {
                    double s = 0.0;
                    for (int p = 0; p < n_aug; ++p) s += Qinv[(size_t)p * n_aug + a] * Qzx[(size_t)j * n_aug + p];
                    proj[(size_t)j * n_aug + a] = s;
                }
            for (int i = 0; i < k; ++i)
                for (int j = 0; j < k; ++j) {
                    double s = 0.0;
                    for (int p = 0; p < n_aug; ++p) s += Qzx[(size_t)i * n_aug + p] * proj[(size_t)j * n_aug + p];
                    Q[(size_t)j * k + i] = s;
                }
            for (int i = 0; i < k; ++i)
                for (int j = i + 1; j < k; ++j) {
                    double s = 0.5 * (Q[(size_t)j * k + i] + Q[(size_t)i * k + j]);
                    Q[(size_t)j * k + i] = s;
                    Q[(size_t)i * k + j] = s;
                }
            for (int i = 0; i < k; ++i) {
                double s = 0.0;
                for (int p = 0; p < n_aug; ++p) s += Qzx[(size_t)i * n_aug + p] * rhs[p];
                b[i] = s;
            }
            Xhat = dalloc((size_t)n * k);
#pragma omp parallel for schedule(static)
            for (long long r = 0; r < n; ++r)
                for (int j = 0; j < k; ++j) {
                    double s = 0.0;
                    for (int p = 0; p < n_aug; ++p) s += Za[(size_t)p * n + r] * proj[(size_t)j * n_aug + p];
                    Xhat[(size_t)j * n + r] = s;
                }
        }
        free(Za);
        free(Qzz);
        free(Qzy);
        free(Qzx);
        free(Qinv);
        free(rhs);
        free(proj);
        if (info != 0) {
            res->solver_info = info;
            goto done;
        }
    }

    {
        /* solve_with_column_filter (fe_pipeline.f90:1034-1107) */
        double dmax = 0.0;
        for (int j = 0; j < k; ++j) dmax = fmax(dmax, fabs(vdiag[j]));
        dmax = fmax(dmax, 1.0);
        double tol = 1.0e-10 * dmax;
        int* idx = (int*)calloc(k, sizeof(int));
        int kept = 0;
        for (int j = 0; j < k; ++j)
            if (!(fabs(vdiag[j]) <= tol)) idx[kept++] = j;
        res->dof_model = kept;
        if (kept == 0) {
            res->solver_info = -1;
            free(idx);
            goto done;
        }
        double* Qs = dalloc((size_t)kept * kept);
        double* bs = dalloc(kept);
        double* bb = dalloc(kept);
        double* Qi = dalloc((size_t)kept * kept);
        for (int a = 0; a < kept; ++a) {
            bs[a] = b[idx[a]];
            for (int c2 = 0; c2 < kept; ++c2) Qs[(size_t)c2 * kept + a] = Q[(size_t)idx[c2] * k + idx[a]];
        }
        info = orc_chol_solve_invert(kept, Qs, bs, bb, Qi);
        res->solver_info = info;
        if (info != 0) {
            free(idx);
            free(Qs);
            free(bs);
            free(bb);
            free(Qi);
            goto done;
        }
        for (int a = 0; a < kept; ++a) beta[idx[a]] = bb[a];
        res->rank = kept;

        /* compute_standard_errors (fe_pipeline.f90:1109-1420) */
        double* r = dalloc((size_t)n);
        double rss = 0.0;
        for (long long i = 0; i < n; ++i) {
            double v = y[i];
            for (int j = 0; j < k; ++j) v -= W[(size_t)j * n + i] * beta[j];
            r[i] = v;
        }
        for (long long i = 0; i < n; ++i) rss += r[i] * r[i];
        long long pc = (long long)(res->dof_model > 0 ? res->dof_model : 0) + (res->dof_fes > 0 ? res->dof_fes : 0) + 1;
        long long df = n - pc > 1 ? n - pc : 1;
        res->dof_resid = df;
        res->rss = rss;
        double sigma2 = rss / (double)df;
        int cluster_ok = 0;
        if (n_cd > 0) {
            const double* X = Xhat ? Xhat : W;
            double* acc = dalloc((size_t)kept * kept);
            double* meat = dalloc((size_t)k * k);
            double* mk = dalloc((size_t)kept * kept);
            double* cov = dalloc((size_t)kept * kept);
            int32_t* ids = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
            int min_single = INT32_MAX;
            cluster_ok = 1;
            for (int mask = 1; mask < (1 << n_cd); ++mask) {
                int32_t sd[ORC_MAX_CLUSTER_DIMS], ss[ORC_MAX_CLUSTER_DIMS];
                int m = 0;
                for (int j = 0; j < n_cd; ++j)
                    if (mask & (1 << j)) {
                        sd[m] = cdims[j];
                        ss[m] = group_sizes[cdims[j] - 1];
                        ++m;
                    }
                int32_t nc = 0;
                if (m == 1) {
                    nc = group_sizes[sd[0] - 1];
                    if (nc <= 0) {
                        cluster_ok = 0;
                        break;
                    }
                    if (nc < min_single) min_single = nc;
                    for (long long i = 0; i < n; ++i) ids[i] = fe_ids[(size_t)i * n_fe + (sd[0] - 1)];
                } else {
                    int st = orc_cluster_ids(fe_ids, n_fe, n, sd, ss, m, ids, &nc);
                    if (st != 0 || nc <= 0) {
                        cluster_ok = 0;
                        break;
                    }
                }
                cluster_meat(ids, nc, r, X, k, n, meat);
                for (int a = 0; a < kept; ++a)
                    for (int c2 = 0; c2 < kept; ++c2) mk[(size_t)c2 * kept + a] = meat[(size_t)idx[c2] * k + idx[a]];
                sandwich(kept, Qi, mk, cov);
                double wgt = (m % 2 == 1) ? 1.0 : -1.0;
                for (size_t t = 0; t < (size_t)kept * kept; ++t) acc[t] += wgt * cov[t];
            }
            if (cluster_ok) {
                int nested_adj = nested > 0 ? 1 : 0;
                long long pce = (long long)(res->dof_model > 0 ? res->dof_model : 0) + nested_adj;
                double denom = (double)(n - pce > 1 ? n - pce : 1);
                double scalar = (double)(n - 1 > 1 ? n - 1 : 1) / denom;
                if (min_single > 1) scalar = scalar * (double)min_single / (double)(min_single - 1);
                for (size_t t = 0; t < (size_t)kept * kept; ++t) acc[t] *= scalar;
                for (int j = 0; j < kept; ++j)
                    for (int i = j + 1; i < kept; ++i) acc[(size_t)j * kept + i] = acc[(size_t)i * kept + j];
                res->psd_fix_applied = orc_psd_fix(kept, acc);
                for (int a = 0; a < kept; ++a) se[idx[a]] = sqrt(fmax(0.0, acc[(size_t)a * kept + a]));
                if (min_single < INT32_MAX) res->dof_resid = (min_single - 1 > 1) ? min_single - 1 : 1;
                res->n_cluster_dims_used = n_cd;
                res->min_single_cluster = min_single;
            }
            free(acc);
            free(meat);
            free(mk);
            free(cov);
            free(ids);
        }
        if (!cluster_ok) {
            for (int a = 0; a < kept; ++a) se[idx[a]] = sqrt(fmax(0.0, sigma2 * Qi[(size_t)a * kept + a]));
        }
        finalize_stats(res, n);
        free(r);
        free(idx);
        free(Qs);
        free(bs);
        free(bb);
        free(Qi);
    }
done:
    free(Xhat);
    free(is_endog);
    free(sel);
    free(vdiag);
    free(Q);
    free(b);
    free(y);
    free(W);
    free(Z);
    return 0;
}


/* src/core/fe_pipeline.f90:1619-1733 (reconstruct_and_save_fixed_effects). */
int orc_reconstruct_fe(long long n, int k, int n_fe, const double* y, const double* W, const double* beta,
                       const int32_t* fe_ids, const int32_t* sizes, double tol, int max_iter, double* values,
                       long long* counts, int* iterations, double* max_update) {
    *iterations = 0;
    *max_update = 0.0;
    if (n_fe <= 0 || n <= 0) return 0;
    long long* off = (long long*)calloc((size_t)n_fe + 1, sizeof(long long));
    int gmax = 0;
    for (int d = 0; d < n_fe; ++d) {
        off[d + 1] = off[d] + sizes[d];
        if (sizes[d] > gmax) gmax = sizes[d];
    }
    double* r = (double*)malloc(sizeof(double) * (size_t)n);
    double* gsum = (double*)malloc(sizeof(double) * (size_t)(gmax > 0 ? gmax : 1));
    double* gmean = (double*)malloc(sizeof(double) * (size_t)(gmax > 0 ? gmax : 1));
    if (!off || !r || !gsum || !gmean) {
        free(off); free(r); free(gsum); free(gmean);
        return 1;
    }
    for (long long j = 0; j < n; ++j) r[j] = y[j];
    for (int c = 0; c < k; ++c)  /* residual = residual - W(:, j) * beta(j), column by column */
        for (long long j = 0; j < n; ++j) r[j] -= W[(size_t)c * n + j] * beta[c];
    for (long long t = 0; t < off[n_fe]; ++t) {
        values[t] = 0.0;
        counts[t] = 0;
    }
    for (long long j = 0; j < n; ++j)
        for (int d = 0; d < n_fe; ++d) {
            const int g = fe_ids[(size_t)j * n_fe + d];
            if (g >= 1 && g <= sizes[d]) counts[off[d] + g - 1] += 1;
        }
    double mu = 0.0;
    int iter;
    for (iter = 1; iter <= max_iter; ++iter) {
        mu = 0.0;
        for (int d = 0; d < n_fe; ++d) {
            const int G = sizes[d];
            for (int g = 0; g < G; ++g) gsum[g] = 0.0;
            for (long long j = 0; j < n; ++j) {
                const int g = fe_ids[(size_t)j * n_fe + d];
                if (g >= 1 && g <= G) gsum[g - 1] += r[j];
            }
            double wsum = 0.0;
            long long tot = 0;
            for (int g = 0; g < G; ++g) {
                const long long c = counts[off[d] + g];
                if (c > 0) {
                    gmean[g] = gsum[g] / (double)c;
                    wsum += gmean[g] * (double)c;
                    tot += c;
                } else {
                    gmean[g] = 0.0;
                }
            }
            const double center = tot > 0 ? wsum / (double)tot : 0.0;
            for (int g = 0; g < G; ++g) {
                if (counts[off[d] + g] > 0) {
                    gmean[g] -= center;
                    values[off[d] + g] += gmean[g];
                    if (fabs(gmean[g]) > mu) mu = fabs(gmean[g]);
                } else {
                    gmean[g] = 0.0;
                }
            }
            for (long long j = 0; j < n; ++j) {
                const int g = fe_ids[(size_t)j * n_fe + d];
                if (g >= 1 && g <= G) r[j] -= gmean[g - 1];
            }
        }
        if (mu < tol) break;
    }
    *iterations = iter;
    *max_update = mu;
    free(off); free(r); free(gsum); free(gmean);
    return 0;
}
