// Batched estimation of the specifications of one stacked column class after
// the class's shared within-transform (batch_est.cu).
#pragma once

#include "common.cuh"
#include "fegb.h"

#include <vector>

namespace fegb {

constexpr int BE_MAX_COLS = 64;  // class width (1 + k + l, padded) the batched estimator takes
constexpr int BE_MAX_FE = 4;

// One specification of the class, as stacked: rows [row0, row0 + n) of the
// class's columns (y, then W, then Z, then zeros), FE dimension d with G[d]
// groups whose stacked 1-based ids are goff[d] + 1 .. goff[d] + G[d].
struct BeSpecHost {
    long long row0 = 0, n = 0;
    int k = 0, l = 0, n_fe = 0;
    int G[BE_MAX_FE] = {1, 1, 1, 1};
    int goff[BE_MAX_FE] = {0, 0, 0, 0};
    int n_cd = 0;
    int cd[3] = {0, 0, 0};       // 0-based FE dimensions of the clustered SEs (valid, unique, at most 3)
    std::vector<int> endog;      // 1-based endogenous regressor columns
    std::vector<int> instr;      // 1-based instrument columns (empty: all)
    const double* y_raw = nullptr;  // the specification's raw y (device), for the total sum of squares
};

// Whether the batched estimator takes a class: reference GPU conventions, a
// class width of at most BE_MAX_COLS and cluster keys that fit 64 bits.
bool batch_est_eligible(const fegb_config& cfg, int Cw, const std::vector<BeSpecHost>& specs);

// Estimates every specification of the class: Gram products, 2SLS normal
// equations, column filter, Cholesky solve and inverse, residuals and scores,
// clustered SEs with multi-way inclusion-exclusion and the PSD fix, dof and
// R^2, with a fixed number of launches for the whole class. yb and Wb are the
// class's demeaned columns (Wb column-major, ld N, Cw - 1 columns); ids_b[d]
// the stacked 1-based ids. beta[i], se[i] (host) receive specification i's k
// values; results[i] its estimation fields (solver, rank, dof, RSS, TSS, the
// clustering fields and timings); the within-transform fields are left as set
// by the caller, which also derives R^2 and F from them.
int estimate_class_batched(const fegb_config& cfg, const std::vector<BeSpecHost>& specs, long long N, int Cw,
                           const double* yb, const double* Wb, const int32_t* const* ids_b, int n_fe_b,
                           double* const* beta, double* const* se, fegb_result* const* results, cudaStream_t s);

}  // namespace fegb
