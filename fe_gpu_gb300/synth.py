"""Seeded synthetic panels with the shapes of the benchmark workloads.

Every generator returns a fe_host_arrays (y, W, Z column-major, fe_ids of
shape (n_fe, n)) plus a header carrying names. Seeds default to
20261203 + workload index.

* nls_panel          -- unbalanced individual/occupation/year panel
                        (about 4,700 individuals with 1-15 consecutive years).
* worker_firm_panel  -- worker x period panel over firms of Pareto(1.5) sizes
                        with a per-period switching probability; used for the
                        20M-row (1M workers, 100k firms, 20 periods, p=0.1) and
                        150M-row (5M workers, 1M firms, 30 periods, p=0.05)
                        workloads.
* iv_panel           -- 2SLS panel with categorical regressors/instruments.
* reference_panel    -- the reference's own generator
                        (tools/generate_synthetic_data.py:71-177) restated
                        with vectorised tenure; same RNG call sequence.
"""
from __future__ import annotations

from typing import Optional

import numpy as np

from .bin_io import fe_dataset_header, fe_host_arrays

BASE_SEED = 20261203


def _pack(y, W, Z, fe_ids, names_x, names_fe, names_z=(), depvar="y"):
    n = y.shape[0]
    W = np.asfortranarray(W, dtype=np.float64) if W is not None else np.zeros((n, 0), order="F")
    Z = np.asfortranarray(Z, dtype=np.float64) if Z is not None else np.zeros((n, 0), order="F")
    fe = np.asfortranarray(np.vstack(fe_ids).astype(np.int32))
    hdr = fe_dataset_header(n_obs=n, n_regressors=W.shape[1], n_instruments=Z.shape[1], n_fe=fe.shape[0],
                            depvar_name=depvar, regressor_names=list(names_x), instrument_names=list(names_z),
                            fe_names=list(names_fe))
    return hdr, fe_host_arrays(y=np.ascontiguousarray(y, dtype=np.float64), W=W, Z=Z, fe_ids=fe)


def nls_panel(seed: int = BASE_SEED + 0, n_ids: int = 4700, n_years: int = 15, n_occ: int = 13):
    """Unbalanced panel: U{1..15} consecutive years per individual, Zipf(1.1)
    occupations, FE effects N(0, 0.3^2), five regressors (hours, experience,
    union, tenure, weeks unemployed), noise N(0, 0.3^2)."""
    rng = np.random.default_rng(seed)
    lengths = rng.integers(1, n_years + 1, size=n_ids)
    starts = rng.integers(0, n_years - lengths + 1)
    ids = np.repeat(np.arange(1, n_ids + 1, dtype=np.int32), lengths)
    offs = np.arange(ids.size) - np.repeat(np.cumsum(lengths) - lengths, lengths)
    year = (np.repeat(starts, lengths) + offs + 1).astype(np.int32)
    n = ids.size
    p = np.arange(1, n_occ + 1, dtype=np.float64) ** -1.1
    occ = (rng.choice(n_occ, size=n, p=p / p.sum()) + 1).astype(np.int32)
    a_id = rng.normal(0.0, 0.3, n_ids)
    a_occ = rng.normal(0.0, 0.3, n_occ)
    a_year = rng.normal(0.0, 0.3, n_years)
    hours = np.clip(rng.normal(37.0, 10.0, n), 1.0, 80.0)
    exper = rng.gamma(2.0, 3.0, n)
    union = (rng.random(n) < 0.25).astype(np.float64)
    tenure = rng.exponential(5.0, n)
    wks_ue = rng.poisson(2.0, n).astype(np.float64)
    W = np.column_stack([hours, exper, union, tenure, wks_ue])
    beta = np.array([0.012, 0.035, 0.11, 0.021, -0.018])
    y = a_id[ids - 1] + a_occ[occ - 1] + a_year[year - 1] + W @ beta + rng.normal(0.0, 0.3, n)
    return _pack(y, W, None, [ids, occ, year], ["hours", "experience", "union", "tenure", "wks_ue"],
                 ["idcode", "occ_code", "year"], depvar="ln_wage")


def _pareto_sampler(rng, n_firms, alpha):
    w = rng.pareto(alpha, n_firms) + 1.0
    cum = np.cumsum(w)
    total = cum[-1]

    def draw(m):
        return np.minimum(np.searchsorted(cum, rng.random(m) * total, side="right"), n_firms - 1).astype(np.int32)

    return draw


def worker_firm_panel(n_workers: int = 1_000_000, n_firms: int = 100_000, n_periods: int = 20,
                      switch_prob: float = 0.1, n_reg: int = 8, rho: float = 0.3, seed: int = BASE_SEED + 1,
                      tenure_sick: bool = False, pareto_alpha: float = 1.5):
    """Worker x period panel (rows worker-major). Firms have Pareto(alpha)
    sizes; each period a worker moves to a new firm with probability
    switch_prob. With tenure_sick the first two regressors are tenure
    (periods at the current firm) and a Bernoulli(0.05) sick shock and the
    remaining n_reg - 2 are N(0, 1); otherwise all n_reg regressors are N(0, 1)
    with correlation rho to the worker effect."""
    rng = np.random.default_rng(seed)
    draw = _pareto_sampler(rng, n_firms, pareto_alpha)
    firm = np.empty((n_workers, n_periods), dtype=np.int32)
    firm[:, 0] = draw(n_workers)
    tenure = np.zeros((n_workers, n_periods), dtype=np.float64) if tenure_sick else None
    for t in range(1, n_periods):
        move = rng.random(n_workers) < switch_prob
        nf = firm[:, t - 1].copy()
        idx = np.nonzero(move)[0]
        nf[idx] = draw(idx.size)
        firm[:, t] = nf
        if tenure_sick:
            tenure[:, t] = np.where(nf == firm[:, t - 1], tenure[:, t - 1] + 1.0, 0.0)
    n = n_workers * n_periods
    worker = np.repeat(np.arange(1, n_workers + 1, dtype=np.int32), n_periods)
    period = np.tile(np.arange(1, n_periods + 1, dtype=np.int32), n_workers)
    firm_ids = firm.reshape(-1) + 1
    a_w = rng.standard_normal(n_workers)
    psi = rng.normal(0.0, 0.3, n_firms)
    tau = rng.normal(0.0, 0.1, n_periods)
    W = np.empty((n, n_reg), dtype=np.float64, order="F")
    aw_rows = a_w[worker - 1]
    names = []
    j0 = 0
    if tenure_sick:
        W[:, 0] = tenure.reshape(-1)
        W[:, 1] = (rng.random(n) < 0.05).astype(np.float64)
        names += ["tenure", "sick_shock"]
        j0 = 2
    s = np.sqrt(1.0 - rho * rho)
    for j in range(j0, n_reg):
        W[:, j] = rho * aw_rows + s * rng.standard_normal(n)
        names.append(f"x{j + 1 - j0}" if not tenure_sick else f"extra_{j - 1}")
    beta = np.linspace(-0.5, 0.5, n_reg)
    if tenure_sick:
        beta[0], beta[1] = 0.04, -0.2
    y = 0.5 * aw_rows + psi[firm_ids - 1] + tau[period - 1] + W @ beta + rng.normal(0.0, 0.5, n)
    return _pack(y, W, None, [worker, firm_ids, period], names, ["worker", "firm", "time"], depvar="wage")


def reference_panel(workers=1000, firms=200, periods=8, extra_vars=0, seed=1234, intercept=1.0, betas=(0.4, -0.2),
                    extra_coeffs=None, extra_std=0.3, noise_std=0.5, sick_std=0.5):
    """tools/generate_synthetic_data.py:71-177 restated (no instruments):
    same RNG draws in the same order; the per-row tenure loop is replaced by an
    equivalent run-length computation."""
    rng = np.random.default_rng(seed)
    worker_obs = np.repeat(np.arange(workers, dtype=np.int32) + 1, periods)
    time_obs = np.tile(np.arange(periods, dtype=np.int32) + 1, workers)
    n = worker_obs.size
    firm_obs = rng.integers(1, firms + 1, size=n, dtype=np.int32)
    # tenure: periods already spent at the current firm within the worker's run
    f2 = firm_obs.reshape(workers, periods)
    start = np.ones_like(f2, dtype=bool)
    start[:, 1:] = f2[:, 1:] != f2[:, :-1]
    pos = np.broadcast_to(np.arange(periods), (workers, periods))
    run_start = np.maximum.accumulate(np.where(start, pos, 0), axis=1)
    tenure = (pos - run_start).reshape(-1).astype(np.float64)
    sick = rng.normal(0.0, sick_std, size=n)
    if extra_vars > 0:
        if extra_coeffs is not None and len(extra_coeffs) > 0:
            coeffs = np.array(extra_coeffs, dtype=np.float64)
        else:
            coeffs = rng.normal(0.0, 0.5, size=extra_vars)
        extras = rng.normal(0.0, extra_std, size=(extra_vars, n))
        extras += 0.02 * (time_obs - 1)
    else:
        coeffs = np.zeros(0)
        extras = np.zeros((0, n))
    worker_fe = rng.normal(0.0, 0.3, size=workers)
    firm_fe = rng.normal(0.0, 0.2, size=firms)
    time_fe = rng.normal(0.0, 0.1, size=periods)
    eps = rng.normal(0.0, noise_std, size=n)
    b1, b2 = betas
    wages = intercept + b1 * tenure + b2 * sick
    if extra_vars > 0:
        wages += np.dot(coeffs, extras)
    wages += worker_fe[worker_obs - 1] + firm_fe[firm_obs - 1] + time_fe[time_obs - 1] + eps
    W = np.column_stack((tenure, sick, extras.T)) if extra_vars > 0 else np.column_stack((tenure, sick))
    names = ["tenure", "sick_shock"] + [f"extra_{j + 1}" for j in range(extra_vars)]
    hdr, host = _pack(wages, W, None, [worker_obs, firm_obs, time_obs], names, ["worker", "firm", "time"],
                      depvar="wage")
    return hdr, host, coeffs


def iv_panel(n: int = 10_000_000, g=(500_000, 50_000, 30), seed: int = BASE_SEED + 2):
    """2SLS panel with uniform FE assignment, a continuous and a 4-level
    categorical endogenous regressor, a continuous and a 20-level categorical
    instrument, a 20x4 factorial a&&b, a continuous interaction x1&x2 and six
    exogenous N(0, 1) regressors; structural and first-stage errors correlated
    0.4. Returns the raw (unexpanded) variables as a dict plus the FE ids."""
    rng = np.random.default_rng(seed)
    fe = [rng.integers(1, gd + 1, size=n, dtype=np.int32) for gd in g]
    a_fe = [rng.normal(0.0, 0.3, gd) for gd in g]
    x_exog = rng.standard_normal((n, 6))
    zc = rng.integers(1, 21, size=n, dtype=np.int32)     # 20-level instrument
    z1 = rng.standard_normal(n)
    cat_a = rng.integers(1, 21, size=n, dtype=np.int32)  # 20 levels
    cat_b = rng.integers(1, 5, size=n, dtype=np.int32)   # 4 levels
    u = rng.standard_normal(n)
    v1 = 0.4 * u + np.sqrt(1 - 0.16) * rng.standard_normal(n)
    v2 = 0.4 * u + np.sqrt(1 - 0.16) * rng.standard_normal(n)
    zc_eff = rng.normal(0.0, 0.5, 21)
    x_end = 0.5 * z1 + 0.3 * zc_eff[zc] + 0.3 * x_exog[:, 0] + a_fe[0][fe[0] - 1] + v1
    latent = 0.8 * z1 - 0.4 * zc_eff[zc] + v2
    cat_end = np.clip(np.digitize(latent, [-0.8, 0.0, 0.8]) + 1, 1, 4).astype(np.int32)
    y = (0.7 * x_end + np.array([0.0, 0.25, -0.1, 0.4, 0.6])[cat_end] + x_exog @ np.linspace(-0.3, 0.3, 6)
         + 0.15 * x_exog[:, 0] * x_exog[:, 1] + 0.05 * cat_a / 20.0 + 0.1 * (cat_b == 3)
         + sum(a[f - 1] for a, f in zip(a_fe, fe)) + u)
    raw = dict(y=y, x_end=x_end, cat_end=cat_end, z1=z1, zc=zc, cat_a=cat_a, cat_b=cat_b,
               **{f"x{j + 1}": x_exog[:, j] for j in range(6)})
    return raw, fe


IV_FORMULA = ("y ~ x_end i.2.cat_end x1 x2 x3 x4 x5 x6 x1&x2 i.cat_a&&i.cat_b (x_end i.2.cat_end ~ z1 i.zc), "
              "fe(f1 f2 f3) cluster(f1 f2)")


def iv_formula_panel(n: int = 10_000_000, g=(500_000, 50_000, 30), seed: int = BASE_SEED + 2):
    """iv_panel as a raw dataset plus the formula that expands it: regressors
    [x_end, cat_end, x1..x6, cat_a, cat_b], instruments [z1, zc], FEs f1..f3.
    IV_FORMULA expands to 90 regressors (x_end, 3 cat_end dummies with base 2,
    x1..x6, x1&x2, 19 + 3 + 57 columns of i.cat_a&&i.cat_b) and 20 instruments
    (z1 and 19 zc dummies)."""
    raw, fe = iv_panel(n=n, g=g, seed=seed)
    names_x = ["x_end", "cat_end"] + [f"x{j}" for j in range(1, 7)] + ["cat_a", "cat_b"]
    W = np.column_stack([raw[k].astype(np.float64) for k in names_x])
    Z = np.column_stack([raw["z1"], raw["zc"].astype(np.float64)])
    hdr, host = _pack(raw["y"], W, Z, fe, names_x, ["f1", "f2", "f3"], names_z=["z1", "zc"])
    return hdr, host, IV_FORMULA


def batch_specs(n_specs: int = 512, total_rows: float = 100e6, row_range=(5_000, 2_000_000), seed: int = BASE_SEED + 4,
                max_rows: Optional[int] = None):
    """Independent specifications of uneven size for the batched path: rows
    log-uniform in row_range (rescaled so they add up to about total_rows),
    1-3 FEs with level counts proportional to rows^0.7, 2-24 N(0, 1)
    regressors, 75% OLS and 25% 2SLS (1-2 endogenous regressors, 1-3 extra
    instruments), 1-3-way clustering. Per-spec seeds are seed * 1000 + spec.
    Returns [(host arrays, dict(cluster_fe_dims, iv_regressors))]."""
    rng = np.random.default_rng(seed)
    lo, hi = np.log(row_range[0]), np.log(row_range[1])
    rows = np.exp(rng.uniform(lo, hi, n_specs))
    rows *= total_rows / rows.sum()
    rows = np.clip(np.round(rows), 500, max_rows or np.inf).astype(np.int64)
    out = []
    for s in range(n_specs):
        r = np.random.default_rng(seed * 1000 + s)
        n = int(rows[s])
        n_fe = int(r.integers(1, 4))
        G = [max(2, int(round(c * n ** 0.7))) for c in r.uniform(0.2, 1.0, n_fe)]
        fe = [r.integers(1, g + 1, size=n, dtype=np.int32) for g in G]
        k = int(r.integers(2, 25))
        iv = r.random() < 0.25
        n_endog = int(r.integers(1, 3)) if iv else 0
        n_endog = min(n_endog, k - 1)
        l = n_endog + int(r.integers(0, 3)) if iv else 0
        X = r.standard_normal((n, k))
        Zm = r.standard_normal((n, l)) if l else np.zeros((n, 0))
        u = r.standard_normal(n)
        for j in range(n_endog):  # endogenous columns driven by the instruments and the error
            X[:, j] += Zm @ r.uniform(0.4, 0.8, l) + 0.4 * u
        y = X @ r.uniform(-1, 1, k) + sum(r.normal(0, 0.3, g)[f - 1] for g, f in zip(G, fe)) + u
        ncl = int(r.integers(1, n_fe + 1))
        cl = sorted(r.choice(np.arange(1, n_fe + 1), size=ncl, replace=False).tolist())
        host = fe_host_arrays(y=y, W=np.asfortranarray(X), Z=np.asfortranarray(Zm),
                              fe_ids=np.asfortranarray(np.vstack(fe)))
        out.append((host, dict(cluster_fe_dims=cl, iv_regressors=list(range(1, n_endog + 1)))))
    return out
