"""--save-fe on the CPU: the oracle's loop-for-loop restatement of
reconstruct_and_save_fixed_effects (src/core/fe_pipeline.f90:1619-1733)
recovers centred FE values that reproduce the residual, and the CSV writer
follows write_fe_outputs (:1735-1771) with Fortran ES24.16 values."""
import numpy as np

from fe_gpu_gb300.estimator import format_es24_16, write_fe_outputs
from oracle import oracle as O


def _panel(n=4000, seed=0):
    rng = np.random.default_rng(seed)
    fe = np.vstack([rng.integers(1, 80, n), rng.integers(1, 12, n), rng.integers(1, 5, n)]).astype(np.int32)
    W = rng.standard_normal((n, 2))
    beta = np.array([0.5, -1.0])
    y = W @ beta + sum(rng.normal(0, 1, g)[f - 1] for g, f in zip((80, 12, 5), fe)) + 0.7
    return y, W, fe, beta


def test_oracle_reconstruction_reproduces_residual():
    y, W, fe, beta = _panel()
    v, c, it, mu = O.reconstruct_fe(y, W, fe, beta, tol=1e-11)
    assert mu < 1e-11 and it < 10000
    r = y - W @ beta
    fit = sum(v[d][fe[d] - 1] for d in range(3))
    assert np.max(np.abs(fit - (r - r.mean()))) < 1e-9
    for d in range(3):
        assert np.array_equal(c[d], np.bincount(fe[d] - 1, minlength=len(c[d])))
        assert abs(float((v[d] * c[d]).sum())) < 1e-8  # every dimension centred


def test_oracle_reconstruction_iteration_cap():
    y, W, fe, beta = _panel(seed=1)
    v, c, it, mu = O.reconstruct_fe(y, W, fe, beta, tol=0.0, max_iter=3)
    assert it == 4  # a DO loop that runs to completion leaves its index one past the end


def test_es24_16_and_csv_layout(tmp_path):
    assert format_es24_16(1.0) == "  1.0000000000000000E+00"
    assert format_es24_16(-1.2345678901234567e-4) == " -1.2345678901234567E-04"
    assert format_es24_16(0.0) == "  0.0000000000000000E+00"
    assert format_es24_16(1e-300) == "  1.0000000000000000-300"
    assert all(len(format_es24_16(x)) == 24 for x in (3.0, -2.5e200, 7e-7))
    paths = write_fe_outputs(str(tmp_path / "out"), [np.array([0.5, 0.0, -1.25])], [np.array([2, 0, 1])])
    assert open(paths[0]).read() == ("level_id,fe_value\n1,  5.0000000000000000E-01\n"
                                     "3, -1.2500000000000000E+00\n")
