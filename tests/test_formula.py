"""Formula front end on the CPU: the parser and column planner against the
reference's own example runs (coefficient names, IV columns, instrument
counts printed in Examples/01TESTS_fe_gpu_small_output.txt), name bindings,
and the oracle's restatement of the per-row expansion."""
import json
from pathlib import Path

import numpy as np
import pytest

from fe_gpu_gb300.formula import bind_names, parse_formula_string, plan_design
from oracle import design_ref as D

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "formula_expansion_log.json").read_text())


def _levels_fn():
    regs, insts = GOLD["raw_regressors"], GOLD["raw_instruments"]
    lv = GOLD["levels"]

    def levels_of(m, c):
        name = (regs if m == "W" else insts)[c]
        return lv.get(name, [])

    return regs, insts, levels_of


@pytest.mark.parametrize("run", range(len(GOLD["runs"])))
def test_reference_example_formulas_expand_like_the_log(run):
    r = GOLD["runs"][run]
    regs, insts, levels_of = _levels_fn()
    spec = parse_formula_string(r["formula"])
    plan = plan_design(spec, regs, insts, levels_of)
    assert plan.regressor_names == r["names"]
    assert len(plan.regressors) == r["dof_model"]
    endog = [plan.regressor_names[i - 1] for i in plan.iv_regressors]
    assert endog == r["endogenous"]
    if r["estimator"].startswith("2SLS"):
        n_exog = len(plan.regressors) - len(plan.iv_regressors)
        assert n_exog + len(plan.iv_instrument_cols) == r["n_instruments"]
    else:
        assert not plan.iv_regressors


def test_parser_structures():
    s = parse_formula_string("y ~ x1 i.3.a##b c#d x1 i.a (e i.2.f ~ z1 i.g), fe(w Firm t) vce(cluster w t)")
    assert s.depvar_name == "y"
    assert [(t.name, t.is_categorical, t.base_level) for t in s.formula_terms] == [
        ("x1", False, 1), ("a", True, 3), ("b", False, 1)]
    assert [[(f.name, f.is_categorical) for f in it.factors] for it in s.formula_interactions] == [
        [("a", True), ("b", False)], [("c", False), ("d", False)]]
    assert [(t.name, t.is_categorical, t.base_level) for t in s.iv_regressor_terms] == [("e", False, 1),
                                                                                       ("f", True, 2)]
    assert [(t.name, t.is_categorical) for t in s.iv_instrument_terms] == [("z1", False), ("g", True)]
    assert s.fe_name_targets == ["w", "Firm", "t"]
    assert s.cluster_name_targets == ["w", "t"]
    # "i.a" after "i.3.a" is the same categorical term (dedupe ignores the base)
    assert s.use_formula_design and s.formula_has_categorical


def test_parser_edge_cases():
    assert not parse_formula_string("y x1 x2").use_formula_design  # no "~"
    s = parse_formula_string("y ~ a&&b&&c")
    assert [t.name for t in s.formula_terms] == ["a", "b", "c"]
    assert [[f.name for f in it.factors] for it in s.formula_interactions] == [["a", "b"], ["a", "c"], ["b", "c"],
                                                                                ["a", "b", "c"]]
    s = parse_formula_string("y ~ i.x.y x (unclosed")
    assert [t.name for t in s.formula_terms] == ["x.y", "x"]
    assert s.warnings
    s = parse_formula_string("y ~ a&", )
    assert [t.name for t in s.formula_terms] == ["a"] and not s.formula_interactions


def test_bind_names_selection_and_clusters():
    s = parse_formula_string("y ~ x, fe(firm worker) cluster(worker firm)")
    b = bind_names(s, ["worker", "firm", "time"], 3)
    assert b.fe_selection == [2, 1]
    assert b.cluster_fe_dims == [2, 1]  # worker -> position 2, firm -> position 1
    s = parse_formula_string("y ~ x, fe(a b) cluster(p q)")
    b = bind_names(s, ["a", "b"], 2)
    assert b.cluster_fe_dims == [1, 2]  # no name matched: positional fallback


def test_oracle_levels_and_dummies():
    col = np.array([3.0, 1.0, 2.5, -1.0, 3.0000000001, 1e12, 7.0, np.nan, -1.0])
    assert D.collect_levels(col) == [-1, 1, 3, 7]
    # the first 40 distinct values by appearance, then sorted
    col = np.concatenate([np.arange(100, 50, -1), np.arange(0, 10)]).astype(float)
    assert D.collect_levels(col) == sorted(range(100, 60, -1))
    assert np.array_equal(D.dummy(np.array([2.5, -2.5, 1.4999, 2.0]), 3), [1.0, 0.0, 0.0, 0.0])
    src = {("W", 0): np.array([1.0, 2.0, 2.0]), ("W", 1): np.array([0.5, 1.5, 2.5])}
    assert np.array_equal(D.design_column(src, [("W", 0, 2), ("W", 1, None)]), [0.0, 1.5, 2.5])
