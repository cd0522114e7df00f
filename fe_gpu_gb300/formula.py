"""Stata-style formula front end over the device design builder.

    wage ~ x1 i.2.cat x1&x2 i.a&&i.b (xend i.2.cend ~ z1 i.zc), fe(f1 f2 f3) cluster(f1 f2)

The parser restates the reference's (src/cli/fe_cli.f90:487-1020):
terms separated by blanks; ``i.`` marks a categorical term and ``i.<b>.`` its
base level; ``a&b`` (or ``a#b``) is one interaction; ``a&&b`` (or ``a##b``)
expands to every non-empty subset of its parts (main effects and all
interactions, in mask order); ``( ... ~ ... )`` lists endogenous regressors and
excluded instruments; ``fe(...)``, ``cluster(...)`` and ``vce(cluster ...)``
name FE and cluster dimensions.

The planner restates build_formula_design_matrix (src/src_main.f90:595-736)
and its helpers (:793-1440): main terms first, then interactions, each
categorical factor expanded to the dummies of its levels except the base;
levels are the first 40 distinct integer values of the raw column in order of
appearance, sorted (collect_levels_for_column :1390-1435). The planner only
decides which columns to build; levels are collected and the columns are
written on the device (fegb_design_levels, fegb_build_design).

One deliberate difference: the reference reads a main-formula variable that
exists only among the instruments from the regressor matrix at the
instrument's index (append_main_term_columns, src/src_main.f90:1198-1227),
which selects an unrelated column or reads out of bounds. Here such a
formula raises ValueError.
"""
from __future__ import annotations

import copy
import ctypes as C
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

MAX_CATEGORIES = 40  # src/src_main.f90:15


def _lower(s: str) -> str:
    """to_lower of the reference: ASCII A-Z only (src/cli/fe_cli.f90)."""
    return "".join(chr(ord(c) + 32) if "A" <= c <= "Z" else c for c in s)


@dataclass
class fe_formula_term:  # src/core/fe_config.f90:6-10
    name: str = ""
    is_categorical: bool = False
    base_level: int = 1


@dataclass
class fe_formula_interaction:  # src/core/fe_config.f90:12-14
    factors: list = field(default_factory=list)


@dataclass
class FormulaSpec:
    """The formula fields of fe_runtime_config (src/core/fe_config.f90:16-46)."""
    depvar_name: str = ""
    formula_terms: list = field(default_factory=list)
    formula_interactions: list = field(default_factory=list)
    iv_regressor_terms: list = field(default_factory=list)
    iv_instrument_terms: list = field(default_factory=list)
    iv_regressor_names: list = field(default_factory=list)
    iv_instrument_names: list = field(default_factory=list)
    fe_name_targets: list = field(default_factory=list)
    cluster_name_targets: list = field(default_factory=list)
    regressor_name_targets: list = field(default_factory=list)
    use_formula_design: bool = False
    formula_has_categorical: bool = False
    formula_spec: str = ""
    warnings: list = field(default_factory=list)


# ------------------------------ parser ------------------------------------

def _append_name(lst: list, value: str) -> None:  # fe_cli.f90:989-1012
    if value.rstrip():
        lst.append(value.rstrip())


def _split_whitespace(text: str) -> list:  # fe_cli.f90:945-987 (blanks only)
    return [t for t in text.rstrip().split(" ") if t]


def _split_token_by(text: str, sep: str) -> list:  # fe_cli.f90:858-881
    out: list = []
    n = len(text.rstrip())
    start = 0
    while start < n:
        pos = text.find(sep, start, n)
        if pos < 0:
            _append_name(out, text[start:n])
            break
        _append_name(out, text[start:pos])
        start = pos + len(sep)
    return out


def _read_positive_int(text: str) -> Optional[int]:
    """Fortran list-directed integer read of the base level (optional sign and
    digits, surrounding blanks ignored); None when it does not parse."""
    t = text.strip()
    if t[:1] in "+-":
        body = t[1:]
    else:
        body = t
    if not body or not body.isdigit() or not body.isascii():
        return None
    return int(t)


def parse_factor_from_token(text: str) -> fe_formula_term:  # fe_cli.f90:740-772
    term = fe_formula_term()
    s = text.rstrip()
    if len(s) >= 2 and s[:2] == "i.":
        term.is_categorical = True
        rest = s[2:].rstrip()
        dot = rest.find(".")
        if dot >= 0:
            base = _read_positive_int(rest[:dot])
            if base is not None and base > 0:
                term.base_level = base
                term.name = rest[dot + 1:].rstrip()
            else:
                term.name = rest
        else:
            term.name = rest
    else:
        term.name = s
    return term


def _terms_equal(a: fe_formula_term, b: fe_formula_term) -> bool:  # fe_cli.f90:837-841
    return a.is_categorical == b.is_categorical and _lower(a.name.rstrip()) == _lower(b.name.rstrip())


def _append_formula_term(lst: list, term: fe_formula_term) -> None:  # fe_cli.f90:774-796
    low = _lower(term.name.rstrip())
    for t in lst:
        if _lower(t.name.rstrip()) == low:
            t.is_categorical = t.is_categorical or term.is_categorical
            return
    lst.append(copy.copy(term))


def _add_main_term(spec: FormulaSpec, term: fe_formula_term) -> None:  # fe_cli.f90:798-816
    if not term.name.rstrip():
        return
    if term.is_categorical:
        spec.formula_has_categorical = True
    for t in spec.formula_terms:
        if _terms_equal(t, term):
            return
    spec.formula_terms.append(copy.copy(term))


def _add_interaction(spec: FormulaSpec, factors: list) -> None:  # fe_cli.f90:818-835
    if len(factors) <= 1:
        return
    for it in spec.formula_interactions:
        if len(it.factors) == len(factors) and all(_terms_equal(a, b) for a, b in zip(it.factors, factors)):
            return
    spec.formula_interactions.append(fe_formula_interaction([copy.copy(f) for f in factors]))


def _handle_double_hash(spec: FormulaSpec, token: str, delim: str) -> None:  # fe_cli.f90:680-706
    parts = _split_token_by(token, delim)
    n = len(parts)
    for mask in range(1, 1 << n):
        subset = []
        for j in range(n):
            if mask & (1 << j):
                t = parse_factor_from_token(parts[j].rstrip())
                if t.is_categorical:
                    spec.formula_has_categorical = True
                subset.append(t)
        if len(subset) == 1:
            _add_main_term(spec, subset[0])
        else:
            _add_interaction(spec, subset)


def _handle_interaction(spec: FormulaSpec, token: str, delim: str) -> None:  # fe_cli.f90:708-730
    parts = _split_token_by(token, delim)
    if len(parts) <= 1:
        if len(parts) == 1:
            _add_main_term(spec, parse_factor_from_token(parts[0].rstrip()))
        return
    factors = []
    for p in parts:
        t = parse_factor_from_token(p.rstrip())
        if t.is_categorical:
            spec.formula_has_categorical = True
        factors.append(t)
    _add_interaction(spec, factors)


def _process_token(spec: FormulaSpec, token: str) -> None:  # fe_cli.f90:664-678
    if not token.rstrip():
        return
    if "&&" in token:
        _handle_double_hash(spec, token.rstrip(), "&&")
    elif "&" in token:
        _handle_interaction(spec, token.rstrip(), "&")
    elif "##" in token:
        _handle_double_hash(spec, token.rstrip(), "##")
    elif "#" in token:
        _handle_interaction(spec, token.rstrip(), "#")
    else:
        _add_main_term(spec, parse_factor_from_token(token.rstrip()))


def _token_has_factor_notation(token: str) -> bool:  # fe_cli.f90:883-895
    w = token.rstrip()
    return (len(w) >= 2 and w[:2] == "i.") or "#" in w


def _parse_iv_block(spec: FormulaSpec, text: str) -> None:  # fe_cli.f90:593-626
    block = text.rstrip()
    tilde = block.find("~")
    if tilde < 0:
        spec.warnings.append('Invalid IV specification (missing "~") in formula.')
        return
    for tok in _split_whitespace(block[:tilde]):
        t = parse_factor_from_token(tok)
        _append_name(spec.iv_regressor_names, t.name)
        _append_formula_term(spec.iv_regressor_terms, t)
    for tok in _split_whitespace(block[tilde + 1:]):
        t = parse_factor_from_token(tok)
        _append_name(spec.iv_instrument_names, t.name)
        _append_formula_term(spec.iv_instrument_terms, t)


def _parse_rhs_terms(spec: FormulaSpec, rhs: str) -> None:  # fe_cli.f90:554-591
    n = len(rhs.rstrip())
    i = 0
    while i < n:
        ch = rhs[i]
        if ch == " ":
            i += 1
            continue
        if ch == "(":
            start = i + 1
            depth = 1
            while i < n and depth > 0:
                i += 1
                if i >= n:
                    break
                if rhs[i] == "(":
                    depth += 1
                elif rhs[i] == ")":
                    depth -= 1
            if depth != 0:
                spec.warnings.append("Unmatched parenthesis in formula; ignoring trailing text.")
                break
            _parse_iv_block(spec, rhs[start:i])
            i += 1
        else:
            start = i
            while i < n and rhs[i] != " " and rhs[i] != "(":
                i += 1
            token = rhs[start:i].rstrip()
            if not _token_has_factor_notation(token):
                if token and _lower(token) not in [_lower(t) for t in spec.regressor_name_targets]:
                    spec.regressor_name_targets.append(token)
            _process_token(spec, token)


def _extract_parenthesized(text: str, open_pos: int) -> str:  # fe_cli.f90:897-918
    depth = 1
    i = open_pos + 1
    while i < len(text):
        if text[i] == "(":
            depth += 1
        elif text[i] == ")":
            depth -= 1
            if depth == 0:
                break
        i += 1
    if depth != 0:
        return ""
    return text[open_pos + 1:i]


def _parse_options(spec: FormulaSpec, tail: str) -> None:  # fe_cli.f90:628-662
    low = _lower(tail)
    pos = low.find("fe(")
    if pos >= 0:
        spec.fe_name_targets = _split_whitespace(_extract_parenthesized(tail, pos + 2))
    pos = low.find("cluster(")
    if pos >= 0:
        spec.cluster_name_targets = _split_whitespace(_extract_parenthesized(tail, pos + 7))
    pos = low.find("vce(")
    if pos >= 0:
        block = _extract_parenthesized(tail, pos + 3)
        if block.rstrip() and _lower(block).find("cluster") == 0:
            spec.cluster_name_targets = _split_whitespace(block[7:].lstrip())


def parse_formula_string(raw: str) -> FormulaSpec:  # fe_cli.f90:487-538
    """Parses one formula the way the reference CLI does (see module docstring)."""
    spec = FormulaSpec()
    work = raw.rstrip()
    if not work:
        return spec
    comma = work.find(",")
    if comma >= 0:
        main_part, tail = work[:comma].rstrip(), work[comma + 1:].rstrip()
    else:
        main_part, tail = work, ""
    tilde = main_part.find("~")
    if tilde < 0:
        spec.warnings.append('Formula is missing "~" separator; ignoring entry.')
        return spec
    spec.depvar_name = main_part[:tilde].rstrip()
    _parse_rhs_terms(spec, main_part[tilde + 1:].rstrip())
    if tail:
        _parse_options(spec, tail)
    if spec.formula_terms or spec.formula_interactions:
        spec.use_formula_design = True
        spec.formula_spec = work
    return spec


# ------------------------------ planner -----------------------------------

@dataclass
class DesignColumn:
    """One expanded column: product of factors (source matrix 'W' or 'Z',
    0-based column, dummy level or None for the raw value)."""
    name: str
    factors: list          # [(matrix, col, level_or_None), ...]
    endogenous: bool = False


@dataclass
class DesignPlan:
    regressors: list                      # DesignColumn for every expanded regressor (W)
    instruments: Optional[list]           # DesignColumn for every expanded instrument (Z); None = Z unchanged
    iv_regressors: list                   # 1-based endogenous regressor columns
    iv_instrument_cols: list              # 1-based instrument columns to use
    warnings: list = field(default_factory=list)

    @property
    def regressor_names(self) -> list:
        return [c.name for c in self.regressors]


@dataclass
class _VarInfo:  # variable_info_entry of src/src_main.f90
    name: str
    needs_levels: bool
    base_level: int = 1
    column_index: int = 0     # 1-based; 0 = not found
    is_instrument: bool = False
    levels: Optional[list] = None
    valid: bool = False


def _find_index(names: Sequence[str], name: str) -> int:
    low = _lower(name.rstrip())
    for i, nm in enumerate(names):
        if _lower(nm.rstrip()) == low:
            return i + 1
    return 0


def _base_for_name(spec: FormulaSpec, name: str) -> int:  # src_main.f90:1099-1132
    low = _lower(name.rstrip())
    for t in spec.formula_terms:
        if _lower(t.name.rstrip()) == low:
            return t.base_level
    for it in spec.formula_interactions:
        for t in it.factors:
            if _lower(t.name.rstrip()) == low:
                return t.base_level
    for t in spec.iv_regressor_terms:
        if _lower(t.name.rstrip()) == low:
            return t.base_level
    for t in spec.iv_instrument_terms:
        if _lower(t.name.rstrip()) == low:
            return t.base_level
    return 1


def _append_factor_name(names: list, cats: list, name: str, is_cat: bool) -> None:  # src_main.f90:987-1008
    if not name.rstrip():
        return
    low = _lower(name.rstrip())
    for i, nm in enumerate(names):
        if _lower(nm.rstrip()) == low:
            cats[i] = cats[i] or is_cat
            return
    names.append(name.rstrip())
    cats.append(is_cat)


LevelsFn = Callable[[str, int], list]  # (matrix 'W' or 'Z', 0-based column) -> levels (sorted, <= 40)


def _collect_infos(spec, names, cats, regressor_names, instrument_names, levels_of, instruments_only, warnings):
    infos = []
    for name, cat in zip(names, cats):
        info = _VarInfo(name=name, needs_levels=cat, base_level=_base_for_name(spec, name))
        if instruments_only:
            info.column_index = _find_index(instrument_names, name)
            info.is_instrument = True
        else:
            info.column_index = _find_index(regressor_names, name)
            if info.column_index <= 0:
                info.column_index = _find_index(instrument_names, name)
                info.is_instrument = info.column_index > 0
        if info.column_index <= 0:
            warnings.append(f'Variable "{name}" not found in dataset; dropping.')
            infos.append(info)
            continue
        if info.needs_levels:
            info.levels = list(levels_of("Z" if info.is_instrument else "W", info.column_index - 1))
            if len(info.levels) <= 1:
                warnings.append(f'Categorical variable "{name}" has <=1 level; skipping dummy expansion.')
                info.needs_levels = False
        info.valid = True
        infos.append(info)
    return infos


def _find_info(infos: list, name: str):
    low = _lower(name.rstrip())
    for info in infos:
        if _lower(info.name.rstrip()) == low:
            return info
    return None


def _is_endogenous(spec: FormulaSpec, name: str) -> bool:  # src_main.f90:1164-1176
    low = _lower(name.rstrip())
    return any(_lower(t.name.rstrip()) == low for t in spec.iv_regressor_terms)


def _base_index(levels: list, base_level: int) -> int:
    """0-based position of the base level; the first level when absent
    (find_level_index, src_main.f90:1086-1097, and its callers)."""
    return levels.index(base_level) if base_level in levels else 0


def _factor_block(spec, term, infos, instruments_only):
    """[(name, factors, endog)] of one factor (build_factor_block,
    src_main.f90:1322-1380; append_main_term_columns :1178-1231)."""
    info = _find_info(infos, term.name)
    if info is None or not info.valid:
        return None
    if info.is_instrument and not instruments_only:
        raise ValueError(f'formula variable "{term.name}" is only an instrument column; the reference would read an '
                         f'unrelated regressor column for it')
    mat = "Z" if info.is_instrument else "W"
    col = info.column_index - 1
    endog = False if instruments_only else _is_endogenous(spec, term.name)
    if not term.is_categorical:
        return [(term.name.rstrip(), [(mat, col, None)], endog)]
    if info.levels is None or len(info.levels) <= 1:
        return None
    b = _base_index(info.levels, term.base_level)
    return [(f"{term.name.rstrip()}:{lv}", [(mat, col, lv)], endog) for i, lv in enumerate(info.levels) if i != b]


def plan_design(spec: FormulaSpec, regressor_names: Sequence[str], instrument_names: Sequence[str],
                levels_of: LevelsFn) -> DesignPlan:
    """Column plan of build_formula_design_matrix (src/src_main.f90:595-736)."""
    warnings: list = []
    names, cats = [], []
    for t in spec.formula_terms:
        _append_factor_name(names, cats, t.name, t.is_categorical)
    for it in spec.formula_interactions:
        for t in it.factors:
            _append_factor_name(names, cats, t.name, t.is_categorical)
    infos = _collect_infos(spec, names, cats, regressor_names, instrument_names, levels_of, False, warnings)
    cols: list = []
    for t in spec.formula_terms:  # append_main_term_columns, in term order
        block = _factor_block(spec, t, infos, False)
        if block:
            cols += [DesignColumn(nm, f, e) for nm, f, e in block]
    for it in spec.formula_interactions:  # append_interaction_columns :1233-1320
        if len(it.factors) <= 1:
            continue
        cur = _factor_block(spec, it.factors[0], infos, False)
        if cur is None:
            continue
        for fac in it.factors[1:]:
            nxt = _factor_block(spec, fac, infos, False)
            if nxt is None:
                cur = None
                break
            cur = [(f"{a[0]}&{b[0]}", a[1] + b[1], a[2] or b[2]) for a in cur for b in nxt]
        if cur:
            cols += [DesignColumn(nm, f, e) for nm, f, e in cur]
    iv_regs = [i + 1 for i, c in enumerate(cols) if c.endogenous]

    inst_cols = None
    iv_inst = []
    if spec.iv_instrument_terms and len(instrument_names) > 0:  # :694-735
        inames, icats = [], []
        for t in spec.iv_instrument_terms:
            _append_factor_name(inames, icats, t.name, t.is_categorical)
        iinfos = _collect_infos(spec, inames, icats, regressor_names, instrument_names, levels_of, True, warnings)
        built: list = []
        for t in spec.iv_instrument_terms:  # append_instrument_term_columns :1233-1267
            block = _factor_block(spec, t, iinfos, True)
            if block:
                built += [DesignColumn(nm, f, False) for nm, f, _ in block]
        if built:
            inst_cols = built
            iv_inst = list(range(1, len(built) + 1))
        else:
            warnings.append("IV instrument expansion produced no columns; skipping.")
    elif spec.iv_instrument_names and len(instrument_names) > 0:
        # explicit instrument names without expansion (apply_config_bindings, fe_cli.f90:1160-1170)
        iv_inst = sorted(i for i in (_find_index(instrument_names, nm) for nm in spec.iv_instrument_names) if i > 0)
    return DesignPlan(regressors=cols, instruments=inst_cols, iv_regressors=iv_regs, iv_instrument_cols=iv_inst,
                      warnings=warnings)


@dataclass
class FormulaBinding:
    """FE selection and cluster dimensions of a formula (apply_config_bindings,
    src/cli/fe_cli.f90:1104-1174, and apply_fe_filter, src/src_main.f90:488-575)."""
    fe_selection: list       # 1-based FE dimensions of the dataset to keep, in order
    cluster_fe_dims: list    # 1-based, within the selection
    warnings: list = field(default_factory=list)


def bind_names(spec: FormulaSpec, fe_names: Sequence[str], n_fe: int,
               cluster_fe_dims: Sequence[int] = ()) -> FormulaBinding:
    warnings: list = []

    def map_names(req):
        out = []
        for nm in req:
            i = _find_index(fe_names, nm)
            if i > 0:
                out.append(i)
            else:
                warnings.append(f'Unable to match name "{nm}" in dataset metadata.')
        return out

    clusters = list(cluster_fe_dims)
    if not clusters and spec.cluster_name_targets and fe_names is not None:
        mapped = map_names(spec.cluster_name_targets)
        if mapped:
            clusters = mapped
        elif n_fe > 0:  # positional fallback when no name matched
            clusters = list(range(1, min(len(spec.cluster_name_targets), n_fe) + 1))
    selection = list(range(1, n_fe + 1))
    if spec.fe_name_targets and fe_names:
        mapped = map_names(spec.fe_name_targets)
        if mapped:
            selection = mapped
    clusters = sorted(clusters)  # sort_cluster_dimensions
    # apply_fe_filter: cluster dims follow their FE dimension into the selection
    remap = {d: j + 1 for j, d in enumerate(selection)}
    clusters = [remap[d] for d in clusters if d in remap]
    return FormulaBinding(fe_selection=selection, cluster_fe_dims=clusters, warnings=warnings)


# ------------------------------ device path --------------------------------

def device_levels(d_col: int, n: int, stream: Optional[int] = None, max_levels: int = MAX_CATEGORIES) -> list:
    """Levels of a device column (fegb_design_levels)."""
    from . import _native as N

    out = (C.c_int * max(1, max_levels))()
    cnt = C.c_int(0)
    st = N.lib().fegb_design_levels(C.c_void_p(d_col), n, max_levels, out, C.byref(cnt),
                                    C.c_void_p(stream) if stream else None)
    N.check(st, "fegb_design_levels")
    return [int(out[i]) for i in range(cnt.value)]


def build_columns(columns: Sequence[DesignColumn], sources: dict, n: int, d_out: int, ld: int,
                  stream: Optional[int] = None) -> None:
    """Writes the planned columns into the device matrix d_out (column j at
    d_out + j*ld*8) with fegb_build_design. sources maps (matrix, col) to a
    device column pointer."""
    from . import _native as N

    if not columns:
        return
    keys = sorted({(m, c) for col in columns for (m, c, _) in col.factors})
    index = {k: i for i, k in enumerate(keys)}
    src = (C.c_void_p * len(keys))(*[C.c_void_p(int(sources[k])) for k in keys])
    recs = (N.FegbDesignColumn * len(columns))()
    for j, col in enumerate(columns):
        if len(col.factors) > N.DESIGN_MAX_FACTORS:
            raise ValueError(f"column {col.name} has more than {N.DESIGN_MAX_FACTORS} factors")
        recs[j].n_factors = len(col.factors)
        for f, (m, c, lv) in enumerate(col.factors):
            recs[j].factors[f].src = index[(m, c)]
            recs[j].factors[f].level = 0 if lv is None else int(lv)
            recs[j].factors[f].is_dummy = 0 if lv is None else 1
    st = N.lib().fegb_build_design(src, len(keys), n, recs, len(columns), C.c_void_p(d_out), ld,
                                   C.c_void_p(stream) if stream else None)
    N.check(st, "fegb_build_design")


@dataclass
class FormulaFit:
    """Device-side pieces of a formula fit, kept for inspection."""
    spec: FormulaSpec
    plan: DesignPlan
    binding: FormulaBinding
    n: int
    k: int
    l: int
    buffers: dict


class RawDevice:
    """The raw dataset columns on the device (y, regressors, instruments, FE ids)."""

    def __init__(self, header, host):
        from .estimator import DeviceBuffer

        y = np.ascontiguousarray(host.y, dtype=np.float64)
        self.n = n = y.shape[0]
        W = np.asfortranarray(host.W, dtype=np.float64) if host.W is not None else np.zeros((n, 0), order="F")
        Z = np.asfortranarray(host.Z, dtype=np.float64) if host.Z is not None else np.zeros((n, 0), order="F")
        fe = np.asarray(host.fe_ids, dtype=np.int32)
        self.k_raw, self.l_raw = W.shape[1], Z.shape[1]
        self.n_fe = fe.shape[0] if fe.ndim == 2 else 0
        self.header = header
        self.y = DeviceBuffer.from_array(y)
        self.W = DeviceBuffer.from_array(W)
        self.Z = DeviceBuffer.from_array(Z)
        self.fe = [DeviceBuffer.from_array(np.ascontiguousarray(fe[d])) for d in range(self.n_fe)]
        self.h2d_bytes = y.nbytes + W.nbytes + Z.nbytes + fe.nbytes

    def col_ptr(self, m: str, c: int) -> int:
        return (self.W if m == "W" else self.Z).ptr + 8 * self.n * c


def expand_formula(formula: str, raw: RawDevice, cfg=None, stream: Optional[int] = None):
    """Parses and binds the formula and builds its expanded design on the
    device from resident raw columns (the reference CLI flow of
    src/src_main.f90:85-100: apply_config_bindings, apply_fe_filter,
    build_formula_design_matrix). Returns (FormulaFit, cfg) with cfg carrying
    the bound cluster dimensions and IV columns."""
    from .estimator import DeviceBuffer, fe_runtime_config

    spec = parse_formula_string(formula)
    if not spec.use_formula_design:
        raise ValueError("formula has no right-hand-side terms: " + "; ".join(spec.warnings))
    cfg = copy.copy(cfg) if cfg is not None else fe_runtime_config()
    header = raw.header
    binding = bind_names(spec, list(header.fe_names), raw.n_fe, cfg.cluster_fe_dims)
    n = raw.n
    plan = plan_design(spec, list(header.regressor_names), list(header.instrument_names),
                       lambda m, c: device_levels(raw.col_ptr(m, c), n, stream))
    sources = {(m, c): raw.col_ptr(m, c) for col in plan.regressors + (plan.instruments or [])
               for (m, c, _) in col.factors}
    k = len(plan.regressors)
    bufs = {"y": raw.y, "fe": [raw.fe[d - 1] for d in binding.fe_selection]}
    bufs["W"] = DeviceBuffer(8 * n * max(k, 1))
    build_columns(plan.regressors, sources, n, bufs["W"].ptr, n, stream)
    if plan.instruments is not None:
        l = len(plan.instruments)
        bufs["Z"] = DeviceBuffer(8 * n * max(l, 1))
        build_columns(plan.instruments, sources, n, bufs["Z"].ptr, n, stream)
    else:
        l = raw.l_raw
        bufs["Z"] = raw.Z
    cfg.cluster_fe_dims = list(binding.cluster_fe_dims)
    cfg.iv_regressors = list(plan.iv_regressors)
    cfg.iv_instrument_cols = list(plan.iv_instrument_cols)
    return FormulaFit(spec=spec, plan=plan, binding=binding, n=n, k=k, l=l, buffers=bufs), cfg


def prepare_formula(formula: str, header, host, cfg=None, stream: Optional[int] = None):
    """Uploads the raw columns and expands the formula on the device."""
    return expand_formula(formula, RawDevice(header, host), cfg, stream)


def fit_formula(ff: FormulaFit, cfg, header, stream: Optional[int] = None, profile: bool = False):
    """Fits an expanded formula (fegb_estimate_device); the result carries the
    expanded coefficient names and the FormulaFit as .formula."""
    from .bin_io import fe_dataset_header
    from .estimator import fe_gpu_estimate_device

    hdr = copy.copy(header) if header is not None else fe_dataset_header()
    hdr.regressor_names = ff.plan.regressor_names
    if ff.plan.instruments is not None:
        hdr.instrument_names = [c.name for c in ff.plan.instruments]
    hdr.fe_names = [header.fe_names[d - 1] for d in ff.binding.fe_selection] if header and header.fe_names else []
    if ff.spec.depvar_name:
        hdr.depvar_name = ff.spec.depvar_name
    b = ff.buffers
    res = fe_gpu_estimate_device(cfg, ff.n, ff.k, ff.l, b["y"].ptr, b["W"].ptr if ff.k else None,
                                 b["Z"].ptr if ff.l else None, [x.ptr for x in b["fe"]], stream=stream, header=hdr,
                                 profile=profile)
    res.formula = ff
    return res


def fe_gpu_estimate_formula(formula: str, header, host, cfg=None, stream: Optional[int] = None,
                            profile: bool = False):
    """`fe_gpu --formula "..."` on host data: parse, bind names, upload, expand
    the design on the device, fit."""
    ff, cfg2 = prepare_formula(formula, header, host, cfg, stream)
    return fit_formula(ff, cfg2, header, stream, profile)
