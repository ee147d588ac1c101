"""Reduction tree -> flat GPU plan (the role of compiler.compile_components).

The reference (datashader/compiler.py:36-150) turns a reduction tree into
``create`` / ``append`` / ``combine`` / ``finalize`` functions by generating
Python source and numba-compiling it.  Here the same tree becomes a flat,
hashable :class:`Plan`: a list of deduplicated GPU base accumulators (the
``dsgb_base`` structs of include/dsgb.h) and a list of finalize steps
(``dsgb_output``), one per user-visible aggregate.  The fused append is the
CUDA kernel itself, which walks the base list for every row.

Base choice per reduction follows the reference's GPU/partitioned base
decomposition (reductions.py ``_build_bases``): sum -> (sum, count) with a
NaN mask at finalize (:1047-1051, 1091-1096), mean -> (sum, count)
(:1287-1288), first/last -> row-index selector + gather (:1352-1360),
where(max|min) -> an argmax/argmin {value, row} pair (:1929-1956 with the
first-row tie rule of :1178-1182, 1223-1227).  Antialiased lines use the
CPU append semantics of reductions.py (``_append_antialias*``) with the
global self_intersect / overwrite / two-stage flags of compiler.py:539-554
and antialias.py:30-58.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import torch

from . import _native as N
from . import reductions as rd


@dataclass(frozen=True)
class BaseSpec:
    op: int
    col: Optional[str]
    cat: Optional[str]      # name of the category-code column
    ncat: int
    flags: int = 0
    fold: int = 0           # two-stage plans over several lines: the stage-2 fold (DSGB_FOLD_*), 0 = none

    @property
    def elem_bytes(self):
        if self.op in (N.BASE_COUNT, N.BASE_AA_CNT0):
            return 4
        if self.op == N.BASE_ANY:
            return 1
        if self.op in (N.BASE_ARGMAX, N.BASE_ARGMIN, N.BASE_AA_ARGMAX):
            return 16
        return 8

    @property
    def torch_dtype(self):
        if self.op in (N.BASE_COUNT, N.BASE_AA_CNT0):
            return torch.uint32
        if self.op == N.BASE_ANY:
            return torch.uint8
        if self.op in (N.BASE_SUM, N.BASE_AA_SUM):
            return torch.float64
        return torch.int64

    @property
    def words(self):
        """int64 words per cell for pair bases (2), else 1."""
        return 2 if self.elem_bytes == 16 else 1


@dataclass
class OutSpec:
    fin: int                 # dsgb_fin_op, or 0 = the output is base b0 itself
    b0: int
    b1: int = -1
    col: Optional[str] = None
    dtype: torch.dtype = torch.float64
    categories: Optional[list] = None
    cat_dim: Optional[str] = None
    as_bool: bool = False


@dataclass
class Plan:
    bases: list
    outputs: list                 # [(key or None, OutSpec)]
    columns: list                 # value / category columns the kernels read
    antialias: bool = False
    self_intersect: bool = True
    overwrite: bool = True
    use_2_stage: bool = False
    derived: dict = field(default_factory=dict)   # name -> (column, modulo, offset)

    @property
    def is_dataset(self):
        return self.outputs and self.outputs[0][0] is not None


# AntialiasCombination (antialias.py:8-14)
_S1, _S2, _MIN, _MAX, _FIRST, _LAST = range(1, 7)


def _aa_combos(red, si):
    """Reduction._antialias_stage_2 of the CPU bases of ``red``."""
    if isinstance(red, rd.by):
        return _aa_combos(red.reduction, si)
    if isinstance(red, (rd.count, rd.sum, rd._sum_zero)):
        return [_S1 if si else _S2]
    if isinstance(red, rd.mean):
        return [_S1 if si else _S2] * 2
    if isinstance(red, (rd.any, rd.max, rd._max_row_index)):
        return [_MAX]
    if isinstance(red, (rd.min, rd._min_row_index)):
        return [_MIN]
    if isinstance(red, rd.first):
        return [_FIRST]
    if isinstance(red, rd.last):
        return [_LAST]
    if isinstance(red, rd.where):
        c = _aa_combos(red.selector, si)
        return c + c
    raise NotImplementedError(f"{type(red).__name__} reduction not implemented for antialiased lines")


def aa_stage_flags(agg):
    """(self_intersect, overwrite, use_2_stage_agg): compiler.py:539-554 + antialias.py:30-58."""
    reds = list(rd.traverse_aggregation(agg))
    si = not rd.builtins_any(r._antialias_requires_2_stages() for r in reds)
    combos = [c for r in reds for c in _aa_combos(r, si)]
    use_2 = rd.builtins_any(c in (_S2, _MIN, _FIRST, _LAST) for c in combos)
    overwrite = not rd.builtins_any(c == _S1 for c in combos)
    return si, overwrite, use_2


def _stage2_fold(red, si=False):
    """The stage-2 fold that a two-stage plan over several lines applies to the
    bases of ``red`` (compiler.py:153-196 with the combinations of
    reductions.py: count and sum SUM_2AGG, or SUM_1AGG when the plan keeps
    self_intersect (a two-stage plan whose only two-stage reductions are where,
    which does not ask for self_intersect=False, reductions.py:1842-1915): both
    combinations fold by nansum, so the additive self-intersecting bases (sum
    and count of the row mask) add up; any and max MAX, min MIN, first
    FIRST, last LAST, the row indexes MIN / MAX over -1; mean, _sum_zero and
    _count_ignore_antialiasing append additively in either mode and fold by
    SUM_2AGG over zeros, a plain sum; where folds its {selector, row} pair by
    the selector's own append, reductions.py:1992-2018)."""
    if isinstance(red, (rd._count_ignore_antialiasing, rd._sum_zero, rd.mean)):
        return N.FOLD_ADD
    if isinstance(red, rd.where):
        sel = red.selector
        if isinstance(sel, rd._min_row_index):
            return N.FOLD_ROW_MIN
        if isinstance(sel, rd._max_row_index):
            return N.FOLD_MAX
        for cls, fold in ((rd.max, N.FOLD_WHERE_MAX), (rd.min, N.FOLD_WHERE_MIN), (rd.first, N.FOLD_WHERE_FIRST),
                          (rd.last, N.FOLD_WHERE_LAST)):
            if isinstance(sel, cls):
                return fold
        return 0
    if isinstance(red, rd.count):
        return N.FOLD_ADD if si else N.FOLD_SUM_F32   # float32 aggregate (reductions.py:542-543)
    if isinstance(red, rd.any):
        return N.FOLD_MAX
    if isinstance(red, rd.sum) and not isinstance(red, rd._sum_zero):
        return N.FOLD_ADD if si else N.FOLD_SUM
    if isinstance(red, rd.max):
        return N.FOLD_MAX
    if isinstance(red, rd.min):
        return N.FOLD_MIN
    if isinstance(red, rd.first):
        return N.FOLD_FIRST
    if isinstance(red, rd.last):
        return N.FOLD_LAST
    if isinstance(red, rd._min_row_index):
        return N.FOLD_ROW_MIN
    if isinstance(red, rd._max_row_index):
        return N.FOLD_MAX
    return 0


class _Builder:
    def __init__(self, schema, antialias, si, use_2=False):
        self.schema = schema
        self.antialias = antialias
        self.si = si
        self.use_2 = use_2
        self.bases = []
        self.index = {}
        self.columns = []
        self.derived = {}

    def col(self, name):
        if name is None or name == rd.SpecialColumn.RowIndex:
            return None
        if name not in self.columns:
            self.columns.append(name)
        return name

    def base(self, op, col, cat, ncat, flags=0, fold=0):
        spec = BaseSpec(op, self.col(col), cat, ncat, flags, fold)
        if spec not in self.index:
            self.index[spec] = len(self.bases)
            self.bases.append(spec)
        return self.index[spec]

    def categorizer(self, by_red):
        cz = by_red.categorizer
        cats = cz.categories(self.schema)
        if isinstance(cz, rd.category_modulo):
            name = f"__category_modulo__{cz.column}__{cz.modulo}__{cz.offset}"
            self.derived[name] = (cz.column, cz.modulo, cz.offset)
        else:
            name = cz.column
        if name not in self.columns:
            self.columns.append(name)
        return name, len(cats), cats, cz.column

    def reduction(self, red, cat=None, ncat=1, categories=None, cat_dim=None):
        """OutSpec of one (possibly categorical) reduction."""
        if isinstance(red, rd.by):
            if cat is not None:
                raise NotImplementedError("nested by() reductions")
            name, n, cats, dim = self.categorizer(red)
            return self.reduction(red.reduction, name, n, cats, dim)
        kw = dict(categories=categories, cat_dim=cat_dim)
        fold = _stage2_fold(red, self.si) if (self.antialias and self.use_2) else 0
        B = lambda op, col, flags=0: self.base(op, col, cat, ncat, flags, fold)  # noqa: E731
        c = red.column if not isinstance(red, rd._max_or_min_row_index) else None
        aa = self.antialias
        if isinstance(red, rd._count_ignore_antialiasing):
            if aa:
                return OutSpec(0, B(N.BASE_AA_CNT0, c), dtype=torch.uint32, **kw)
            return OutSpec(0, B(N.BASE_COUNT, c), dtype=torch.uint32, **kw)
        if isinstance(red, rd.count):
            if not aa:
                return OutSpec(0, B(N.BASE_COUNT, c), dtype=torch.uint32, **kw)
            if self.si:    # reductions.py:560-569, 586-592: float32 sum of aa - prev
                return OutSpec(N.FIN_SUM_F32, B(N.BASE_AA_SUM, c, N.BASEF_UNWEIGHTED),
                               B(N.BASE_COUNT, c), dtype=torch.float32, **kw)
            return OutSpec(N.FIN_KEY_F32, B(N.BASE_AA_MAX, c, N.BASEF_UNWEIGHTED),
                           dtype=torch.float32, **kw)
        if isinstance(red, rd.any):
            if aa:         # reductions.py:848-852: float32 max of aa
                return OutSpec(N.FIN_KEY_F32, B(N.BASE_AA_MAX, c, N.BASEF_UNWEIGHTED),
                               dtype=torch.float32, **kw)
            return OutSpec(0, B(N.BASE_ANY, c), dtype=torch.uint8, as_bool=True, **kw)
        if isinstance(red, rd._sum_zero):
            return OutSpec(0, B(N.BASE_AA_SUM if aa else N.BASE_SUM, c), dtype=torch.float64, **kw)
        if isinstance(red, rd.sum):
            if aa and not self.si:   # reductions.py:1077-1084: max of field*aa
                return OutSpec(N.FIN_KEY_F64, B(N.BASE_AA_MAX, c), **kw)
            return OutSpec(N.FIN_SUM_NAN, B(N.BASE_AA_SUM if aa else N.BASE_SUM, c),
                           B(N.BASE_COUNT, c), **kw)
        if isinstance(red, rd.mean):
            if aa:
                return OutSpec(N.FIN_MEAN, B(N.BASE_AA_SUM, c), B(N.BASE_AA_CNT0, c), **kw)
            return OutSpec(N.FIN_MEAN, B(N.BASE_SUM, c), B(N.BASE_COUNT, c), **kw)
        if isinstance(red, (rd.max, rd.min, rd.first, rd.last)) and aa:
            # every antialiased max/min/first/last keeps the largest field*aa
            return OutSpec(N.FIN_KEY_F64, B(N.BASE_AA_MAX, c), **kw)
        if isinstance(red, rd.max):
            return OutSpec(N.FIN_KEY_F64, B(N.BASE_MAX, c), **kw)
        if isinstance(red, rd.min):
            return OutSpec(N.FIN_KEY_F64, B(N.BASE_MIN, c), **kw)
        if isinstance(red, rd.first):
            return OutSpec(N.FIN_GATHER, B(N.BASE_MIN_ROW, c), col=self.col(c), **kw)
        if isinstance(red, rd.last):
            return OutSpec(N.FIN_GATHER, B(N.BASE_MAX_ROW, c), col=self.col(c), **kw)
        if isinstance(red, rd._min_row_index):
            return OutSpec(N.FIN_ROW, B(N.BASE_MIN_ROW, None), dtype=torch.int64, **kw)
        if isinstance(red, rd._max_row_index):
            return OutSpec(N.FIN_ROW, B(N.BASE_MAX_ROW, None), dtype=torch.int64, **kw)
        if isinstance(red, rd.where):
            sel = red.selector
            sc = sel.column if not isinstance(sel, rd._max_or_min_row_index) else None
            if isinstance(sel, rd._min_row_index):
                b = B(N.BASE_MIN_ROW, None)
            elif isinstance(sel, rd._max_row_index):
                b = B(N.BASE_MAX_ROW, None)
            elif aa:
                b = B(N.BASE_AA_ARGMAX, sc)
            elif isinstance(sel, rd.max):
                b = B(N.BASE_ARGMAX, sc)
            elif isinstance(sel, rd.min):
                b = B(N.BASE_ARGMIN, sc)
            elif isinstance(sel, rd.first):
                b = B(N.BASE_MIN_ROW, sc)
            else:
                b = B(N.BASE_MAX_ROW, sc)
            if red.column == rd.SpecialColumn.RowIndex:
                return OutSpec(N.FIN_ROW, b, dtype=torch.int64, **kw)
            return OutSpec(N.FIN_GATHER, b, col=self.col(red.column), **kw)
        raise NotImplementedError(f"{type(red).__name__} is not supported on the GPU path")


_cache = {}


def compile_plan(agg, schema, *, antialias=False):
    """Flatten ``agg`` for ``schema`` (memoized like compile_components)."""
    key = (hash(agg), agg, schema.signature(), antialias)
    hit = _cache.get(key)
    if hit is not None:
        return hit
    if antialias:
        si, overwrite, use_2 = aa_stage_flags(agg)
    else:
        si, overwrite, use_2 = True, False, False
    b = _Builder(schema, antialias, si, use_2)
    if isinstance(agg, rd.summary):
        outs = [(k, b.reduction(v)) for k, v in zip(agg.keys, agg.values)]
    else:
        outs = [(None, b.reduction(agg))]
    if len(b.bases) > 16:
        raise NotImplementedError("more than 16 base accumulators in one pass")
    plan = Plan(b.bases, outs, b.columns, antialias, si, overwrite, use_2, b.derived)
    _cache[key] = plan
    return plan
