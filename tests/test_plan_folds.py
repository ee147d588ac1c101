"""Host logic of two-stage antialiased plans (no GPU): which plans are two-stage,
and the stage-2 fold each base of a compiled plan carries (compiler.py:153-268,
antialias.py:30-58 of the reference)."""
from __future__ import annotations

import pytest

import datashader_gb300 as ds
from datashader_gb300 import _native as N
from datashader_gb300.compiler import compile_plan


class _Schema:
    """A stand-in frame schema: float64 columns v, w and an int8 category column."""

    def signature(self):
        return (("v", "torch.float64", ()), ("w", "torch.float64", ()), ("cat", "torch.int8", (0, 1, 2)))

    def __contains__(self, name):
        return name in ("v", "w", "cat")

    def dtype_kind(self, name):
        return "i" if name == "cat" else "f"

    def is_categorical(self, name):
        return name == "cat"

    def categories(self, name):
        return [0, 1, 2]


S = _Schema()


def _folds(agg):
    plan = compile_plan(agg, S, antialias=True)
    return plan, {(b.op, b.fold) for b in plan.bases}


def test_single_stage_plans_carry_no_fold():
    for agg in (ds.count(), ds.sum("v"), ds.max("v"), ds.any(), ds.mean("v"), ds.where(ds.max("v"))):
        plan, folds = _folds(agg)
        assert not plan.use_2_stage
        assert all(f == 0 for _, f in folds)


@pytest.mark.parametrize("agg, want", [
    (ds.count(self_intersect=False), {(N.BASE_AA_MAX, N.FOLD_SUM_F32)}),
    (ds.sum("v", self_intersect=False), {(N.BASE_AA_MAX, N.FOLD_SUM)}),
    (ds.min("v"), {(N.BASE_AA_MAX, N.FOLD_MIN)}),
    (ds.first("v"), {(N.BASE_AA_MAX, N.FOLD_FIRST)}),
    (ds.last("v"), {(N.BASE_AA_MAX, N.FOLD_LAST)}),
    (ds._min_row_index(), {(N.BASE_MIN_ROW, N.FOLD_ROW_MIN)}),
    (ds.where(ds.min("v"), "w"), {(N.BASE_AA_ARGMAX, N.FOLD_WHERE_MIN)}),
    (ds.where(ds.first("v")), {(N.BASE_AA_ARGMAX, N.FOLD_WHERE_FIRST)}),
    (ds.where(ds.last("v")), {(N.BASE_AA_ARGMAX, N.FOLD_WHERE_LAST)}),
])
def test_two_stage_folds(agg, want):
    plan, folds = _folds(agg)
    assert plan.use_2_stage
    assert folds == want


def test_where_keeps_self_intersect_and_additive_count():
    """where does not ask for self_intersect=False (reductions.py:1842-1915): the plan
    is two-stage with self_intersect kept, so count and sum stay additive (SUM_1AGG,
    folded by nansum)."""
    plan, folds = _folds(ds.summary(c=ds.count(), s=ds.sum("v"), w=ds.where(ds.first("v"))))
    assert plan.use_2_stage and plan.self_intersect and not plan.overwrite
    assert (N.BASE_AA_SUM, N.FOLD_ADD) in folds and (N.BASE_COUNT, N.FOLD_ADD) in folds
    assert (N.BASE_AA_ARGMAX, N.FOLD_WHERE_FIRST) in folds


def test_mixed_summary_folds_and_distinct_bases():
    """max and min of one column keep separate bases once their folds differ; mean
    and _count_ignore_antialiasing fold additively."""
    plan, folds = _folds(ds.summary(mx=ds.max("v"), mn=ds.min("v"), m=ds.mean("w"),
                                    k=ds._count_ignore_antialiasing("v")))
    assert plan.use_2_stage and not plan.self_intersect
    assert {(N.BASE_AA_MAX, N.FOLD_MAX), (N.BASE_AA_MAX, N.FOLD_MIN)} <= folds
    assert (N.BASE_AA_SUM, N.FOLD_ADD) in folds and (N.BASE_AA_CNT0, N.FOLD_ADD) in folds
    assert len([b for b in plan.bases if b.op == N.BASE_AA_MAX]) == 2


def test_categorical_two_stage_fold():
    plan, folds = _folds(ds.by("cat", ds.first("v")))
    assert plan.use_2_stage and folds == {(N.BASE_AA_MAX, N.FOLD_FIRST)}
    assert plan.bases[0].ncat == 3
