"""Reduction objects with datashader's public names and arguments.

Mirrors datashader/reductions.py for the reductions on the GPU hot path:
count, any, sum, mean, min, max, first, last, where, by / count_cat,
summary, the internal _sum_zero, _count_ignore_antialiasing,
_min_row_index and _max_row_index, and the categorizers category_codes /
category_modulo.  Each reduction knows how to validate itself against a
source schema (column names -> dtype, categories); the GPU plan that
implements it is produced by :mod:`datashader_gb300.compiler`.
"""
from __future__ import annotations

from enum import Enum

import numpy as np


class SpecialColumn(Enum):
    """reductions.py:45-55: RowIndex is the virtual row-index column."""
    RowIndex = 1


_NUMERIC_KINDS = set("biuf")


class Expr:
    """Hashable by type and inputs (utils.py:61-92)."""

    def _hashable_inputs(self):
        return tuple(self.inputs_key())

    def inputs_key(self):
        return (getattr(self, "column", None),)

    def __hash__(self):
        return hash((type(self), self._hashable_inputs()))

    def __eq__(self, other):
        return type(self) is type(other) and self._hashable_inputs() == other._hashable_inputs()


class CategoryPreprocess(Expr):
    def __init__(self, column):
        self.column = column

    @property
    def cat_column(self):
        return self.column


class category_codes(CategoryPreprocess):
    """Category codes of a categorical column (reductions.py:143-169)."""

    def categories(self, schema):
        return list(schema.categories(self.column))

    def validate(self, schema):
        if self.column not in schema:
            raise ValueError("specified column not found")
        if not schema.is_categorical(self.column):
            raise ValueError("input must be categorical")


class category_modulo(category_codes):
    """(column - offset) % modulo on an integer column (reductions.py:171-206)."""

    def __init__(self, column, modulo, offset=0):
        super().__init__(column)
        self.modulo = int(modulo)
        self.offset = offset

    def inputs_key(self):
        return (self.column, self.modulo, self.offset)

    def categories(self, schema):
        return list(range(self.modulo))

    def validate(self, schema):
        if self.column not in schema:
            raise ValueError("specified column not found")
        if schema.dtype_kind(self.column) not in "biu":
            raise ValueError("input must be an integer column")


class Reduction(Expr):
    """Base class for per-bin reductions (reductions.py:299-470)."""

    def __init__(self, column=None):
        self.column = column

    def validate(self, schema):
        if self.column == SpecialColumn.RowIndex:
            return
        if self.column not in schema:
            raise ValueError("specified column not found")
        if schema.dtype_kind(self.column) not in _NUMERIC_KINDS:
            raise ValueError("input must be numeric")

    def is_categorical(self):
        return False

    def uses_row_index(self):
        return False

    def _antialias_requires_2_stages(self):
        return False

    def __repr__(self):
        return f"{type(self).__name__}({self.column!r})"


class OptionalFieldReduction(Reduction):
    def validate(self, schema):
        if self.column is not None:
            super().validate(schema)


class SelfIntersectingOptionalFieldReduction(OptionalFieldReduction):
    def __init__(self, column=None, self_intersect=True):
        super().__init__(column)
        self.self_intersect = self_intersect

    def inputs_key(self):
        return (self.column, self.self_intersect)

    def _antialias_requires_2_stages(self):
        return not self.self_intersect


class count(SelfIntersectingOptionalFieldReduction):
    """Count elements in each bin: uint32, or float32 with antialiased lines
    (reductions.py:532-664)."""

    def __repr__(self):
        return "count()" if self.column is None else f"count({self.column!r})"


class _count_ignore_antialiasing(count):
    """Count that ignores antialiasing, used by mean (reductions.py:667-693)."""


class any(OptionalFieldReduction):
    """Whether any elements map to each bin (reductions.py:824-889)."""


class FloatingReduction(Reduction):
    pass


class _sum_zero(FloatingReduction):
    """Sum with a zero initial value (reductions.py:938-996)."""


class SelfIntersectingFloatingReduction(FloatingReduction):
    def __init__(self, column=None, self_intersect=True):
        super().__init__(column)
        self.self_intersect = self_intersect

    def inputs_key(self):
        return (self.column, self.self_intersect)

    def _antialias_requires_2_stages(self):
        return not self.self_intersect


class sum(SelfIntersectingFloatingReduction):
    """Sum of the non-NaN values in each bin, NaN where nothing landed
    (reductions.py:1030-1098)."""


class min(FloatingReduction):
    """Minimum non-NaN value; the first row wins ties (reductions.py:1160-1213)."""

    def _antialias_requires_2_stages(self):
        return True


class max(FloatingReduction):
    """Maximum non-NaN value; the first row wins ties (reductions.py:1216-1260)."""


class mean(Reduction):
    """Mean of the non-NaN values (reductions.py:1280-1297)."""


class _first_or_last(Reduction):
    def uses_row_index(self):
        return True

    def _antialias_requires_2_stages(self):
        return True


class first(_first_or_last):
    """First non-NaN value in row order (reductions.py:1375-1412)."""


class last(_first_or_last):
    """Last non-NaN value in row order (reductions.py:1415-1454)."""


class _max_or_min_row_index(OptionalFieldReduction):
    def __init__(self):
        super().__init__(column=SpecialColumn.RowIndex)

    def uses_row_index(self):
        return True

    def __repr__(self):
        return f"{type(self).__name__}()"


class _max_row_index(_max_or_min_row_index):
    """Largest row index in each bin, -1 where empty (reductions.py:2251-2307)."""


class _min_row_index(_max_or_min_row_index):
    """Smallest row index in each bin, -1 where empty (reductions.py:2310-2372)."""

    def _antialias_requires_2_stages(self):
        return True


class where(FloatingReduction):
    """Value of ``lookup_column`` (or the row index) at the row chosen by
    ``selector`` (reductions.py:1842-2166)."""

    def __init__(self, selector, lookup_column=None):
        if not isinstance(selector, (first, last, max, min, _max_or_min_row_index)):
            raise TypeError("selector can only be a first, first_n, last, last_n, "
                            "max, max_n, min or min_n reduction")
        if lookup_column is None:
            lookup_column = SpecialColumn.RowIndex
        super().__init__(lookup_column)
        self.selector = selector
        self.columns = (selector.column, lookup_column)

    def inputs_key(self):
        return (self.column, hash(self.selector))

    def uses_row_index(self):
        return True

    def validate(self, schema):
        if self.column != SpecialColumn.RowIndex:
            super().validate(schema)
        self.selector.validate(schema)
        if self.column != SpecialColumn.RowIndex and self.column == self.selector.column:
            raise ValueError("where and its contained reduction cannot use the same column")

    def __repr__(self):
        return f"where(selector={self.selector!r}, lookup_column={self.column!r})"


class by(Reduction):
    """Apply ``reduction`` separately per category (reductions.py:696-823)."""

    def __init__(self, cat_column, reduction=None):
        super().__init__()
        if reduction is None:
            reduction = count()
        if isinstance(cat_column, CategoryPreprocess):
            self.categorizer = cat_column
        elif isinstance(cat_column, str):
            self.categorizer = category_codes(cat_column)
        else:
            raise TypeError("first argument must be a column name or a CategoryPreprocess instance")
        self.column = self.categorizer.column
        self.reduction = reduction
        cols = getattr(reduction, "columns", None)
        self.columns = (self.categorizer.column,) + (tuple(cols[::-1]) if cols is not None
                                                     else (getattr(reduction, "column", None),))

    def inputs_key(self):
        return (hash(self.categorizer), hash(self.reduction))

    @property
    def cat_column(self):
        return self.columns[0]

    @property
    def val_column(self):
        return self.columns[1]

    def is_categorical(self):
        return True

    def uses_row_index(self):
        return self.reduction.uses_row_index()

    def _antialias_requires_2_stages(self):
        return self.reduction._antialias_requires_2_stages()

    def validate(self, schema):
        self.categorizer.validate(schema)
        self.reduction.validate(schema)

    def __repr__(self):
        return f"{type(self).__name__}(column={self.column!r}, reduction={self.reduction!r})"


class count_cat(by):
    """Alias for by(column, count()) (reductions.py:1263-1278)."""

    def __init__(self, column):
        super().__init__(column, count())

    def __repr__(self):
        return f"count_cat(column={self.column!r})"


class summary(Expr):
    """Several named reductions computed in one pass, keys sorted
    (reductions.py:2169-2233)."""

    def __init__(self, **kwargs):
        ks, vs = zip(*sorted(kwargs.items()))
        self.keys = ks
        self.values = vs

    def __hash__(self):
        return hash((type(self), tuple(self.keys), tuple(self.values)))

    def __eq__(self, other):
        return type(self) is type(other) and self.keys == other.keys and self.values == other.values

    def is_categorical(self):
        return builtins_any(v.is_categorical() for v in self.values)

    def uses_row_index(self):
        return builtins_any(v.uses_row_index() for v in self.values)

    def validate(self, schema):
        for v in self.values:
            v.validate(schema)

    def __repr__(self):
        return "summary(" + ", ".join(f"{k}={v!r}" for k, v in zip(self.keys, self.values)) + ")"


def builtins_any(it):
    for v in it:
        if v:
            return True
    return False


def traverse_aggregation(agg):
    """compiler.py:557-563 -- left-to-right traversal of a reduction tree."""
    if isinstance(agg, summary):
        for a in agg.values:
            yield from traverse_aggregation(a)
    else:
        yield agg


__all__ = [
    "SpecialColumn", "Reduction", "count", "any", "sum", "mean", "min", "max", "first", "last",
    "where", "by", "count_cat", "summary", "_sum_zero", "_count_ignore_antialiasing",
    "_min_row_index", "_max_row_index", "category_codes", "category_modulo",
]

# keep numpy referenced for categorizer users
_ = np
