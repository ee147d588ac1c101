"""Glyphs on the GPU path: Point, LineAxis0 and the multi-line layouts.

Mirrors datashader/glyphs/points.py (_PointLike 98-151, Point 156-242) and
datashader/glyphs/line.py (_AntiAliasedLine 28-41, LineAxis0 59-103,
LineAxis0Multi 106-196, LinesAxis1 197-264, LinesAxis1XConstant 309-381,
LinesAxis1YConstant 383-430).  The extend loops themselves live in libdsgb
(points.cu, line.cu).
"""
from __future__ import annotations


class _PointLike:
    def __init__(self, x, y):
        self.x = x
        self.y = y

    @property
    def x_label(self):
        return self.x

    @property
    def y_label(self):
        return self.y

    def required_columns(self):
        return [self.x, self.y]

    def validate(self, schema):
        """points.py:116-121: x and y must be numeric columns."""
        for c in (self.x, self.y):
            if c not in schema:
                raise ValueError(f"column {c!r} not found")
            if schema.dtype_kind(c) not in "iuf":
                raise ValueError("x and y must be real")

    def __hash__(self):
        return hash((type(self), self.x, self.y))

    def __eq__(self, other):
        return type(self) is type(other) and (self.x, self.y) == (other.x, other.y)


class Point(_PointLike):
    """A point, with center at ``x`` and ``y``; points on the upper bounds
    map into the previous bin (points.py:156-168)."""


class LineAxis0(_PointLike):
    """A line, with vertices defined by ``x`` and ``y`` (line.py:59-103)."""

    antialiased = False
    line_width = 0

    def set_line_width(self, line_width):
        """line.py:31-35."""
        self.line_width = line_width
        self.antialiased = line_width > 0


class _MultiLine:
    """Multi-line glyphs (line.py:106-196, 197-430): several x / y columns,
    or a constant numpy array for one of the two.  ``layout`` is the
    dsgb_lines layout (1: lines run down the rows, 2: one line per row)."""

    antialiased = False
    line_width = 0
    layout = 0

    def __init__(self, x, y):
        self.x = x
        self.y = y

    x_label = "x"
    y_label = "y"

    def set_line_width(self, line_width):
        self.line_width = line_width
        self.antialiased = line_width > 0

    def _names(self, v):
        return [] if _is_array(v) else list(v)

    def required_columns(self):
        return self._names(self.x) + self._names(self.y)

    def validate(self, schema):
        for c in self.required_columns():
            if c not in schema:
                raise ValueError(f"column {c!r} not found")
            if schema.dtype_kind(c) not in "iuf":
                raise ValueError("x and y columns must be real")
        nx = len(self.x)
        ny = len(self.y)
        if nx != ny:
            raise ValueError(f"x and y coordinate lengths do not match: {nx} != {ny}")

    def __hash__(self):
        return hash((type(self), tuple(map(_key, (self.x, self.y)))))

    def __eq__(self, other):
        return type(self) is type(other) and _key(self.x) == _key(other.x) and _key(self.y) == _key(other.y)


def _is_array(v):
    return hasattr(v, "shape") and hasattr(v, "dtype")


def _key(v):
    return tuple(v.tolist()) if _is_array(v) else tuple(v)


class LineAxis0Multi(_MultiLine):
    """Several lines, column j of ``x`` and ``y`` running down the rows (line.py:106-196)."""
    layout = 1


class LinesAxis1(_MultiLine):
    """One line per row through the columns of ``x`` and ``y`` (line.py:197-264)."""
    layout = 2


class LinesAxis1XConstant(LinesAxis1):
    """One line per row; ``x`` is one numpy array shared by every line (line.py:309-381)."""


class LinesAxis1YConstant(LinesAxis1):
    """One line per row; ``y`` is one numpy array shared by every line (line.py:383-430)."""


class LinesAxis1Ragged(_MultiLine):
    """One line per row through ragged x and y columns (RaggedColumn; line.py:457-523)."""
    layout = 3

    def required_columns(self):
        return [self.x, self.y]

    def validate(self, schema):
        for c, name in ((self.x, "x"), (self.y, "y")):
            if c not in schema:
                raise ValueError(f"column {c!r} not found")
            if schema.dtype_kind(c) != "R":
                raise ValueError(f"{name} must be a RaggedArray")

    def __hash__(self):
        return hash((type(self), self.x, self.y))

    def __eq__(self, other):
        return type(self) is type(other) and self.x == other.x and self.y == other.y
