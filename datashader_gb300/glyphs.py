"""Glyphs on the GPU path: Point and LineAxis0.

Mirrors datashader/glyphs/points.py (_PointLike 98-151, Point 156-242) and
datashader/glyphs/line.py (_AntiAliasedLine 28-41, LineAxis0 59-103).  The
extend loops themselves live in libdsgb (points.cu, line.cu).
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
