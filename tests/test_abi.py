"""The C-ABI library builds, loads and exports every symbol include/dsgb.h declares (no GPU)."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

from datashader_gb300 import _native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "dsgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(dsgb_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_header_and_python_list_agree():
    assert _declared_functions() == sorted(N.EXPORTED)


def test_library_loads_and_exports_every_symbol():
    L = N.lib()
    for name in _declared_functions():
        assert hasattr(L, name), name
        assert ctypes.cast(getattr(L, name), ctypes.c_void_p).value


def test_abi_version_and_error_string():
    L = N.lib()
    assert L.dsgb_abi_version() == 2
    assert isinstance(L.dsgb_last_error(), bytes)


def test_argument_errors_return_codes_without_a_gpu():
    """Invalid arguments are rejected on the host before any CUDA call."""
    L = N.lib()
    cv = N.CanvasDesc(0, 0, 0, 0, 1, 0, 1, 0, 0, 1, 0, 1)
    rc = L.dsgb_points(None, 0, 10, 0, 0, 1, ctypes.byref(cv), None, 0, None, 0, 0, None)
    assert rc == -1
    assert b"invalid" in L.dsgb_last_error()
    rc = L.dsgb_eq_hist_u32(None, 0, 0, None, None, None, None, 0, 255, 0, None, 0, None)
    assert rc == -1
    assert L.dsgb_device_status(None, 1) == -1


def test_struct_layouts_match_header():
    assert ctypes.sizeof(N.Column) == 16
    assert ctypes.sizeof(N.CanvasDesc) == 16 + 8 * 8
    assert ctypes.sizeof(N.Base) == 32
    assert ctypes.sizeof(N.Output) == 24


def test_plan_compiler_bases(tmp_path):
    """Host logic: the reduction tree flattens to deduplicated bases."""
    import numpy as np
    import datashader_gb300 as ds
    from datashader_gb300.compiler import compile_plan

    class Schema:
        cols = {"x": "f", "y": "f", "v": "f", "cat": "c"}

        def __contains__(self, k):
            return k in self.cols

        def dtype_kind(self, k):
            return self.cols[k]

        def is_categorical(self, k):
            return k == "cat"

        def categories(self, k):
            return ["a", "b", "c"]

        def signature(self):
            return ("test",)

    agg = ds.summary(s=ds.sum("v"), m=ds.mean("v"), c=ds.count("v"), b=ds.by("cat", ds.count()))
    plan = compile_plan(agg, Schema())
    ops = [(b.op, b.col, b.cat) for b in plan.bases]
    assert ops.count((N.BASE_SUM, "v", None)) == 1
    assert ops.count((N.BASE_COUNT, "v", None)) == 1
    assert (N.BASE_COUNT, None, "cat") in ops
    assert len(plan.bases) == 3
    assert np.all([o.b0 >= 0 for _, o in plan.outputs])


@pytest.mark.parametrize("spec,flags", [
    ("sum", (True, False, False)), ("max", (True, True, False)),
    ("min", (False, True, True)), ("count_no_si", (False, True, True)),
])
def test_antialias_stage_flags(spec, flags):
    """compiler.py:539-554 + antialias.py:30-58 host logic."""
    import datashader_gb300 as ds
    from datashader_gb300.compiler import aa_stage_flags
    agg = {"sum": ds.sum("v"), "max": ds.max("v"), "min": ds.min("v"),
           "count_no_si": ds.count(self_intersect=False)}[spec]
    assert aa_stage_flags(agg) == flags
