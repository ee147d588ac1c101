"""Extract golden vectors from the reference's own test files into JSON fixtures.

Reads (as text, via ``ast``; nothing from the reference is imported or run):

* ``datashader/tests/test_pandas.py``      -- the antialiased-line solution
  arrays (``line_antialias_sol_*``, ``line_antialias_nan_sol_*``), the
  ``line_antialias_df`` input frame and the LineAxis0 entry of
  ``line_antialias_nan_params``;
* ``datashader/tests/test_pandas.py`` -- the multi-line cases of
  ``line_manual_range_params`` / ``line_autorange_params`` (ragged-array
  entries skipped) and the ``sol`` arrays of ``test_line_manual_range``,
  ``test_line_autorange``, ``test_line_autorange_axis1_x_constant``,
  ``test_line_autorange_axis1_ragged`` and
  ``test_line_agg_sum_axis1_none_constant`` (with its frame);
* ``datashader/tests/test_transfer_functions.py`` -- ``eq_hist_sol`` and
  ``eq_hist_sol_rescale_discrete_levels`` (uint32 RGBA images), the
  linear / log / cbrt ``solution_lists`` and the ``sol`` arrays of
  ``test_span_cmap_single`` and ``test_shade_cmap``;
* ``datashader/tests/test_composite.py`` -- every ``assert_equal(op(src,
  dst), o)`` of the source / over / add / saturate tests: the module's
  literal ``src`` and colours, each test body's numpy statements on ``o``
  replayed in order (they are plain numpy on literals), the operator under
  test never called;
* ``datashader/tests/test_tiles.py`` -- the extent, zoom and expected tile
  of ``test_meters_to_tile``;
* ``datashader/tests/data/test_00{1..7}_{antialias,noaa}_{normal,clipped}.png``
  -- the shaded images of ``test_antialias.py`` (the PNG files the test module
  writes beside its NetCDF copies), decoded with zlib and the PNG filters of
  the PNG specification and stored as uint32 RGBA in aggregate orientation
  (row 0 = y minimum: the PNG rows flipped back, as ``Image.to_pil`` flips them).

Usage::

    python tests/golden/make_golden.py /path/to/reference

The output files (``tests/golden/*.json``) are committed; the GPU machine never
needs the reference checkout.
"""
from __future__ import annotations

import ast
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class _FakePd:
    """Stand-in for the ``pd`` names the literal expressions use."""

    @staticmethod
    def DataFrame(data=None, dtype=None, **kw):
        data = dict(data if data is not None else kw)
        return {k: np.asarray(v, dtype=dtype) if dtype else np.asarray(v) for k, v in data.items()}

    @staticmethod
    def array(v, dtype=None):
        return v


def _literal_assignments(path, wanted_prefixes, extra_names=()):
    src = open(path).read()
    tree = ast.parse(src)
    ns = {"np": np, "nan": np.nan, "pd": _FakePd, "sp": None}
    out = {}
    for node in tree.body:
        if not isinstance(node, ast.Assign) or len(node.targets) != 1:
            continue
        tgt = node.targets[0]
        if isinstance(tgt, ast.Name):
            name = tgt.id
            if name.startswith(wanted_prefixes) or name in extra_names:
                code = compile(ast.Expression(node.value), path, "eval")
                ns[name] = eval(code, ns)  # literal numpy expressions only
                out[name] = (ns[name], node.lineno)
        elif isinstance(tgt, ast.Subscript) and isinstance(tgt.value, ast.Name):
            # e.g. eq_hist_sol_rescale_discrete_levels['c'] = ...['b']
            name = tgt.value.id
            if name in out:
                code = compile(ast.Module([node], []), path, "exec")
                exec(code, ns)
    return out


def _jsonable(a):
    a = np.asarray(a)
    if a.dtype.kind == "f":
        return {"dtype": str(a.dtype), "shape": list(a.shape),
                "data": [None if np.isnan(v) else float(v) for v in a.ravel()]}
    return {"dtype": str(a.dtype), "shape": list(a.shape), "data": [int(v) for v in a.ravel()]}


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _decode_png_rgba(path):
    """8-bit RGBA PNG -> uint8 [h][w][4] (filter types 0-4 of the PNG specification)."""
    import struct
    import zlib
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(data):
        (n,) = struct.unpack(">I", data[pos:pos + 4])
        tag = data[pos + 4:pos + 8]
        chunks[tag] = chunks.get(tag, b"") + data[pos + 8:pos + 8 + n]
        pos += 12 + n
    w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", chunks[b"IHDR"])
    assert (depth, ctype, interlace) == (8, 6, 0), (depth, ctype, interlace)
    raw = zlib.decompress(chunks[b"IDAT"])
    stride, bpp = 4 * w, 4
    out = np.zeros((h, stride), dtype=np.int64)
    prev = [0] * stride
    for y in range(h):
        ftype = raw[y * (stride + 1)]
        line = raw[y * (stride + 1) + 1:(y + 1) * (stride + 1)]
        cur = [0] * stride
        for i in range(stride):
            a = cur[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            pred = (0, a, b, (a + b) // 2, _paeth(a, b, c))[ftype]
            cur[i] = (line[i] + pred) & 0xFF
        out[y] = cur
        prev = cur
    return out.astype(np.uint8).reshape(h, w, 4)


def _antialias_images(tests):
    images = {}
    for t in range(1, 8):
        for aa in ("antialias", "noaa"):
            for cv in ("normal", "clipped"):
                name = f"test_{t:03d}_{aa}_{cv}"
                rgba = _decode_png_rgba(os.path.join(tests, "data", name + ".png"))
                u32 = np.ascontiguousarray(np.flipud(rgba)).view("<u4")[..., 0]
                images[name] = dict(_jsonable(u32), source=f"datashader/tests/data/{name}.png")
    return images


def main(ref_root):
    tests = os.path.join(ref_root, "datashader", "tests")
    pandas_path = os.path.join(tests, "test_pandas.py")
    found = _literal_assignments(
        pandas_path, ("line_antialias_sol_", "line_antialias_nan_sol_"),
        extra_names=("line_antialias_df", "line_antialias_nan_params"))
    goldens = {}
    for name, (val, line) in found.items():
        if name == "line_antialias_df":
            goldens[name] = {"source": f"datashader/tests/test_pandas.py:{line}",
                             "columns": {k: _jsonable(v) for k, v in val.items()}}
        elif name == "line_antialias_nan_params":
            frame, kw, sol_false, sol_true = val[0]   # the LineAxis0 entry
            goldens["line_antialias_nan_axis0"] = {
                "source": f"datashader/tests/test_pandas.py:{line}",
                "columns": {k: _jsonable(np.asarray(v, dtype=frame.get("dtype", "float64")))
                            for k, v in frame["data"].items()},
                "sol_self_intersect_false": _jsonable(sol_false),
                "sol_self_intersect_true": _jsonable(sol_true)}
        else:
            goldens[name] = dict(_jsonable(val), source=f"datashader/tests/test_pandas.py:{line}")
    with open(os.path.join(HERE, "line_antialias.json"), "w") as f:
        json.dump(goldens, f, indent=0)

    tf_path = os.path.join(tests, "test_transfer_functions.py")
    found = _literal_assignments(tf_path, ("eq_hist_sol",))
    eq = {}
    for name, (val, line) in found.items():
        src = f"datashader/tests/test_transfer_functions.py:{line}"
        if isinstance(val, dict):
            eq[name] = {k: dict(_jsonable(v), source=src) for k, v in val.items()}
        else:
            eq[name] = dict(_jsonable(val), source=src)
    with open(os.path.join(HERE, "eq_hist.json"), "w") as f:
        json.dump(eq, f, indent=0)

    lines = {}
    for name, (val, line) in _literal_assignments(pandas_path, ("line_manual_range_params",
                                                                "line_autorange_params")).items():
        cases = []
        for df_args, kw in val:
            if isinstance(kw.get("x"), str) and isinstance(kw.get("y"), str) and kw.get("axis") == 1:
                # ragged arrays: per-row vertex lists
                cols = {k: [[float(v) for v in row] for row in vals] for k, vals in df_args[0].items()}
                cases.append({"columns": cols, "kwargs": dict(kw), "ragged": True})
                continue
            cols = {k: [float(v) for v in vals] for k, vals in df_args[0].items()}
            kwj = {k: ({"array": [float(v) for v in np.ravel(v)]} if isinstance(v, np.ndarray) else v)
                   for k, v in kw.items()}
            cases.append({"columns": cols, "kwargs": kwj})
        lines[name] = {"source": f"datashader/tests/test_pandas.py:{line}", "cases": cases}
    for fn, sols in _function_all_sols(pandas_path, ("test_line_manual_range", "test_line_autorange",
                                                     "test_line_autorange_axis1_x_constant",
                                                     "test_line_agg_sum_axis1_none_constant",
                                                     "test_line_autorange_axis1_ragged")).items():
        lines[fn] = [dict(_jsonable(np.asarray(v)), source=f"datashader/tests/test_pandas.py:{ln}") for v, ln in sols]
    with open(os.path.join(HERE, "lines_multi.json"), "w") as f:
        json.dump(lines, f, indent=0)

    shade = {}
    for name, (val, line) in _literal_assignments(tf_path, ("solution_lists",)).items():
        src = f"datashader/tests/test_transfer_functions.py:{line}"
        shade[name] = {how: dict(_jsonable(np.array(v, dtype="u4")), source=src) for how, v in val.items()}
    for fn, (val, line) in _function_sols(tf_path, ("test_span_cmap_single", "test_shade_cmap")).items():
        shade[fn] = dict(_jsonable(np.array(val, dtype="u4")), source=f"datashader/tests/test_transfer_functions.py:{line}")
    with open(os.path.join(HERE, "shade.json"), "w") as f:
        json.dump(shade, f, indent=0)
    comp = _composite_cases(os.path.join(tests, "test_composite.py"))
    with open(os.path.join(HERE, "composite.json"), "w") as f:
        json.dump(comp, f, indent=0)
    tiles = _meters_to_tile_case(os.path.join(tests, "test_tiles.py"))
    with open(os.path.join(HERE, "tiles.json"), "w") as f:
        json.dump(tiles, f, indent=0)
    aa_images = _antialias_images(tests)
    with open(os.path.join(HERE, "antialias_images.json"), "w") as f:
        json.dump(aa_images, f, indent=0)
    print("wrote", sorted(goldens), sorted(eq), sorted(shade), sorted(lines), len(comp["cases"]), "composite cases",
          sorted(tiles))


def _meters_to_tile_case(path):
    """Literal extent, zoom and asserted tile of test_meters_to_tile."""
    tree = ast.parse(open(path).read())
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name == "test_meters_to_tile":
            env = {}
            for st in node.body:
                if (isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name)
                        and st.targets[0].id in ("full_extent_of_data", "zoom")):
                    env[st.targets[0].id] = ast.literal_eval(st.value)
                elif isinstance(st, ast.Assert) and isinstance(st.test, ast.Compare):
                    env["expected"] = ast.literal_eval(st.test.comparators[0])
                    env["source"] = f"datashader/tests/test_tiles.py:{st.lineno}"
            return {"meters_to_tile": {"extent": list(env["full_extent_of_data"]), "zoom": env["zoom"],
                                       "expected": list(env["expected"]), "source": env["source"]}}
    raise ValueError("test_meters_to_tile not found")


def _composite_cases(path):
    """(operator, src, dst, expected) of each assertion in test_composite.py."""
    tree = ast.parse(open(path).read())
    ns = {"np": np}
    for node in tree.body:                       # module literals: src and the colours
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Name):
            exec(compile(ast.Module([node], type_ignores=[]), path, "exec"), ns)
    cases = []
    for node in tree.body:
        if not (isinstance(node, ast.FunctionDef) and node.name.startswith("test_")):
            continue
        env = dict(ns)
        for st in node.body:
            if isinstance(st, ast.Assign):         # o = ..., o[...] = ...: numpy on literals
                exec(compile(ast.Module([st], type_ignores=[]), path, "exec"), env)
            elif isinstance(st, ast.Expr) and isinstance(st.value, ast.Call):
                call = st.value
                fn = ast.unparse(call.func)
                if fn != "np.testing.assert_equal":
                    continue
                op_call, want = call.args
                op = op_call.func.id
                src = eval(compile(ast.Expression(op_call.args[0]), path, "eval"), env)
                dst = eval(compile(ast.Expression(op_call.args[1]), path, "eval"), env)
                exp = eval(compile(ast.Expression(want), path, "eval"), env)
                cases.append({"op": op, "src": np.asarray(src, dtype=np.uint32).ravel().tolist(),
                              "shape": list(np.shape(src)), "dst": int(np.uint32(dst)),
                              "expected": np.asarray(exp, dtype=np.uint32).ravel().tolist(),
                              "source": f"datashader/tests/test_composite.py:{st.lineno}"})
    return {"cases": cases}


def _function_all_sols(path, names):
    """Every literal ``sol = np.array(...)`` inside each named test function, in source order."""
    tree = ast.parse(open(path).read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            found = []
            for st in ast.walk(node):
                if (isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name) and st.targets[0].id == "sol"
                        and isinstance(st.value, ast.Call)):
                    code = compile(ast.Expression(st.value), path, "eval")
                    found.append((eval(code, {"np": np, "nan": np.nan}), st.lineno))
            out[node.name] = sorted(found, key=lambda t: t[1])
    return out


def _function_sols(path, names):
    """The first literal ``sol = np.array(...)`` inside each named test function."""
    tree = ast.parse(open(path).read())
    out = {}
    for node in tree.body:
        if isinstance(node, ast.FunctionDef) and node.name in names:
            for st in node.body:
                if (isinstance(st, ast.Assign) and isinstance(st.targets[0], ast.Name) and st.targets[0].id == "sol"
                        and isinstance(st.value, ast.Call)):
                    code = compile(ast.Expression(st.value), path, "eval")
                    out[node.name] = (eval(code, {"np": np}), st.lineno)
                    break
    return out


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
