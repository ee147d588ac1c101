"""Compositing kernel and the tile-service driver on the GPU.

* dsgb_composite against every assertion of the reference's
  test_composite.py and against the compositing oracle on random images
  (bit-exact: float64 in the reference's order), through tf.stack and
  tf.set_background as well;
* render_tiles end to end: each written PNG equals the tile cut from the
  oracle's super-tile image (oracle counts -> oracle linear shading with the
  level's span -> oracle 'over' black), and the level's span equals the
  minimum / maximum of the oracle's super-tile aggregates.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest
import torch

import datashader_gb300 as ds
import oracle
from datashader_gb300 import tiles as T
from datashader_gb300 import transfer_functions as tf
from oracle import composite as C

from test_tiles_host import _decode_png

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _u32(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.uint32).view(np.int32)).cuda().view(torch.uint32)


def _np(t):
    return t.view(torch.int32).cpu().numpy().view(np.uint32)


def test_composite_kernel_matches_reference_vectors():
    for c in json.load(open(os.path.join(GOLD, "composite.json")))["cases"]:
        src = np.array(c["src"], dtype=np.uint32).reshape(c["shape"])
        got = _np(tf._composite(_u32(src), c["dst"], c["op"]))
        assert np.array_equal(got, np.array(c["expected"], dtype=np.uint32).reshape(c["shape"])), c["source"]


@pytest.mark.parametrize("op", ["source", "over", "add", "saturate"])
def test_composite_kernel_vs_oracle_random(op):
    rng = np.random.default_rng(7)
    n = 1_000_003                                               # ragged tail after the 4-pixel vectors
    src = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    dst = rng.integers(0, 2 ** 32, n, dtype=np.uint64).astype(np.uint32)
    # alphas that hit the edge cases: 0, 255 and equal / complementary pairs
    src[::5] &= 0x00FFFFFF
    dst[::7] |= 0xFF000000
    dst[1::11] = (dst[1::11] & 0x00FFFFFF) | ((255 - (src[1::11] >> 24)) << 24)
    assert np.array_equal(_np(tf._composite(_u32(src), _u32(dst), op)), C.OPS[op](src, dst))
    # one background value for every pixel, and unaligned buffers (the scalar loop)
    assert np.array_equal(_np(tf._composite(_u32(src), 0x80402010, op)), C.OPS[op](src, np.uint32(0x80402010)))
    s1 = _u32(src)[1:]
    d1 = _u32(dst)[1:]
    assert np.array_equal(_np(tf._composite(s1, d1, op)), C.OPS[op](src[1:], dst[1:]))


def test_stack_and_set_background():
    rng = np.random.default_rng(8)
    imgs = [rng.integers(0, 2 ** 32, (64, 96), dtype=np.uint64).astype(np.uint32) for _ in range(3)]
    gi = [tf.Image(_u32(a), ["y", "x"], {"x": np.arange(96.0), "y": np.arange(64.0)}, {}) for a in imgs]
    for how in ("over", "add", "saturate", "source"):
        want = imgs[0]
        for a in imgs[1:]:
            want = C.OPS[how](a, want)
        assert np.array_equal(_np(tf.stack(*gi, how=how).data), want)
    bg = tf.set_background(gi[1], "black")
    assert np.array_equal(_np(bg.data), C.over(imgs[1], np.uint32(0xFF000000)))
    assert tf.set_background(gi[1]) is gi[1]
    with pytest.raises(ValueError):
        tf.stack(*gi, how="nope")
    with pytest.raises(ValueError):
        tf.stack(gi[0], tf.Image(_u32(imgs[0][:10]), ["y", "x"], {}, {}))


CMAP = ["#440154", "#21918c", "#fde725"]


def test_render_tiles_end_to_end(tmp_path):
    rng = np.random.default_rng(9)
    n = 2_000_000
    x = rng.normal(0, 500000, n)
    y = rng.normal(0, 500000, n)
    frame = ds.TensorFrame({"x": torch.from_numpy(x).cuda(), "y": torch.from_numpy(y).cuda()})
    aggs = {}

    def load(x_range, y_range):
        return frame

    def rasterize(df, x_range, y_range, height, width):
        return ds.Canvas(plot_width=width, plot_height=height, x_range=x_range, y_range=y_range).points(df, "x", "y")

    def shader(agg, span=None):
        return tf.set_background(tf.shade(agg, cmap=CMAP, span=span, how="linear"), "black")

    seen = []

    def post(img, **kw):
        seen.append((kw["x"], kw["y"], kw["z"], img.width, img.height))
        return img

    extent = (-500000, -500000, 500000, 500000)
    levels = [0, 1, 2, 5]
    checked = 0
    res = T.render_tiles(extent, levels, load, rasterize, shader, post, str(tmp_path))
    assert sorted(res) == levels
    for z in levels:
        assert res[z]["success"] and res[z]["supertile_count"] >= 1
        sts = list(T.gen_super_tiles(extent, z))
        assert res[z]["supertile_count"] == len(sts)
        # the oracle's super tiles, their span, and every written tile
        ref_aggs = [oracle.points({"x": x, "y": y}, "x", "y", st["tile_size"], st["tile_size"], st["x_range"],
                                  st["y_range"], [oracle.spec("count")])[0] for st in sts]
        span = (min(float(a.min()) for a in ref_aggs), max(float(a.max()) for a in ref_aggs))
        assert tuple(res[z]["stats"]) == span
        for st, ragg in zip(sts, ref_aggs):
            img = C.over(oracle.shade_interp(ragg, how="linear", cmap=CMAP, span=span), np.uint32(0xFF000000))
            size = st["tile_size"]
            xs = st["x_range"][0] + (np.arange(size) + 0.5) * (st["x_range"][1] - st["x_range"][0]) / size
            ys = st["y_range"][0] + (np.arange(size) + 0.5) * (st["y_range"][1] - st["y_range"][0]) / size
            tdef = T.MercatorTileDefinition(st["x_range"], st["y_range"], tile_size=256)
            for tx, ty, zz, (dx0, dy0, dx1, dy1) in tdef.get_tiles_by_extent(
                    (st["x_range"][0], st["y_range"][0], st["x_range"][1], st["y_range"][1]), z):
                c0, c1 = np.searchsorted(xs, dx0), np.searchsorted(xs, dx1, side="right")
                r0, r1 = np.searchsorted(ys, dy0), np.searchsorted(ys, dy1, side="right")
                if r1 == r0 or c1 == c0:
                    continue        # a neighbour's tile (the scheme lists one row past the lower edge)
                want = T.uint32_to_uint8(np.ascontiguousarray(img[r0:r1, c0:c1][::-1]))
                got = _decode_png((tmp_path / str(zz) / str(tx) / f"{ty}.png").read_bytes())
                checked += 1
                assert np.array_equal(got, want), (z, tx, ty)
    assert checked == len(seen) == 1 + 4 + 16 + 1024                 # every tile written, each checked once
    assert {(t[2]) for t in seen} == set(levels) and all(t[3] == t[4] == 256 for t in seen)
