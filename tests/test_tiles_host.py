"""Tile-service driver host logic and the compositing oracle (no GPU).

* the compositing oracle against every assertion of the reference's
  test_composite.py (tests/golden/composite.json);
* MercatorTileDefinition against the reference's test_meters_to_tile and
  the tile arithmetic it implies (tiles.py:138-292);
* super tiles per level, the PNG encoder (decoded back with zlib) and the
  cutting of a shaded super tile into flipped 256x256 tiles (tiles.py:295-400).
"""
from __future__ import annotations

import json
import os
import struct
import zlib

import numpy as np
import pytest
import torch

from datashader_gb300 import tiles as T
from datashader_gb300.core import Aggregate
from oracle import composite as C

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_composite_oracle_matches_reference_vectors():
    cases = json.load(open(os.path.join(GOLD, "composite.json")))["cases"]
    assert len(cases) == 21
    for c in cases:
        src = np.array(c["src"], dtype=np.uint32).reshape(c["shape"])
        got = C.OPS[c["op"]](src, np.uint32(c["dst"]))
        want = np.array(c["expected"], dtype=np.uint32).reshape(c["shape"])
        assert np.array_equal(got, want), (c["op"], c["source"])


def test_meters_to_tile_reference_case():
    g = json.load(open(os.path.join(GOLD, "tiles.json")))["meters_to_tile"]
    xmin, ymin, xmax, ymax = g["extent"]
    tdef = T.MercatorTileDefinition((xmin, xmax), (ymin, ymax), tile_size=256)
    assert tdef.meters_to_tile(xmin, ymin, g["zoom"]) == tuple(g["expected"])


def test_tile_scheme_round_trips():
    world = 20037508.34
    tdef = T.MercatorTileDefinition((-world, world), (-world, world))
    for z in range(0, 6):
        tiles = tdef.get_tiles_by_extent((-world, -world, world, world), z)
        assert len(tiles) == 4 ** z
        for tx, ty, zz, (x0, y0, x1, y1) in tiles:
            assert zz == z and x0 < x1 and y0 < y1
            # the centre of a tile maps back to that tile (Google rows)
            assert tdef.meters_to_tile((x0 + x1) / 2, (y0 + y1) / 2, z) == (tx, ty)
        # row 0 is the top of the map
        top = [t for t in tiles if t[1] == 0]
        assert all(t[3][3] == max(u[3][3] for u in tiles) for t in top)
    assert tdef.get_level_by_extent((-world, -world, world, world), 256, 256) == 0
    assert tdef.get_level_by_extent((0, 0, 1000, 1000), 256, 256) == 15
    assert not tdef.is_valid_tile(-1, 0, 3) and not tdef.is_valid_tile(0, 8, 3) and tdef.is_valid_tile(7, 7, 3)
    assert T.invert_y_tile(0, 3) == 7


def test_super_tiles_per_level():
    world = 20037508.34
    ext = (-world, -world, world, world)
    for z, count, size in ((0, 1, 256), (3, 1, 2048), (4, 1, 4096), (5, 4, 4096), (6, 16, 4096)):
        sts = list(T.gen_super_tiles(ext, z))
        assert len(sts) == count
        assert all(s["tile_size"] == size and s["level"] == z for s in sts)


def _decode_png(payload):
    assert payload[:8] == b"\x89PNG\r\n\x1a\n"
    pos, chunks = 8, {}
    while pos < len(payload):
        (n,) = struct.unpack(">I", payload[pos:pos + 4])
        tag, body = payload[pos + 4:pos + 8], payload[pos + 8:pos + 8 + n]
        (crc,) = struct.unpack(">I", payload[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(tag + body) & 0xFFFFFFFF
        chunks[tag] = chunks.get(tag, b"") + body
        pos += 12 + n
    w, h, depth, ctype = struct.unpack(">IIBB", chunks[b"IHDR"][:10])
    assert (depth, ctype) == (8, 6)
    raw = np.frombuffer(zlib.decompress(chunks[b"IDAT"]), dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 4)


def test_png_encoder_round_trip():
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, (37, 53, 4), dtype=np.uint8)
    assert np.array_equal(_decode_png(T.encode_png(img)), img)


def _fake_image(x_range, y_range, size, seed=0):
    rng = np.random.default_rng(seed)
    data = rng.integers(0, 2 ** 32, (size, size), dtype=np.uint64).astype(np.uint32)
    xs = x_range[0] + (np.arange(size) + 0.5) * (x_range[1] - x_range[0]) / size
    ys = y_range[0] + (np.arange(size) + 0.5) * (y_range[1] - y_range[0]) / size
    return Aggregate(torch.from_numpy(data.view(np.int32)).view(torch.uint32), ["y", "x"], {"x": xs, "y": ys},
                     {}), data


@pytest.mark.parametrize("level", [1, 3])
def test_sub_tiles_cut_flipped_and_written(tmp_path, level, monkeypatch):
    world = 20037508.34
    monkeypatch.setattr(T, "find_spec", lambda name: None)         # the zlib PNG path, Pillow or not
    for st in T.gen_super_tiles((-world, -world, world, world), level):
        img, data = _fake_image(st["x_range"], st["y_range"], st["tile_size"], seed=level)
        T.create_sub_tiles(img, level, st, str(tmp_path))
        n = st["tile_size"] // 256
        tdef = T.MercatorTileDefinition(st["x_range"], st["y_range"], tile_size=256)
        tiles = tdef.get_tiles_by_extent((st["x_range"][0], st["y_range"][0], st["x_range"][1], st["y_range"][1]),
                                         level)
        assert len(tiles) == n * n
        for tx, ty, z, _ in tiles:
            got = _decode_png((tmp_path / str(z) / str(tx) / f"{ty}.png").read_bytes())
            # tile column tx, Google row ty of the super tile: rows flipped (y grows down in tiles)
            col = tx - min(t[0] for t in tiles)
            row = ty - min(t[1] for t in tiles)
            block = data[::-1][row * 256:(row + 1) * 256, col * 256:(col + 1) * 256]
            assert np.array_equal(got, T.uint32_to_uint8(np.ascontiguousarray(block)))
