"""Tile-service driver (datashader/tiles.py): web-mercator tile sets written
as ``output_path/z/x/y.png``.

Flow per zoom level, as in the reference (tiles.py:70-130): the extent is
cut into super tiles of up to 16x16 tiles (gen_super_tiles); each super
tile is rasterised once by the caller's ``rasterize_func`` (normally this
package's Canvas.points on the GPU); the colour span of the level is the
minimum and maximum over every super tile's aggregate (calculate_zoom_level
_stats, reduced on the device by dsgb_bounds); each super tile is shaded by
the caller's ``shader_func`` with that span and cut into its 256x256 tiles
by pixel-centre coordinates (TileRenderer.render), rows flipped so that y
grows downward, and written out.

GB300 specifics: the aggregates and the shaded super tile stay on the
device; one device-to-host copy per super tile feeds the tile encoder.
Super tiles render one after another on the GPU stream, so dask (which the
reference needs to parallelise them on CPU workers) is not used.  Pillow
is used for images when it is installed; without it tiles are RGBA
``RGBAImage`` objects and PNG files are written with zlib (JPG needs
Pillow).  S3 output (S3TileRenderer) and the Bokeh tile previewer are out
of scope.
"""
from __future__ import annotations

import ctypes
import math
import os
import struct
import zlib
from importlib.util import find_spec

import numpy as np
import torch

from . import _native as N
from .core import dsgb_dtype

__all__ = ["render_tiles", "MercatorTileDefinition"]


# ---------------------------------------------------------------- helpers

def _create_dir(path):
    os.makedirs(path, exist_ok=True)


def uint32_to_uint8(img):
    """utils.py:1012-1014: a uint32 raster viewed as H x W x 4 RGBA bytes."""
    return img.view(dtype=np.uint8).reshape(img.shape + (4,))


def invert_y_tile(y, z):
    """TMS <-> Google tile row (tiles.py:133-135)."""
    return (2 ** z) - 1 - y


def _device_minmax(t):
    """NaN-skipping (min, max) of a device tensor (dsgb_bounds)."""
    t = t.contiguous().reshape(-1)
    col = N.Column(t.data_ptr(), dsgb_dtype(t), 0)
    out = torch.empty(2, dtype=torch.float64, device=t.device)
    N.check(N.lib().dsgb_bounds(ctypes.byref(col), t.numel(), out.data_ptr(),
                                torch.cuda.current_stream(t.device).cuda_stream), "dsgb_bounds")
    mn, mx = out.cpu().tolist()
    return mn, mx


# ------------------------------------------------------------ tile driver

def _get_super_tile_min_max(tile_info, load_data_func, rasterize_func):
    """The aggregate of one super tile (tiles.py:35-41)."""
    size = tile_info["tile_size"]
    df = load_data_func(tile_info["x_range"], tile_info["y_range"])
    return rasterize_func(df, x_range=tile_info["x_range"], y_range=tile_info["y_range"],
                          height=size, width=size)


def calculate_zoom_level_stats(super_tiles, load_data_func, rasterize_func, color_ranging_strategy="fullscan"):
    """Rasterise every super tile of a level and take the colour span
    (tiles.py:44-67): (0, 1) for boolean aggregates, else the minimum and
    maximum over the super tiles' NaN-skipping minima and maxima."""
    if color_ranging_strategy != "fullscan":
        raise ValueError("Invalid color_ranging_strategy option")
    lows, highs = [], []
    is_bool = False
    for st in super_tiles:
        agg = _get_super_tile_min_max(st, load_data_func, rasterize_func)
        st["agg"] = agg
        if agg.dtype == torch.bool:
            is_bool = True
            continue
        mn, mx = _device_minmax(agg.data)
        if math.isfinite(mn):
            lows.append(mn)
        if math.isfinite(mx):
            highs.append(mx)
    if is_bool:
        return super_tiles, (0, 1)
    if not lows:
        return super_tiles, (math.nan, math.nan)
    return super_tiles, (min(lows), max(highs))


def render_tiles(full_extent, levels, load_data_func, rasterize_func, shader_func, post_render_func, output_path,
                 color_ranging_strategy="fullscan"):
    """Render the tiles of ``levels`` over ``full_extent`` (xmin, ymin, xmax,
    ymax in web-mercator metres) into ``output_path/z/x/y.png``
    (tiles.py:70-87).  Returns {level: {success, stats, supertile_count}}."""
    results = {}
    for level in levels:
        print(f"calculating statistics for level {level}")
        super_tiles, span = calculate_zoom_level_stats(list(gen_super_tiles(full_extent, level)), load_data_func,
                                                       rasterize_func, color_ranging_strategy=color_ranging_strategy)
        print(f"rendering {len(super_tiles)} supertiles for zoom level {level} with span={span}")
        for st in super_tiles:
            render_super_tile(st, span, output_path, shader_func, post_render_func)
            st.pop("agg", None)                  # release the device aggregate
        results[level] = dict(success=True, stats=span, supertile_count=len(super_tiles))
    return results


def gen_super_tiles(extent, zoom_level, span=None):
    """Super tiles of a level: up to 16x16 tiles each (tiles.py:90-104)."""
    xmin, ymin, xmax, ymax = extent
    size = min(16 * 256, (2 ** zoom_level) * 256)
    sdef = MercatorTileDefinition(x_range=(xmin, xmax), y_range=(ymin, ymax), tile_size=size)
    for _, _, _, (sx0, sy0, sx1, sy1) in sdef.get_tiles_by_extent(extent, zoom_level):
        yield {"level": zoom_level, "x_range": (sx0, sx1), "y_range": (sy0, sy1), "tile_size": sdef.tile_size,
               "span": span}


def render_super_tile(tile_info, span, output_path, shader_func, post_render_func):
    """Shade one super tile with the level's span and write its tiles (tiles.py:107-110)."""
    img = shader_func(tile_info["agg"], span=span)
    return create_sub_tiles(img, tile_info["level"], tile_info, output_path, post_render_func)


def create_sub_tiles(data_array, level, tile_info, output_path, post_render_func=None):
    """tiles.py:113-130: the 256x256 tiles of one shaded super tile."""
    _create_dir(output_path)
    tdef = MercatorTileDefinition(x_range=tile_info["x_range"], y_range=tile_info["y_range"], tile_size=256)
    if output_path.startswith("s3:"):
        raise NotImplementedError("S3 tile output is not supported")
    renderer = FileSystemTileRenderer(tdef, output_location=output_path, post_render_func=post_render_func)
    return renderer.render(data_array, level=level)


# ------------------------------------------------------ tile definition

class MercatorTileDefinition:
    """Web-mercator tile scheme (tiles.py:138-292): level z has 2^z x 2^z
    tiles of ``tile_size`` pixels; the resolution (metres a pixel) at level z
    is initial_resolution / 2^z, measured from the origin offsets; tile rows
    count downward (Google scheme), TMS rows upward."""

    def __init__(self, x_range, y_range, tile_size=256, min_zoom=0, max_zoom=30,
                 x_origin_offset=20037508.34, y_origin_offset=20037508.34,
                 initial_resolution=156543.03392804097):
        self.x_range = x_range
        self.y_range = y_range
        self.tile_size = tile_size
        self.min_zoom = min_zoom
        self.max_zoom = max_zoom
        self.x_origin_offset = x_origin_offset
        self.y_origin_offset = y_origin_offset
        self.initial_resolution = initial_resolution
        self._resolutions = [self._get_resolution(z) for z in range(min_zoom, max_zoom + 1)]

    def to_ogc_tile_metadata(self, output_file_path):
        """Not written by the reference either (tiles.py:196-200)."""
        return None

    def to_esri_tile_metadata(self, output_file_path):
        """Not written by the reference either (tiles.py:202-206)."""
        return None

    def is_valid_tile(self, x, y, z):
        n = 2 ** z
        return 0 <= x < n and 0 <= y < n

    def _get_resolution(self, z):
        return self.initial_resolution / (2 ** z)

    def get_resolution_by_extent(self, extent, height, width):
        return [(extent[2] - extent[0]) / width, (extent[3] - extent[1]) / height]

    def get_level_by_extent(self, extent, height, width):
        """The deepest level whose resolution is at least the extent's (the
        coarser of its x and y resolutions), or 0 (tiles.py:226-240)."""
        resolution = max(self.get_resolution_by_extent(extent, height, width))
        for i, r in enumerate(self._resolutions):
            if resolution > r:
                return max(i - 1, 0)
        return len(self._resolutions) - 1

    def pixels_to_meters(self, px, py, level):
        res = self._get_resolution(level)
        return (px * res) - self.x_origin_offset, (py * res) - self.y_origin_offset

    def meters_to_pixels(self, mx, my, level):
        res = self._get_resolution(level)
        return (mx + self.x_origin_offset) / res, (my + self.y_origin_offset) / res

    def pixels_to_tile(self, px, py, level):
        """Tile column and Google row of a pixel (tiles.py:254-259): the column
        is ceil(px / size) - 1 except that 0 stays 0, the TMS row is
        max(ceil(py / size) - 1, 0)."""
        tx = math.ceil(px / self.tile_size)
        if tx != 0:
            tx -= 1
        ty = max(math.ceil(py / self.tile_size) - 1, 0)
        return int(tx), invert_y_tile(int(ty), level)

    def pixels_to_raster(self, px, py, level):
        return px, (self.tile_size << level) - py

    def meters_to_tile(self, mx, my, level):
        px, py = self.meters_to_pixels(mx, my, level)
        return self.pixels_to_tile(px, py, level)

    def get_tiles_by_extent(self, extent, level):
        """(tx, ty, level, (xmin, ymin, xmax, ymax)) of every valid tile that
        meets the extent, rows top to bottom (tiles.py:269-284)."""
        xmin, ymin, xmax, ymax = extent
        txmin, tymax = self.meters_to_tile(xmin, ymin, level)   # y metres grow up, Google rows down
        txmax, tymin = self.meters_to_tile(xmax, ymax, level)
        return [(tx, ty, level, self.get_tile_meters(tx, ty, level))
                for ty in range(tymin, tymax + 1) for tx in range(txmin, txmax + 1)
                if self.is_valid_tile(tx, ty, level)]

    def get_tile_meters(self, tx, ty, level):
        ty = invert_y_tile(ty, level)
        x0, y0 = self.pixels_to_meters(tx * self.tile_size, ty * self.tile_size, level)
        x1, y1 = self.pixels_to_meters((tx + 1) * self.tile_size, (ty + 1) * self.tile_size, level)
        return x0, y0, x1, y1


# ----------------------------------------------------------- renderers

class RGBAImage:
    """A tile image when Pillow is absent: ``data`` is H x W x 4 uint8 (RGBA),
    ``save`` writes PNG."""

    def __init__(self, data):
        self.data = np.ascontiguousarray(data, dtype=np.uint8)

    @property
    def width(self):
        return self.data.shape[1]

    @property
    def height(self):
        return self.data.shape[0]

    def save(self, fp, format="PNG"):
        if str(format).upper() != "PNG":
            raise ValueError("only PNG tiles can be written without Pillow")
        payload = encode_png(self.data)
        if hasattr(fp, "write"):
            fp.write(payload)
        else:
            with open(fp, "wb") as f:
                f.write(payload)


def encode_png(rgba):
    """PNG bytes of an H x W x 4 uint8 image: 8-bit RGBA, no interlace, every
    scanline with filter type 0, one zlib-compressed IDAT chunk."""
    rgba = np.ascontiguousarray(rgba, dtype=np.uint8)
    h, w = rgba.shape[:2]
    rows = np.zeros((h, 1 + 4 * w), dtype=np.uint8)
    rows[:, 1:] = rgba.reshape(h, 4 * w)

    def chunk(tag, body):
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(rows.tobytes(), 6)) + chunk(b"IEND", b""))


def _label_slice(coords, lo, hi):
    """Index range of the (increasing) coordinates within [lo, hi], as label
    slicing selects them."""
    return int(np.searchsorted(coords, lo, side="left")), int(np.searchsorted(coords, hi, side="right"))


class TileRenderer:
    """Cuts a shaded super tile into the tiles of its definition (tiles.py:295-339)."""

    def __init__(self, tile_definition, output_location, tile_format="PNG", post_render_func=None):
        self.tile_def = tile_definition
        self.output_location = output_location
        self.tile_format = tile_format
        self.post_render_func = post_render_func
        self._pil = find_spec("PIL") is not None
        if self.tile_format not in ("PNG", "JPG"):
            raise ValueError("Invalid output format")
        if self.tile_format == "JPG" and not self._pil:
            raise ImportError("pillow is required to write JPG tiles")

    def render(self, da, level):
        xmin, xmax = self.tile_def.x_range
        ymin, ymax = self.tile_def.y_range
        tiles = self.tile_def.get_tiles_by_extent((xmin, ymin, xmax, ymax), level)
        xs = np.asarray(da.coords[da.dims[1]], dtype=np.float64)
        ys = np.asarray(da.coords[da.dims[0]], dtype=np.float64)
        data = da.data.cpu().numpy() if isinstance(da.data, torch.Tensor) else np.asarray(da.data)
        for x, y, z, (dx0, dy0, dx1, dy1) in tiles:
            c0, c1 = _label_slice(xs, dx0, dx1)
            r0, r1 = _label_slice(ys, dy0, dy1)
            arr = data[r0:r1, c0:c1]
            if 0 in arr.shape:
                continue
            arr = np.flip(arr, 0)                        # tile rows go down
            if arr.ndim == 2 and arr.dtype == np.uint32:
                arr = uint32_to_uint8(np.ascontiguousarray(arr))
            if self._pil:
                from PIL.Image import fromarray
                img = fromarray(np.ascontiguousarray(arr))
            else:
                img = RGBAImage(arr)
            if self.post_render_func:
                img = self.post_render_func(img, x=x, y=y, z=z)
            yield img, x, y, z


class FileSystemTileRenderer(TileRenderer):
    """Writes each tile to ``output_location/z/x/y.<format>`` (tiles.py:391-400)."""

    def render(self, da, level):
        for img, x, y, z in super().render(da, level):
            directory = os.path.join(self.output_location, str(z), str(x))
            _create_dir(directory)
            img.save(os.path.join(directory, f"{y}.{self.tile_format.lower()}"), self.tile_format)
