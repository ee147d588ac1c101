"""tf.shade (how='eq_hist' | 'linear' | 'log' | 'cbrt') and eq_hist on the GPU.

Mirrors datashader/transfer_functions/__init__.py: shade (616-745) for 2-D
aggregates, the _interpolate prologue (251-297), eq_hist (148-223),
_rescale_discrete_levels (234-248), the linear / log / cbrt interpolators
(220-223) and the list-colormap and single-colour RGBA branches (317-351).
Each shade is one libdsgb call (eq_hist.cu, shade.cu); matplotlib colormap
callables and categorical (3-D) shading are outside the GPU path.
"""
from __future__ import annotations

import ctypes

import torch

from . import _native as N
from .core import Aggregate

# CSS named colours (the subset most used with datashader palettes).
_CSS = {
    "aliceblue": "#F0F8FF", "antiquewhite": "#FAEBD7", "aqua": "#00FFFF", "aquamarine": "#7FFFD4",
    "azure": "#F0FFFF", "beige": "#F5F5DC", "black": "#000000", "blue": "#0000FF",
    "blueviolet": "#8A2BE2", "brown": "#A52A2A", "cadetblue": "#5F9EA0", "chartreuse": "#7FFF00",
    "coral": "#FF7F50", "cornflowerblue": "#6495ED", "crimson": "#DC143C", "cyan": "#00FFFF",
    "darkblue": "#00008B", "darkcyan": "#008B8B", "darkgray": "#A9A9A9", "darkgreen": "#006400",
    "darkgrey": "#A9A9A9", "darkorange": "#FF8C00", "darkred": "#8B0000", "darkviolet": "#9400D3",
    "deeppink": "#FF1493", "deepskyblue": "#00BFFF", "dodgerblue": "#1E90FF", "firebrick": "#B22222",
    "forestgreen": "#228B22", "fuchsia": "#FF00FF", "gold": "#FFD700", "gray": "#808080",
    "green": "#008000", "greenyellow": "#ADFF2F", "grey": "#808080", "hotpink": "#FF69B4",
    "indigo": "#4B0082", "ivory": "#FFFFF0", "khaki": "#F0E68C", "lavender": "#E6E6FA",
    "lightblue": "#ADD8E6", "lightcoral": "#F08080", "lightcyan": "#E0FFFF", "lightgray": "#D3D3D3",
    "lightgreen": "#90EE90", "lightgrey": "#D3D3D3", "lightpink": "#FFB6C1", "lightyellow": "#FFFFE0",
    "lime": "#00FF00", "magenta": "#FF00FF", "maroon": "#800000", "navy": "#000080",
    "olive": "#808000", "orange": "#FFA500", "orangered": "#FF4500", "orchid": "#DA70D6",
    "pink": "#FFC0CB", "plum": "#DDA0DD", "purple": "#800080", "red": "#FF0000",
    "royalblue": "#4169E1", "salmon": "#FA8072", "seagreen": "#2E8B57", "silver": "#C0C0C0",
    "skyblue": "#87CEEB", "steelblue": "#4682B4", "tan": "#D2B48C", "teal": "#008080",
    "tomato": "#FF6347", "turquoise": "#40E0D0", "violet": "#EE82EE", "white": "#FFFFFF",
    "yellow": "#FFFF00", "yellowgreen": "#9ACD32",
}


def rgb(x):
    """colors.py:99-128: colour name, '#RRGGBB' or an (r, g, b) tuple."""
    if isinstance(x, str):
        h = x if x.startswith("#") else _CSS.get(x)
        if h is None:
            raise ValueError(f"Unknown color: '{x}'")
        if not (h.startswith("#") and len(h) == 7):
            raise ValueError("Invalid hex color")
        return int(h[1:3], 16), int(h[3:5], 16), int(h[5:7], 16)
    if isinstance(x, tuple) and len(x) == 3:
        if min(x) < 0 or max(x) > 255:
            raise ValueError("Invalid RGB tuple")
        return x
    raise TypeError(f"Don't know how to convert {x} to RGB")


class Image(Aggregate):
    """A uint32 RGBA image (transfer_functions/__init__.py:25-58)."""


_WS = {}


def _workspace(device, nbins):
    size = int(N.lib().dsgb_eq_hist_workspace_size(nbins))
    key = (device, nbins)
    t = _WS.get(key)
    if t is None or t.numel() < size:
        t = torch.empty(size, dtype=torch.uint8, device=device)
        _WS[key] = t
    return t


def _run_eq_hist(data, nbins=256 * 256, cmap=None, alpha=255, rescale_discrete_levels=False,
                 stream=None):
    """One libdsgb eq_hist call.  Returns (equalised f64, levels tensor, rgba or None)."""
    if data.dtype == torch.uint32:
        fn = N.lib().dsgb_eq_hist_u32
    elif data.dtype == torch.float64:
        fn = N.lib().dsgb_eq_hist_f64
    else:
        raise NotImplementedError(f"eq_hist on the GPU path takes uint32 or float64 aggregates, not {data.dtype}")
    data = data.contiguous()
    dev = data.device
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    out = torch.empty(data.shape, dtype=torch.float64, device=dev)
    levels = torch.empty(1, dtype=torch.int64, device=dev)
    rgba = None
    cmap_buf = None
    ncol = 0
    if cmap is not None:
        cols = [rgb(c) for c in cmap]
        if not 1 <= len(cols) <= 256:
            raise ValueError("colormap must have 1..256 colours")
        ncol = len(cols)
        cmap_buf = (ctypes.c_double * (3 * ncol))(*[float(v) for c in cols for v in c])
        rgba = torch.empty(data.shape, dtype=torch.uint32, device=dev)
    ws = _workspace(dev, nbins)
    rc = fn(data.data_ptr(), data.numel(), nbins, out.data_ptr(), levels.data_ptr(),
            rgba.data_ptr() if rgba is not None else None, cmap_buf, ncol, int(alpha),
            int(bool(rescale_discrete_levels)), ws.data_ptr(), ws.numel(), stream)
    N.check(rc, "dsgb_eq_hist")
    return out, levels, rgba


def eq_hist_agg(agg, nbins=256 * 256):
    """The eq_hist step of shade: mask (0 / NaN), offset, equalise.

    Returns (equalised float64 tensor with NaN where masked, discrete_levels)."""
    data = agg.data if isinstance(agg, Aggregate) else agg
    out, levels, _ = _run_eq_hist(data, nbins)
    return out, int(levels.item())


_HOW_CODE = {"linear": 0, "log": 1, "cbrt": 2}


def _run_shade(data, how, cmap, alpha, min_alpha, span, stream=None):
    """One libdsgb shade call (how in linear / log / cbrt).  Returns the RGBA tensor."""
    if data.dtype == torch.uint32:
        fn = N.lib().dsgb_shade_u32
    elif data.dtype == torch.float64:
        fn = N.lib().dsgb_shade_f64
    else:
        raise NotImplementedError(f"shade on the GPU path takes uint32 or float64 aggregates, not {data.dtype}")
    data = data.contiguous()
    dev = data.device
    if stream is None:
        stream = torch.cuda.current_stream(dev).cuda_stream
    single = isinstance(cmap, str) or (isinstance(cmap, tuple) and len(cmap) == 3 and
                                       not isinstance(cmap[0], str))
    cmap_buf, ncol, single_buf = None, 0, None
    if single:
        single_buf = (ctypes.c_uint8 * 3)(*rgb(cmap))
    else:
        cols = [rgb(c) for c in cmap]
        if not 1 <= len(cols) <= 256:
            raise ValueError("colormap must have 1..256 colours")
        ncol = len(cols)
        cmap_buf = (ctypes.c_double * (3 * ncol))(*[float(v) for c in cols for v in c])
    span_buf = (ctypes.c_double * 2)(float(span[0]), float(span[1])) if span is not None else None
    rgba = torch.empty(data.shape, dtype=torch.uint32, device=dev)
    size = int(N.lib().dsgb_shade_workspace_size())
    ws = _WS.get(("shade", dev))
    if ws is None:
        ws = torch.empty(size, dtype=torch.uint8, device=dev)
        _WS[("shade", dev)] = ws
    N.check(fn(data.data_ptr(), data.numel(), _HOW_CODE[how], span_buf, cmap_buf, ncol, single_buf, int(alpha),
               int(min_alpha), rgba.data_ptr(), ws.data_ptr(), ws.numel(), stream), "dsgb_shade")
    return rgba


def _check_cmap(cmap):
    """Colour validation before any device work: colors.rgb's ValueError /
    TypeError for an unknown colour (colors.py:99-126), and a ValueError for an
    empty list (the reference fails unpacking its channels,
    transfer_functions/__init__.py:317-320)."""
    if isinstance(cmap, str) or (isinstance(cmap, tuple) and len(cmap) == 3 and not isinstance(cmap[0], str)):
        rgb(cmap)
        return
    if isinstance(cmap, (list, tuple)):
        if len(cmap) == 0:
            raise ValueError("not enough values to unpack: the colormap is empty")
        for c in cmap:
            rgb(c)


def _shade_input(data):
    """The aggregate as the kernels take it: uint32 or float64.  A bool
    aggregate (any()) becomes 0 / 1 uint32, which masks and offsets exactly as
    the reference's bool prologue (mask = ~data, data as int8, offset 1:
    transfer_functions/__init__.py:263-268); a float32 one (antialiased count /
    any) is widened to float64 exactly (the reference subtracts the offset and
    applies log1p / cbrt in float32, so those steps can differ in the last
    float32 bit, one colour step at most)."""
    if data.dtype == torch.bool:
        return data.to(torch.int32).view(torch.uint32)
    if data.dtype == torch.float32:
        return data.to(torch.float64)
    return data


def shade(agg, cmap=("lightblue", "darkblue"), color_key=None, how="eq_hist", alpha=255,
          min_alpha=40, span=None, name=None, color_baseline=None, rescale_discrete_levels=False):
    """tf.shade for a 2-D aggregate (transfer_functions/__init__.py:616-745):
    how in eq_hist / linear / log / cbrt; a list colormap, or one colour with
    an alpha ramp (linear / log / cbrt)."""
    if not isinstance(agg, Aggregate):
        raise TypeError("agg must be instance of DataArray")
    name = agg.name if name is None else name
    if not ((0 <= min_alpha <= 255) and (0 <= alpha <= 255)):
        raise ValueError(f"min_alpha ({min_alpha}) and alpha ({alpha}) must be between 0 and 255")
    if agg.ndim != 2:
        raise NotImplementedError("only 2-D aggregates are shaded on the GPU path")
    _check_cmap(cmap)
    data = _shade_input(agg.data)
    if how in _HOW_CODE:
        if span is not None and not span[0] <= span[1]:
            raise ValueError("span must be (low, high)")
        rgba = _run_shade(data, how, cmap, alpha, min_alpha, span)
        return Image(rgba, agg.dims, agg.coords, agg.attrs, name=name)
    if how != "eq_hist":
        raise ValueError(f"Unknown interpolation method: {how}")
    if span is not None:
        raise ValueError("span is not (yet) valid to use with eq_hist")
    if isinstance(cmap, str) or not isinstance(cmap, (list, tuple)):
        raise NotImplementedError("only list colormaps are on the GPU path")
    _, _, rgba = _run_eq_hist(data, cmap=list(cmap), alpha=alpha,
                              rescale_discrete_levels=rescale_discrete_levels)
    return Image(rgba, agg.dims, agg.coords, agg.attrs, name=name)


# ---------------------------------------------------------------- compositing

_COMPOSITE = {"source": 0, "over": 1, "add": 2, "saturate": 3}


def _composite(src, dst, how):
    """op(src, dst) per pixel on the GPU (dsgb_composite): dst is a tensor of
    src's shape or one uint32 pixel value."""
    if how not in _COMPOSITE:
        ops = ", ".join(repr(k) for k in _COMPOSITE)
        raise ValueError(f"Operator {how!r} not one of the supported image operators: {ops}")
    src = src.contiguous()
    out = torch.empty_like(src)
    if isinstance(dst, torch.Tensor):
        dst = dst.contiguous()
        dptr, dval = dst.data_ptr(), 0
    else:
        dptr, dval = None, int(dst) & 0xFFFFFFFF
    N.check(N.lib().dsgb_composite(src.data_ptr(), dptr, dval, src.numel(), _COMPOSITE[how], out.data_ptr(),
                                   torch.cuda.current_stream(src.device).cuda_stream), "dsgb_composite")
    return out


def stack(*imgs, **kwargs):
    """tf.stack (transfer_functions/__init__.py:115-145): later images are
    composited onto earlier ones with ``how`` (default 'over')."""
    if not imgs:
        raise ValueError("No images passed in")
    shapes = []
    for i in imgs:
        if not isinstance(i, Image):
            raise TypeError(f"Expected `Image`, got: `{type(i)}`")
        if not shapes:
            shapes.append(i.shape)
        elif i.shape not in shapes:
            raise ValueError("The stacked images must have the same shape.")
    name = kwargs.get("name", None)
    how = kwargs.get("how", "over")
    if how not in _COMPOSITE:
        _composite(imgs[0].data, 0, how)            # raises the reference's message
    if len(imgs) == 1:
        return imgs[0]
    acc = imgs[0].data
    for img in imgs[1:]:
        acc = _composite(img.data, acc, how)
    return Image(acc, imgs[0].dims, imgs[0].coords, imgs[0].attrs, name=name)


def set_background(img, color=None, name=None):
    """tf.set_background (transfer_functions/__init__.py:748-767): the image
    composited 'over' an opaque background colour."""
    if not isinstance(img, Image):
        raise TypeError(f"Expected `Image`, got: `{type(img)}`")
    name = img.name if name is None else name
    if color is None:
        return img
    r, g, b = rgb(color)
    background = r | (g << 8) | (b << 16) | (255 << 24)
    return Image(_composite(img.data, background, "over"), img.dims, img.coords, img.attrs, name=name)
