"""Build and load libdsgb (the sm_103a CUDA library behind the C ABI in include/dsgb.h).

The library is compiled in-tree with nvcc for sm_103a only and loaded with
ctypes.  There is no fallback: if the library is missing or a call fails,
an exception is raised.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

_PKG = os.path.dirname(os.path.abspath(__file__))
_ROOT = os.path.dirname(_PKG)
CSRC = os.path.join(_PKG, "csrc")
INCLUDE = os.path.join(_ROOT, "include")
BUILD_DIR = os.path.join(_PKG, "_build")
LIB_PATH = os.path.join(_PKG, "libdsgb.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
BASE_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]
# Files whose floating-point results must match numba's uncontracted arithmetic
# bit for bit are compiled without FMA contraction.
NO_FMA = {"line.cu", "line_backward.cu"}


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _fingerprint():
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cuh", ".h")):
            with open(os.path.join(CSRC, f), "rb") as fh:
                h.update(f.encode() + fh.read())
    with open(os.path.join(INCLUDE, "dsgb.h"), "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(ARCH + BASE_FLAGS).encode())
    return h.hexdigest()[:16]


def nvcc_path():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the sm_103a library cannot be built")
    return p


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every csrc/*.cu for sm_103a and link libdsgb.so (parallel nvcc)."""
    stamp = os.path.join(BUILD_DIR, "fingerprint")
    fp = _fingerprint()
    if (not force and os.path.exists(LIB_PATH) and os.path.exists(stamp)
            and open(stamp).read().strip() == fp):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    nvcc = nvcc_path()

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, src[:-3] + ".o")
        cmd = [nvcc, *ARCH, *BASE_FLAGS, f"-I{INCLUDE}", "-c", os.path.join(CSRC, src), "-o", obj]
        if src in NO_FMA:
            cmd.insert(1, "-fmad=false")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB_PATH + f".tmp{os.getpid()}"
    r = subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(fp)
    return LIB_PATH


# ---------------------------------------------------------------- ctypes ABI

class Column(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class CanvasDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("x_log", ctypes.c_int32), ("y_log", ctypes.c_int32),
                ("sx", ctypes.c_double), ("tx", ctypes.c_double),
                ("sy", ctypes.c_double), ("ty", ctypes.c_double),
                ("xmin", ctypes.c_double), ("xmax", ctypes.c_double),
                ("ymin", ctypes.c_double), ("ymax", ctypes.c_double)]


class Base(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("col", ctypes.c_int32), ("cat_col", ctypes.c_int32),
                ("ncat", ctypes.c_int32), ("flags", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("agg", ctypes.c_void_p)]


class Output(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("base0", ctypes.c_int32), ("base1", ctypes.c_int32),
                ("col", ctypes.c_int32), ("out", ctypes.c_void_p)]


class PyramidConfig(ctypes.Structure):
    _fields_ = [("zmin", ctypes.c_int32), ("zmax", ctypes.c_int32), ("tile_size", ctypes.c_int32),
                ("split", ctypes.c_int32), ("threads", ctypes.c_int32), ("chunk", ctypes.c_int32),
                ("x0", ctypes.c_double), ("x1", ctypes.c_double),
                ("y0", ctypes.c_double), ("y1", ctypes.c_double)]


# dtype codes (dsgb_dtype)
F32, F64, I8, U8, I16, I32, I64, U32, BOOL = range(1, 10)

# base ops (dsgb_base_op)
BASE_COUNT, BASE_ANY, BASE_SUM, BASE_MAX, BASE_MIN, BASE_MIN_ROW, BASE_MAX_ROW, \
    BASE_ARGMAX, BASE_ARGMIN, BASE_AA_SUM, BASE_AA_CNT0, BASE_AA_MAX, BASE_AA_ARGMAX = range(1, 14)
BASEF_UNWEIGHTED = 0x1

# finalize ops (dsgb_fin_op)
FIN_SUM_NAN, FIN_MEAN, FIN_KEY_F64, FIN_ROW, FIN_GATHER, FIN_KEY_F32, FIN_SUM_F32, FIN_COPY = range(1, 9)
FOLD_SUM, FOLD_SUM_F32, FOLD_MAX, FOLD_MIN, FOLD_FIRST, FOLD_LAST, FOLD_ROW_MIN, FOLD_ADD = range(1, 9)
FOLD_WHERE_MAX, FOLD_WHERE_MIN, FOLD_WHERE_FIRST, FOLD_WHERE_LAST = range(9, 13)

FLAG_NO_INIT, FLAG_NO_FINALIZE, FLAG_EXACT_BIN, FLAG_WARP_AGG, FLAG_DETERMINISTIC = 0x1, 0x2, 0x4, 0x8, 0x10
FLAG_ROW_ORDER = 0x20
FLAG_DEBUG_CHECKS = 0x40
STATUS_CAS_GUARD, STATUS_INDEX = 0x1, 0x2

# every symbol include/dsgb.h declares
EXPORTED = (
    "dsgb_abi_version", "dsgb_last_error", "dsgb_device_status", "dsgb_fp64_probe", "dsgb_device_sm_count", "dsgb_bases_init", "dsgb_combine",
    "dsgb_finalize", "dsgb_finalize_partitioned", "dsgb_select_by_owner", "dsgb_points", "dsgb_points_workspace_size", "dsgb_points_workspace_size_flags",
    "dsgb_points_ws", "dsgb_points_segments",
    "dsgb_bucket_sort_workspace_size", "dsgb_bucket_sort", "dsgb_line_axis0", "dsgb_line_workspace_size", "dsgb_line_axis0_ws", "dsgb_lines", "dsgb_lines_2stage", "dsgb_lines_ragged", "dsgb_lines_ragged_2stage", "dsgb_line_axis0_backward", "dsgb_line_axis0_backward_ws",
    "dsgb_points_backward", "dsgb_bounds", "dsgb_eq_hist_workspace_size", "dsgb_eq_hist_u32",
    "dsgb_eq_hist_f64", "dsgb_eq_hist_u32_static", "dsgb_shade_workspace_size", "dsgb_shade_u32", "dsgb_shade_f64", "dsgb_composite", "dsgb_pyramid_tile_offset", "dsgb_pyramid_workspace_size", "dsgb_pyramid", "dsgb_pyramid_status",
)

_lock = threading.Lock()
_lib = None


class DsgbError(RuntimeError):
    pass


def _declare(L):
    P = ctypes.c_void_p
    i32, i64, dbl, u32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_uint32
    PC, PB, PO = ctypes.POINTER(Column), ctypes.POINTER(Base), ctypes.POINTER(Output)
    L.dsgb_abi_version.restype = ctypes.c_int
    L.dsgb_last_error.restype = ctypes.c_char_p
    L.dsgb_device_sm_count.restype = ctypes.c_int
    L.dsgb_device_status.argtypes = [ctypes.POINTER(u32), i32]
    L.dsgb_fp64_probe.argtypes = [P, i32, i32, ctypes.POINTER(i64), P]
    L.dsgb_bases_init.argtypes = [PB, i32, i64, P]
    L.dsgb_combine.argtypes = [PB, PB, i32, i64, P]
    L.dsgb_finalize.argtypes = [PC, i32, i64, PB, i32, PO, i32, i64, P]
    L.dsgb_finalize_partitioned.argtypes = [PC, i32, i32, ctypes.POINTER(i64), ctypes.POINTER(i64), PB, i32, PO, i32,
                                            i64, P]
    L.dsgb_select_by_owner.argtypes = [PB, i32, ctypes.POINTER(i64), ctypes.POINTER(i64), ctypes.POINTER(P), P,
                                       i64, P]
    L.dsgb_points.argtypes = [PC, i32, i64, i64, i32, i32, ctypes.POINTER(CanvasDesc), PB, i32, PO, i32, u32, P]
    L.dsgb_points_workspace_size.argtypes = [i64, ctypes.POINTER(CanvasDesc), PB, i32]
    L.dsgb_points_workspace_size.restype = ctypes.c_size_t
    L.dsgb_points_workspace_size_flags.argtypes = [i64, ctypes.POINTER(CanvasDesc), PB, i32, u32]
    L.dsgb_points_workspace_size_flags.restype = ctypes.c_size_t
    L.dsgb_points_ws.argtypes = [PC, i32, i64, i64, i32, i32, ctypes.POINTER(CanvasDesc), PB, i32, PO, i32,
                                 P, ctypes.c_size_t, u32, P]
    L.dsgb_points_segments.argtypes = [PC, i32, i64, i32, i32, ctypes.POINTER(CanvasDesc), PB, i32, PO, i32,
                                       P, P, i32, u32, P]
    L.dsgb_bucket_sort_workspace_size.argtypes = [i32]
    L.dsgb_bucket_sort_workspace_size.restype = ctypes.c_size_t
    L.dsgb_bucket_sort.argtypes = [PC, i32, i64, i32, i32, P, i32, P, P, P, ctypes.c_size_t, P]
    L.dsgb_line_axis0.argtypes = [PC, i32, i64, i64, i32, i32, ctypes.POINTER(CanvasDesc), dbl, i32, i32, i32,
                                  PB, i32, PO, i32, u32, P]
    L.dsgb_line_workspace_size.argtypes = [i64]
    L.dsgb_line_workspace_size.restype = ctypes.c_size_t
    L.dsgb_line_axis0_ws.argtypes = [PC, i32, i64, i64, i32, i32, ctypes.POINTER(CanvasDesc), dbl, i32, i32, i32,
                                     PB, i32, PO, i32, P, ctypes.c_size_t, u32, P]
    L.dsgb_lines.argtypes = [PC, i32, i64, i64, i32, P, P, i64, i64, i64, ctypes.POINTER(CanvasDesc), dbl, i32, i32,
                             PB, i32, PO, i32, u32, P]
    L.dsgb_lines_2stage.argtypes = [PC, i32, i64, i64, i32, P, P, i64, i64, i64, ctypes.POINTER(CanvasDesc), dbl,
                                    i32, PB, i32, ctypes.POINTER(i32), ctypes.POINTER(P), PO, i32, u32, P]
    L.dsgb_lines_ragged.argtypes = [PC, i32, i64, i64, P, i64, P, P, i64, P, ctypes.POINTER(CanvasDesc), dbl, i32,
                                    PB, i32, PO, i32, u32, P]
    L.dsgb_lines_ragged_2stage.argtypes = [PC, i32, i64, i64, P, i64, P, P, i64, P, ctypes.POINTER(CanvasDesc),
                                           dbl, i32, PB, i32, ctypes.POINTER(i32), ctypes.POINTER(P), PO, i32,
                                           u32, P]
    L.dsgb_line_axis0_backward.argtypes = [PC, i32, i64, i32, i32, i32, ctypes.POINTER(CanvasDesc), dbl, i32,
                                           P, P, P, P, P]
    L.dsgb_line_axis0_backward_ws.argtypes = [PC, i32, i64, i32, i32, i32, ctypes.POINTER(CanvasDesc), dbl, i32,
                                              P, P, P, P, P, ctypes.c_size_t, P]
    L.dsgb_points_backward.argtypes = [PC, i32, i64, i32, i32, i32, ctypes.POINTER(CanvasDesc), P, P, P, u32, P]
    L.dsgb_bounds.argtypes = [PC, i64, P, P]
    L.dsgb_eq_hist_workspace_size.argtypes = [i32]
    L.dsgb_eq_hist_workspace_size.restype = ctypes.c_size_t
    for nm in ("dsgb_eq_hist_u32", "dsgb_eq_hist_f64"):
        getattr(L, nm).argtypes = [P, i64, i32, P, P, P, P, i32, i32, i32, P, ctypes.c_size_t, P]
    L.dsgb_shade_workspace_size.argtypes = []
    L.dsgb_shade_workspace_size.restype = ctypes.c_size_t
    L.dsgb_composite.argtypes = [P, P, u32, i64, i32, P, P]
    for nm in ("dsgb_shade_u32", "dsgb_shade_f64"):
        getattr(L, nm).argtypes = [P, i64, i32, P, P, i32, P, i32, i32, P, P, ctypes.c_size_t, P]
    L.dsgb_eq_hist_u32_static.argtypes = [P, i64, i32, P, P, P, P, i32, i32, i32, P]
    L.dsgb_pyramid_tile_offset.argtypes = [i32, i32, i32]
    L.dsgb_pyramid_tile_offset.restype = i64
    L.dsgb_pyramid_workspace_size.argtypes = [i64, i32, ctypes.POINTER(PyramidConfig)]
    L.dsgb_pyramid_workspace_size.restype = ctypes.c_size_t
    L.dsgb_pyramid.argtypes = [PC, i32, i64, i32, i32, i32, ctypes.POINTER(PyramidConfig), P, P, P,
                               ctypes.c_size_t, u32, P]
    L.dsgb_pyramid_status.argtypes = [P, i64, i32, ctypes.POINTER(PyramidConfig), P, P]
    non_int = ("dsgb_last_error", "dsgb_eq_hist_workspace_size", "dsgb_pyramid_tile_offset",
               "dsgb_points_workspace_size", "dsgb_pyramid_workspace_size", "dsgb_bucket_sort_workspace_size",
               "dsgb_points_workspace_size_flags", "dsgb_shade_workspace_size", "dsgb_line_workspace_size")
    for nm in EXPORTED:
        if nm not in non_int:
            getattr(L, nm).restype = ctypes.c_int
    return L


def lib(build_if_missing: bool = True):
    """The loaded libdsgb (built on first use when nvcc is available)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                if not build_if_missing:
                    raise DsgbError(f"{LIB_PATH} is missing; run datashader_gb300._native.build()")
                build()
            _lib = _declare(ctypes.CDLL(LIB_PATH))
    return _lib


def device_status(clear: bool = True) -> int:
    """Wait for the current device and return the DSGB_STATUS_* bits its kernels raised."""
    bits = ctypes.c_uint32(0)
    check(lib().dsgb_device_status(ctypes.byref(bits), int(clear)), "dsgb_device_status")
    return int(bits.value)


def check(rc: int, what: str = "dsgb call"):
    if rc != 0:
        msg = lib().dsgb_last_error().decode(errors="replace")
        raise DsgbError(f"{what} failed with status {rc}: {msg}")
    return rc
