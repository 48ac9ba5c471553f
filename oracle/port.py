"""ctypes wrapper of the CPU oracle (oracle/src/rt_oracle.cpp). TEST INFRASTRUCTURE ONLY.

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the checker
and the timed CPU baseline; the renderer never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")


class Params(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_level", C.c_int32),
                ("ref_tiles", C.c_int32), ("threads", C.c_int32), ("check", C.c_int32), ("seed", C.c_uint64),
                ("tiles", C.POINTER(C.c_int32)), ("n_tiles", C.c_int32), ("block", C.c_int32), ("mode", C.c_int32),
                ("check_mask", C.POINTER(C.c_uint8)), ("tile_seconds", C.POINTER(C.c_double)),
                ("tile_rays", C.POINTER(C.c_int64))]


def _lib() -> C.CDLL:
    if not os.path.exists(LIB):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    lib = C.CDLL(LIB)
    P = C.c_void_p
    lib.orc_render_f32.argtypes = [P, C.POINTER(Params), P, P, P, P, P, P, P, P]
    lib.orc_render_f32.restype = C.c_int
    lib.orc_render_f64.argtypes = [P, C.POINTER(Params), P, P, P, P, P, P]
    lib.orc_render_f64.restype = C.c_int
    lib.orc_morton_sort.argtypes = [P, C.c_int64, P, P]
    lib.orc_morton_sort.restype = C.c_int
    return lib


_L = None


def lib() -> C.CDLL:
    global _L
    if _L is None:
        _L = _lib()
    return _L


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _desc_ptr(scene):
    # a raytrace_gb300.SceneHost or anything exposing desc_ptr()
    return C.cast(scene.desc_ptr(), C.c_void_p)


def render(scene, width: int, height: int, spp: int = 1, max_level: int = 3, seed: int = 0, ref_tiles: bool = False,
           threads: int | None = None, check: bool = True, tiles=None, fp64: bool = False, block: int = 8,
           mode: int = 0x80, check_pixels=None) -> dict:
    """Render with the oracle. Returns rgb (float32 or float64), rgb8, obj, prim, t, ambiguous
    (with `reasons` bits: 1 near-tie, 2 winner differs from the exact per-primitive search,
    4 shadow blocker at the light distance, 8 shadow result differs, 16 texel read past the
    texel array, undefined in the reference; bit 16 is set with or without `check`),
    counts (primary, secondary, shadow), seconds (wall) and, per entry of `tiles` (or per tile of
    the frame), tile_seconds (thread-seconds spent on it) and tile_rays. `tiles` limits the render to those 64x64
    tile indices (row-major over the rendered region). `block` splits tiles into smaller work units
    for the thread pool (64 keeps the reference's whole-tile units). `mode` is a RT_MODE_* value
    (the reference's MY_MODEL_* test modes; ray tracing by default). `check_pixels` (a boolean
    height x width array) limits the brute-force check to those pixels: the check costs a pass
    over every primitive per ray, too slow for millions of triangles on a whole tile."""
    L = lib()
    threads = threads or os.cpu_count() or 1
    tl = None if tiles is None else np.ascontiguousarray(tiles, np.int32)
    cm = None
    if check_pixels is not None:
        cm = np.ascontiguousarray(check_pixels, np.uint8)
        if cm.shape != (height, width):
            raise ValueError(f"check_pixels must be {height}x{width}, not {cm.shape}")
    n_entries = len(tl) if tl is not None else (((width // 64 if ref_tiles else (width + 63) // 64)) *
                                                 ((height // 64 if ref_tiles else (height + 63) // 64)))
    tile_s = np.zeros(max(1, n_entries), np.float64)
    tile_r = np.zeros(max(1, n_entries), np.int64)
    p = Params(width, height, spp, max_level, int(ref_tiles), threads, int(check and not fp64), seed,
               tl.ctypes.data_as(C.POINTER(C.c_int32)) if tl is not None else None, 0 if tl is None else len(tl),
               block, mode, cm.ctypes.data_as(C.POINTER(C.c_uint8)) if cm is not None else None,
               tile_s.ctypes.data_as(C.POINTER(C.c_double)), tile_r.ctypes.data_as(C.POINTER(C.c_int64)))
    obj = np.full((height, width), -1, np.int32)
    prim = np.zeros((height, width), np.int32)
    t = np.full((height, width), 1e20, np.float32)
    counts = np.zeros(4, np.int64)
    secs = C.c_double()
    if fp64:
        rgb = np.zeros((height, width, 3), np.float64)
        rc = L.orc_render_f64(_desc_ptr(scene), C.byref(p), _p(rgb), _p(obj), _p(prim), _p(t), _p(counts), C.byref(secs))
        rgb8 = None
        amb = np.zeros((height, width), bool)
        reasons = np.zeros((height, width), np.uint8)
    else:
        rgb = np.zeros((height, width, 3), np.float32)
        rgb8 = np.zeros((height, width, 3), np.uint8)
        amb8 = np.zeros((height, width), np.uint8)
        rc = L.orc_render_f32(_desc_ptr(scene), C.byref(p), _p(rgb), _p(rgb8), _p(obj), _p(prim), _p(t), _p(amb8),
                              _p(counts), C.byref(secs))
        amb = amb8 != 0
        reasons = amb8
    if rc:
        raise RuntimeError(f"oracle render failed ({rc})")
    return {"rgb": rgb, "rgb8": rgb8, "obj": obj, "prim": prim, "t": t, "ambiguous": amb, "reasons": reasons,
            "counts": counts[:3].copy(), "seconds": secs.value, "tile_seconds": tile_s[:n_entries].copy(),
            "tile_rays": tile_r[:n_entries].copy()}


def morton_sort(tri_p: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    tri_p = np.ascontiguousarray(tri_p, np.float32).reshape(-1, 9)
    n = tri_p.shape[0]
    codes = np.empty(n, np.uint32)
    perm = np.empty(n, np.uint32)
    if lib().orc_morton_sort(_p(tri_p), n, _p(codes), _p(perm)):
        raise RuntimeError("oracle morton sort failed")
    return codes, perm
