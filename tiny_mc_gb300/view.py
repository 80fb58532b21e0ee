"""The viewer's two jobs (cg_mc.c) without a graphics stack: the progressive
walk with snapshots, and the fragment shader's colour map into an image
buffer (written as a binary PPM where a file is wanted)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import Params, _check, lib


def _setup(L):
    if getattr(L, "_view_ready", False):
        return
    vp, u64, u32, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
    L.tmc_colormap.argtypes = [vp, u32, u32, u32, vp, vp, vp]
    L.tmc_colormap.restype = i32
    L.tmc_colormap_host.argtypes = [vp, u32, u32, u32, vp, vp]
    L.tmc_colormap_host.restype = i32
    L.tmc_progressive_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Params)]
    L.tmc_progressive_create.restype = i32
    L.tmc_progressive_advance.argtypes = [vp, u64]
    L.tmc_progressive_advance.restype = i32
    L.tmc_progressive_snapshot.argtypes = [vp, vp, vp, ctypes.POINTER(u64), i32]
    L.tmc_progressive_snapshot.restype = i32
    L.tmc_progressive_render.argtypes = [vp, u32, u32, vp]
    L.tmc_progressive_render.restype = i32
    L.tmc_progressive_destroy.argtypes = [vp]
    L.tmc_progressive_destroy.restype = i32
    L._view_ready = True


def colormap(heats: np.ndarray, width: int = 800, height: int = 800):
    """(red float [h, w], rgba uint8 [h, w, 4]) of the viewer's colour map."""
    L = lib()
    _setup(L)
    h = np.ascontiguousarray(heats, np.float32)
    red = np.zeros((height, width), np.float32)
    rgba = np.zeros((height, width, 4), np.uint8)
    _check(L.tmc_colormap_host(h.ctypes.data, len(h), width, height, red.ctypes.data, rgba.ctypes.data),
           "tmc_colormap_host")
    return red, rgba


def write_ppm(path: str, rgba: np.ndarray) -> None:
    """Binary PPM (P6), top row first (the image's row 0 is the bottom row)."""
    h, w = rgba.shape[:2]
    with open(path, "wb") as f:
        f.write(f"P6\n{w} {h}\n255\n".encode())
        f.write(np.ascontiguousarray(rgba[::-1, :, :3]).tobytes())


class Progressive:
    """``tmc_progressive``: advance frame by frame, read snapshots without waiting."""

    def __init__(self, p: Params):
        L = lib()
        _setup(L)
        self.p = p
        h = ctypes.c_void_p()
        _check(L.tmc_progressive_create(ctypes.byref(h), ctypes.byref(p)), "tmc_progressive_create")
        self.handle = h

    def advance(self, n_photons: int) -> None:
        _check(lib().tmc_progressive_advance(self.handle, n_photons), "tmc_progressive_advance")

    def snapshot(self, wait: bool = False):
        """(new, heat, heat2, photons); new is False if nothing newer finished."""
        heat = np.zeros(self.p.shells, np.float32)
        heat2 = np.zeros(self.p.shells, np.float32)
        n = ctypes.c_uint64(0)
        r = lib().tmc_progressive_snapshot(self.handle, heat.ctypes.data, heat2.ctypes.data,
                                           ctypes.byref(n), int(wait))
        if r < 0:
            _check(r, "tmc_progressive_snapshot")
        return bool(r), heat, heat2, n.value

    def render(self, width: int = 800, height: int = 800) -> np.ndarray:
        rgba = np.zeros((height, width, 4), np.uint8)
        _check(lib().tmc_progressive_render(self.handle, width, height, rgba.ctypes.data),
               "tmc_progressive_render")
        return rgba

    def close(self):
        if getattr(self, "handle", None):
            lib().tmc_progressive_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
