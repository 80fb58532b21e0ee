"""ctypes wrapper of the CPU oracle (tmc_oracle.c) and of the reference
builds in oracle/_ref/.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg — as the oracle results are compared against,
never as the product path.

What each call restates (reference = computacionparalela/tiny_mc):
  walk_fx, photon_hashes   photon.c:6-51 in FP32, photon.c's evaluation order
  walk_f64                 photon.c:6-51 with every operation in FP64
  native_run               tiny_mc.c:43-49 (srand + photon loop, libc rand)
  ref_*                    the reference's own photon.c (oracle/_ref/)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# the reference's source tree: $TMC_REFERENCE_TREE, else a directory named
# "reference" beside this repository's root
REFERENCE_TREE = os.environ.get("TMC_REFERENCE_TREE") or os.path.normpath(
    os.path.join(HERE, os.pardir, os.pardir, "reference"))

LOG_TMC = 0
LOG_NATIVE = 1

CONFIGS = {
    # name: (shells, microns_per_shell, mu_a, mu_s); the same optics the
    # Makefile compiles the reference's photon.c at
    "params_h": (101, 50.0, 2.0, 20.0),
    "high_albedo": (1001, 10.0, 0.1, 100.0),
    "one_shell": (1, 50.0, 2.0, 20.0),
    "low_albedo": (101, 50.0, 10.0, 1.0),
    "fine_shells": (4001, 1.0, 2.0, 20.0),
}


class OParams(ctypes.Structure):
    _fields_ = [
        ("shells", ctypes.c_uint32),
        ("microns_per_shell", ctypes.c_float),
        ("mu_a", ctypes.c_float),
        ("mu_s", ctypes.c_float),
        ("seed", ctypes.c_uint64),
    ]


def build(ref: bool | None = None) -> None:
    """make liboracle.so; and _ref/ when the reference tree is present."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref is None:
        ref = os.path.isfile(os.path.join(REFERENCE_TREE, "photon.c"))
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REFERENCE_TREE], check=True)


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(ref=False)
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, u32, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
        P = ctypes.POINTER(OParams)
        L.tmo_philox4x32_10.argtypes = [vp, vp, vp]
        L.tmo_logf.argtypes = [ctypes.c_float]
        L.tmo_logf.restype = ctypes.c_float
        L.tmo_logf_max_ulp.argtypes = [ctypes.c_float, ctypes.c_float, u32, vp]
        L.tmo_logf_max_ulp.restype = ctypes.c_double
        L.tmo_stream_dump.argtypes = [u64, u64, u32, vp]
        L.tmo_walk_fx.argtypes = [P, u64, u64, i32, vp, vp, vp, i32]
        L.tmo_walk_fx.restype = i32
        L.tmo_walk_photon_f32.argtypes = [P, u64, i32, vp, vp]
        L.tmo_photon_hashes.argtypes = [P, u64, u32, i32, vp, vp, vp]
        L.tmo_photon_hashes.restype = i32
        L.tmo_walk_f64.argtypes = [P, u64, u64, vp, vp, vp, i32]
        L.tmo_walk_f64.restype = i32
        L.tmo_native_run.argtypes = [P, u64, u32, vp, vp, u32, vp, vp]
        L.tmo_native_run.restype = i32
        L.tmo_native_rate.argtypes = [P, u64, u32, vp]
        L.tmo_native_rate.restype = ctypes.c_double
        L.tmo_colormap.argtypes = [vp, u32, u32, u32, vp, vp]
        L.tmo_colormap.restype = None
        _lib = L
    return _lib


def oparams(shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0, seed=1) -> OParams:
    return OParams(shells, microns_per_shell, mu_a, mu_s, seed)


def cfg(name: str, seed: int = 1) -> OParams:
    s, m, a, b = CONFIGS[name]
    return oparams(s, m, a, b, seed)


def philox(ctr, key) -> np.ndarray:
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().tmo_philox4x32_10(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def stream(seed: int, photon: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.int32)
    lib().tmo_stream_dump(seed, photon, n, out.ctypes.data)
    return out


def logf(x: float) -> float:
    return lib().tmo_logf(x)


def logf_max_ulp(lo: float, hi: float, stride: int = 1):
    """(largest ulp error of tmo_logf against double log over every stride-th
    float of [lo, hi], share correctly rounded)."""
    share = ctypes.c_double(0.0)
    worst = lib().tmo_logf_max_ulp(lo, hi, stride, ctypes.byref(share))
    return worst, share.value


def walk_fx(p: OParams, n: int, id_base: int = 0, log_mode: int = LOG_TMC, nthreads: int = 0):
    """Exact tallies: (tally uint64 [S,4], deposits uint64 [S], steps)."""
    S = p.shells
    tally = np.zeros((S, 4), np.uint64)
    dep = np.zeros(S, np.uint64)
    steps = np.zeros(1, np.uint64)
    nt = nthreads or min(os.cpu_count() or 1, 16)
    rc = lib().tmo_walk_fx(ctypes.byref(p), id_base, n, log_mode, tally.ctypes.data, dep.ctypes.data,
                           steps.ctypes.data, nt)
    if rc != 0:
        raise ValueError(f"tmo_walk_fx: {rc}")
    return tally, dep, int(steps[0])


def walk_f64(p: OParams, n: int, id_base: int = 0, nthreads: int = 0):
    """FP64 oracle: (heat, heat2, deposits)."""
    S = p.shells
    h = np.zeros(S)
    h2 = np.zeros(S)
    dep = np.zeros(S, np.uint64)
    nt = nthreads or min(os.cpu_count() or 1, 16)
    rc = lib().tmo_walk_f64(ctypes.byref(p), id_base, n, h.ctypes.data, h2.ctypes.data,
                            dep.ctypes.data, nt)
    if rc != 0:
        raise ValueError(f"tmo_walk_f64: {rc}")
    return h, h2, dep


def photon_hashes(p: OParams, n: int, id_base: int = 0, log_mode: int = LOG_TMC):
    S = p.shells
    hashes = np.zeros(n, np.uint64)
    hs = np.zeros(S)
    h2s = np.zeros(S)
    rc = lib().tmo_photon_hashes(ctypes.byref(p), id_base, n, log_mode, hashes.ctypes.data,
                                 hs.ctypes.data, h2s.ctypes.data)
    if rc != 0:
        raise ValueError(f"tmo_photon_hashes: {rc}")
    return hashes, hs, h2s


def native_run(p: OParams, n: int, seed: int, batch: int = 0):
    """libc-rand replay of tiny_mc.c:43-49: (heat, heat2[, batch_heat, batch_heat2])."""
    S = p.shells
    h = np.zeros(S, np.float32)
    h2 = np.zeros(S, np.float32)
    if batch:
        nb = n // batch
        bh = np.zeros((nb, S), np.float32)
        bh2 = np.zeros((nb, S), np.float32)
        lib().tmo_native_run(ctypes.byref(p), n, seed, h.ctypes.data, h2.ctypes.data, batch,
                             bh.ctypes.data, bh2.ctypes.data)
        return h, h2, bh, bh2
    lib().tmo_native_run(ctypes.byref(p), n, seed, h.ctypes.data, h2.ctypes.data, 0, None, None)
    return h, h2


def native_rate(p: OParams, n: int, seed: int = 1):
    """(photons/s, steps) of the libc-rand walk on one core."""
    steps = ctypes.c_uint64(0)
    r = lib().tmo_native_rate(ctypes.byref(p), n, seed, ctypes.byref(steps))
    return r, steps.value


def heat_from_tally(p: OParams, tally: np.ndarray):
    """FP64 heat/heat2 from exact tallies (1-albedo computed in float as photon.c:30)."""
    mu_a, mu_s = np.float32(p.mu_a), np.float32(p.mu_s)
    albedo = np.float32(mu_s / np.float32(mu_s + mu_a))
    c = float(np.float32(np.float32(1.0) - albedo))
    t = tally.astype(np.float64)
    sw = t[:, 1] * 2.0 ** 24 + t[:, 0] * 2.0 ** -40
    sw2 = t[:, 3] * 2.0 ** 24 + t[:, 2] * 2.0 ** -40
    return c * sw, c * c * sw2


def colormap(heats: np.ndarray, width: int = 800, height: int = 800):
    """The viewer's colour map (cg_mc.c:38-67): (red float [h, w], rgba uint8 [h, w, 4])."""
    h = np.ascontiguousarray(heats, np.float32)
    red = np.zeros((height, width), np.float32)
    rgba = np.zeros((height, width, 4), np.uint8)
    lib().tmo_colormap(h.ctypes.data, len(h), width, height, red.ctypes.data, rgba.ctypes.data)
    return red, rgba


# ---------------------------------------------------------------- _ref/
def ref_available(name: str, kind: str) -> bool:
    return os.path.exists(os.path.join(REF_DIR, f"libref_{name}_{kind}.so"))


def ref_lib(name: str, kind: str) -> ctypes.CDLL:
    L = ctypes.CDLL(os.path.join(REF_DIR, f"libref_{name}_{kind}.so"))
    vp, u64, u32, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int
    if kind == "inj":
        L.ref_photon_hashes.argtypes = [u64, u64, u32, i32, vp, vp, vp]
        L.ref_photon_hashes.restype = i32
    else:
        L.ref_native_run.argtypes = [u64, ctypes.c_uint, vp, vp]
        L.ref_native_batches.argtypes = [u64, ctypes.c_uint, ctypes.c_uint, vp, vp]
        L.ref_native_rate.argtypes = [u64, ctypes.c_uint]
        L.ref_native_rate.restype = ctypes.c_double
    L.ref_shells.restype = ctypes.c_uint
    return L


def ref_photon_hashes(name: str, n: int, seed: int = 1, id_base: int = 0, log_mode: int = LOG_TMC):
    L = ref_lib(name, "inj")
    S = L.ref_shells()
    hashes = np.zeros(n, np.uint64)
    hs = np.zeros(S)
    h2s = np.zeros(S)
    L.ref_photon_hashes(seed, id_base, n, log_mode, hashes.ctypes.data, hs.ctypes.data,
                        h2s.ctypes.data)
    return hashes, hs, h2s


def ref_native_run(name: str, n: int, seed: int):
    L = ref_lib(name, "nat")
    S = L.ref_shells()
    h = np.zeros(S, np.float32)
    h2 = np.zeros(S, np.float32)
    L.ref_native_run(n, seed, h.ctypes.data, h2.ctypes.data)
    return h, h2


def ref_native_batches(name: str, n: int, seed: int, batch: int):
    L = ref_lib(name, "nat")
    S = L.ref_shells()
    bh = np.zeros((n // batch, S), np.float32)
    bh2 = np.zeros((n // batch, S), np.float32)
    L.ref_native_batches(n, seed, batch, bh.ctypes.data, bh2.ctypes.data)
    return bh, bh2


def ref_binary() -> str:
    return os.path.join(REF_DIR, "tiny_mc_ref")
