"""tiny_mc_gb300 — GB300-native (sm_103a) photon walk of Tiny Monte Carlo.

Python mirror of the C ABI in ``include/tmc.h`` (libtmc_gb300.so, loaded with
ctypes).  The reference's boundary is ``void photon(float *heats, float
*heats_squared)`` (photon.h:3), called once per photon by tiny_mc.c:47-49 with
compile-time knobs from params.h:5-27.  Here one call walks a whole batch:

    heat = np.zeros(101, np.float32); heat2 = np.zeros(101, np.float32)
    photon_batch(heat, heat2, 32768, params())       # += like photon()

There is no CPU fallback: if the CUDA library is not built or no GPU is
present, calls raise.
"""
from __future__ import annotations

import ctypes
import os
import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libtmc_gb300.so")

MATH_EXACT = 0
MATH_FAST = 1

TMC_OK = 0
STATUS = {
    0: "TMC_OK", -1: "TMC_E_INVALID", -2: "TMC_E_CUDA", -3: "TMC_E_NOMEM",
    -4: "TMC_E_TIMEOUT", -5: "TMC_E_OVERFLOW", -6: "TMC_E_NODEVICE", -7: "TMC_E_BUSY",
    -8: "TMC_E_STATE",
}


class TmcError(RuntimeError):
    """A tmc_* call returned a negative status."""

    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        msg = f"{where}: {STATUS.get(status, status)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


class Params(ctypes.Structure):
    """``tmc_params``: the runtime form of params.h's knobs."""
    _fields_ = [
        ("shells", ctypes.c_uint32),
        ("microns_per_shell", ctypes.c_float),
        ("mu_a", ctypes.c_float),
        ("mu_s", ctypes.c_float),
        ("seed", ctypes.c_uint64),
        ("photon_id_base", ctypes.c_uint64),
        ("math", ctypes.c_uint32),
        ("reserved", ctypes.c_uint32),
    ]


class BatchConfig(ctypes.Structure):
    """``tmc_batch_config``."""
    _fields_ = [("block", ctypes.c_int), ("items_per_block", ctypes.c_int),
                ("use_graph", ctypes.c_int), ("stream", ctypes.c_int)]


TALLY_DTYPE = np.dtype([("w_lo", "<u8"), ("w_hi", "<u8"), ("w2_lo", "<u8"), ("w2_hi", "<u8")])

_lib = None


def lib() -> ctypes.CDLL:
    """Load libtmc_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = ctypes.CDLL(LIB_PATH)
        vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
        P = ctypes.POINTER(Params)
        L.tmc_params_default.argtypes = [P]
        L.tmc_params_default.restype = None
        L.tmc_photon_batch.argtypes = [vp, vp, u64, P]
        L.tmc_photon_batch.restype = i32
        L.tmc_photon_batch_fx.argtypes = [vp, u64, P, vp]
        L.tmc_photon_batch_fx.restype = i32
        L.tmc_workspace_bytes.argtypes = []
        L.tmc_workspace_bytes.restype = ctypes.c_size_t
        L.tmc_photon_batch_device.argtypes = [vp, u64, P, vp, vp, vp]
        L.tmc_photon_batch_device.restype = i32
        L.tmc_tally_to_heat.argtypes = [vp, P, vp, vp]
        L.tmc_tally_to_heat.restype = i32
        L.tmc_format_report.argtypes = [ctypes.c_char_p, ctypes.c_size_t, vp, vp, u64, P]
        L.tmc_format_report.restype = i32
        L.tmc_set_plain_launch.argtypes = [i32, i32, i32]
        L.tmc_set_plain_launch.restype = i32
        L.tmc_debug_rand.argtypes = [u64, u64, ctypes.c_uint32, vp]
        L.tmc_debug_rand.restype = i32
        BP = ctypes.POINTER(ctypes.c_void_p)
        L.tmc_batch_create.argtypes = [BP, vp, ctypes.c_uint32, u64, ctypes.c_uint32]
        L.tmc_batch_create.restype = i32
        L.tmc_batch_set_config.argtypes = [vp, ctypes.POINTER(BatchConfig)]
        L.tmc_batch_set_config.restype = i32
        L.tmc_batch_get_config.argtypes = [vp, ctypes.POINTER(BatchConfig)]
        L.tmc_batch_get_config.restype = i32
        L.tmc_batch_autotune.argtypes = [vp, ctypes.c_double, ctypes.c_double, vp]
        L.tmc_batch_autotune.restype = i32
        L.tmc_batch_refine.argtypes = [vp, ctypes.c_uint32, vp]
        L.tmc_batch_refine.restype = i32
        L.tmc_batch_test_wait.argtypes = [vp, ctypes.c_int, ctypes.c_double]
        L.tmc_batch_test_wait.restype = i32
        L.tmc_batch_run.argtypes = [vp, vp]
        L.tmc_batch_run.restype = i32
        L.tmc_batch_read.argtypes = [vp, vp, vp]
        L.tmc_batch_read.restype = i32
        L.tmc_batch_tally_offsets.argtypes = [vp, vp]
        L.tmc_batch_tally_offsets.restype = i32
        L.tmc_batch_info.argtypes = [vp, vp, vp]
        L.tmc_batch_info.restype = i32
        L.tmc_batch_device_tallies.argtypes = [vp]
        L.tmc_batch_device_tallies.restype = vp
        L.tmc_batch_destroy.argtypes = [vp]
        L.tmc_batch_destroy.restype = i32
        L.tmc_batch_plan_items.argtypes = [vp, ctypes.c_uint32, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           vp, u64, vp]
        L.tmc_batch_plan_items.restype = i32
        L.tmc_expected_steps.argtypes = [ctypes.c_float, ctypes.c_float, vp]
        L.tmc_expected_steps.restype = i32
        L.tmc_photon_batch_static.argtypes = [vp, vp, u64, P, vp]
        L.tmc_photon_batch_static.restype = i32
        L.tmc_probe_sfu_rate.argtypes = [vp]
        L.tmc_probe_sfu_rate.restype = i32
        L.tmc_strerror.argtypes = [i32]
        L.tmc_strerror.restype = ctypes.c_char_p
        L.tmc_last_error.argtypes = []
        L.tmc_last_error.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _check(status: int, where: str) -> None:
    if status != TMC_OK:
        raise TmcError(status, where, lib().tmc_last_error().decode(errors="replace"))


def params(shells: int = 101, microns_per_shell: float = 50.0, mu_a: float = 2.0,
           mu_s: float = 20.0, seed: int = 1, photon_id_base: int = 0,
           math: str | int = "exact") -> Params:
    """A ``tmc_params`` (defaults = params.h:5-27, seed 1)."""
    m = {"exact": MATH_EXACT, "fast": MATH_FAST}.get(math, math) if isinstance(math, str) else math
    return Params(shells, microns_per_shell, mu_a, mu_s, seed, photon_id_base, int(m), 0)


def _f32(a: np.ndarray, n: int, name: str) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags.c_contiguous
            and a.size >= n):
        raise ValueError(f"{name} must be a C-contiguous float32 array of >= {n} elements")
    return a


def photon_batch(heat: np.ndarray, heat2: np.ndarray, n_photons: int, p: Params) -> None:
    """Walk ``n_photons`` photons and accumulate (+=) into heat/heat2 (float32)."""
    _f32(heat, p.shells, "heat")
    _f32(heat2, p.shells, "heat2")
    _check(lib().tmc_photon_batch(heat.ctypes.data, heat2.ctypes.data, n_photons, ctypes.byref(p)),
           "tmc_photon_batch")


STATIC_MAX_SHELLS = 4096


def photon_batch_static(heat: np.ndarray, heat2: np.ndarray, n_photons: int, p: Params,
                        stream: int = 0) -> None:
    """photon_batch for callers that cannot let the library allocate device
    memory: its scratch is a fixed array inside the library (shells <= 4096)."""
    _f32(heat, p.shells, "heat")
    _f32(heat2, p.shells, "heat2")
    _check(lib().tmc_photon_batch_static(heat.ctypes.data, heat2.ctypes.data, n_photons,
                                         ctypes.byref(p), stream or None),
           "tmc_photon_batch_static")


def photon_batch_fx(n_photons: int, p: Params, tally: np.ndarray | None = None):
    """Exact integer tallies: returns (tally[shells] of TALLY_DTYPE, photon_steps)."""
    if tally is None:
        tally = np.zeros(p.shells, TALLY_DTYPE)
    steps = ctypes.c_uint64(0)
    _check(lib().tmc_photon_batch_fx(tally.ctypes.data, n_photons, ctypes.byref(p),
                                     ctypes.byref(steps)), "tmc_photon_batch_fx")
    return tally, steps.value


def photon_batch_device(d_tally: int, n_photons: int, p: Params, d_steps: int = 0,
                        d_workspace: int = 0, stream: int = 0) -> None:
    """Device-pointer form (asynchronous on ``stream``)."""
    _check(lib().tmc_photon_batch_device(d_tally or None, n_photons, ctypes.byref(p),
                                         d_steps or None, d_workspace or None, stream or None),
           "tmc_photon_batch_device")


def set_plain_launch(block: int = 0, blocks_per_sm: int = 0, max_blocks: int = 0) -> None:
    """Launch shape of the plain walk (0 = automatic); results do not depend on it."""
    _check(lib().tmc_set_plain_launch(block, blocks_per_sm, max_blocks), "tmc_set_plain_launch")


def debug_rand(seed: int, photon: int, n: int) -> np.ndarray:
    """First n rand() values of a photon's stream, computed on the GPU."""
    out = np.zeros(n, np.int32)
    _check(lib().tmc_debug_rand(seed, photon, n, out.ctypes.data), "tmc_debug_rand")
    return out


def probe_sfu_rate() -> float:
    """Measured MUFU (special-function unit) ops/s of the current GPU."""
    r = ctypes.c_double(0.0)
    _check(lib().tmc_probe_sfu_rate(ctypes.byref(r)), "tmc_probe_sfu_rate")
    return r.value


def workspace_bytes() -> int:
    return int(lib().tmc_workspace_bytes())


def expected_steps(mu_a: float, mu_s: float) -> float:
    """Expected photon steps per photon of photon.c's weight recursion (host)."""
    out = ctypes.c_double(0.0)
    _check(lib().tmc_expected_steps(mu_a, mu_s, ctypes.byref(out)), "tmc_expected_steps")
    return out.value


def plan_items(problems, grid: int, block: int, items_per_block: int) -> np.ndarray:
    """``tmc_batch_plan_items`` (host only): the work items a batch would walk
    on `grid` resident blocks, heaviest first, as uint64 [n][3] (problem,
    first photon, photon count)."""
    from .sweep import PROBLEM_DTYPE
    pr = np.ascontiguousarray(problems, PROBLEM_DTYPE)
    n = ctypes.c_uint64(0)
    _check(lib().tmc_batch_plan_items(pr.ctypes.data, len(pr), grid, block, items_per_block, None, 0,
                                      ctypes.byref(n)), "tmc_batch_plan_items")
    out = np.zeros((max(1, n.value), 3), np.uint64)
    _check(lib().tmc_batch_plan_items(pr.ctypes.data, len(pr), grid, block, items_per_block,
                                      out.ctypes.data, n.value, ctypes.byref(n)), "tmc_batch_plan_items")
    return out[:n.value]


class Batch:
    """Many independent problems in one persistent launch (``tmc_batch``).

    ``problems`` is a structured array of ``sweep.PROBLEM_DTYPE``; all share
    ``seed`` and the arithmetic mode."""

    def __init__(self, problems: np.ndarray, seed: int = 1, math: str | int = "exact"):
        from .sweep import PROBLEM_DTYPE
        self.problems = np.ascontiguousarray(problems, dtype=PROBLEM_DTYPE)
        m = {"exact": MATH_EXACT, "fast": MATH_FAST}.get(math, math) if isinstance(math, str) else math
        h = ctypes.c_void_p()
        _check(lib().tmc_batch_create(ctypes.byref(h), self.problems.ctypes.data, len(self.problems),
                                      seed, int(m)), "tmc_batch_create")
        self.handle = h
        self.offsets = np.zeros(len(self.problems) + 1, np.uint64)
        _check(lib().tmc_batch_tally_offsets(h, self.offsets.ctypes.data), "tmc_batch_tally_offsets")

    def set_config(self, block: int = 0, items_per_block: int = 0, use_graph: bool = False,
                   stream: bool = False) -> None:
        c = BatchConfig(block, items_per_block, int(use_graph), int(stream))
        _check(lib().tmc_batch_set_config(self.handle, ctypes.byref(c)), "tmc_batch_set_config")

    def config(self) -> dict:
        c = BatchConfig()
        _check(lib().tmc_batch_get_config(self.handle, ctypes.byref(c)), "tmc_batch_get_config")
        return {"block": c.block, "items_per_block": c.items_per_block, "use_graph": bool(c.use_graph),
                "stream": bool(c.stream)}

    def autotune(self, scale: float = 1.0 / 64, max_steps_per_photon: float = 2e4) -> float:
        ms = ctypes.c_double(0.0)
        _check(lib().tmc_batch_autotune(self.handle, scale, max_steps_per_photon, ctypes.byref(ms)),
               "tmc_batch_autotune")
        return ms.value

    def refine(self, max_candidates: int = 4) -> float:
        """Second tuning stage: the best autotuned configuration of each
        (kernel, block size), one full run each; keeps the fastest."""
        ms = ctypes.c_double(0.0)
        _check(lib().tmc_batch_refine(self.handle, max_candidates, ctypes.byref(ms)), "tmc_batch_refine")
        return ms.value

    def test_wait(self, hold_buffers: bool, wait_limit_s: float = 0.0) -> None:
        """Test hook of the barrier-free kernel's bounded waits."""
        _check(lib().tmc_batch_test_wait(self.handle, int(hold_buffers), wait_limit_s),
               "tmc_batch_test_wait")

    def run(self, stream: int = 0) -> None:
        _check(lib().tmc_batch_run(self.handle, stream or None), "tmc_batch_run")

    def read(self):
        """(tallies [total shells] TALLY_DTYPE, photon steps per problem)."""
        t = np.zeros(int(self.offsets[-1]), TALLY_DTYPE)
        s = np.zeros(len(self.problems), np.uint64)
        _check(lib().tmc_batch_read(self.handle, t.ctypes.data, s.ctypes.data), "tmc_batch_read")
        return t, s

    def info(self):
        n = ctypes.c_uint32(0)
        w = ctypes.c_double(0.0)
        _check(lib().tmc_batch_info(self.handle, ctypes.byref(n), ctypes.byref(w)), "tmc_batch_info")
        return n.value, w.value

    def tally_of(self, tallies: np.ndarray, i: int) -> np.ndarray:
        return tallies[int(self.offsets[i]):int(self.offsets[i + 1])]

    def device_tallies(self) -> int:
        return int(lib().tmc_batch_device_tallies(self.handle) or 0)

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().tmc_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tally_to_heat(tally: np.ndarray, p: Params):
    """FP64 heat, heat2 from exact tallies (host)."""
    heat = np.zeros(p.shells, np.float64)
    heat2 = np.zeros(p.shells, np.float64)
    _check(lib().tmc_tally_to_heat(tally.ctypes.data, ctypes.byref(p), heat.ctypes.data,
                                   heat2.ctypes.data), "tmc_tally_to_heat")
    return heat, heat2


def tally_sums(tally: np.ndarray):
    """Python-int sums (sum_w, sum_w2) per shell, in 2^-40 units."""
    sw = [int(t["w_hi"]) << 64 | int(t["w_lo"]) for t in tally]
    sw2 = [int(t["w2_hi"]) << 64 | int(t["w2_lo"]) for t in tally]
    return sw, sw2


def format_report(heat: np.ndarray, heat2: np.ndarray, photons: int, p: Params) -> str:
    """tiny_mc.c:58-66's table for float heat/heat2 of ``photons`` photons."""
    _f32(heat, p.shells, "heat")
    _f32(heat2, p.shells, "heat2")
    n = lib().tmc_format_report(None, 0, heat.ctypes.data, heat2.ctypes.data, photons, ctypes.byref(p))
    if n < 0:
        _check(n, "tmc_format_report")
    buf = ctypes.create_string_buffer(n + 1)
    lib().tmc_format_report(buf, n + 1, heat.ctypes.data, heat2.ctypes.data, photons, ctypes.byref(p))
    return buf.value.decode()


def _rep_setup(L) -> None:
    if not getattr(L, "_rep_ready", False):
        vp = ctypes.c_void_p
        L.tmc_report_fp64.argtypes = [vp, ctypes.POINTER(Params), ctypes.c_uint64, vp, vp, vp]
        L.tmc_report_fp64.restype = ctypes.c_int
        L.tmc_format_report_fp64.argtypes = [ctypes.c_char_p, ctypes.c_size_t, vp, vp, ctypes.c_double,
                                             ctypes.POINTER(Params)]
        L.tmc_format_report_fp64.restype = ctypes.c_int
        L._rep_ready = True


def report_fp64(tally: np.ndarray, p: Params, photons: int):
    """tiny_mc.c:60-66's numbers in FP64 on the GPU: (density, error, extra)."""
    L = lib()
    _rep_setup(L)
    t = np.ascontiguousarray(tally, TALLY_DTYPE)
    dens = np.zeros(p.shells - 1, np.float64)
    err = np.zeros(p.shells - 1, np.float64)
    extra = ctypes.c_double(0.0)
    _check(L.tmc_report_fp64(t.ctypes.data, ctypes.byref(p), photons, dens.ctypes.data, err.ctypes.data,
                             ctypes.byref(extra)), "tmc_report_fp64")
    return dens, err, extra.value


def format_report_fp64(density: np.ndarray, error: np.ndarray, extra: float, p: Params) -> str:
    """The report table printed from FP64 values."""
    L = lib()
    _rep_setup(L)
    d = np.ascontiguousarray(density, np.float64)
    e = np.ascontiguousarray(error, np.float64)
    n = L.tmc_format_report_fp64(None, 0, d.ctypes.data, e.ctypes.data, extra, ctypes.byref(p))
    if n < 0:
        _check(n, "tmc_format_report_fp64")
    buf = ctypes.create_string_buffer(n + 1)
    L.tmc_format_report_fp64(buf, n + 1, d.ctypes.data, e.ctypes.data, extra, ctypes.byref(p))
    return buf.value.decode()


def derived(p: Params):
    """(albedo, 1-albedo, shells_per_mfp) as float32, exactly as photon.c:8-9 computes them."""
    mu_a, mu_s = np.float32(p.mu_a), np.float32(p.mu_s)
    albedo = np.float32(mu_s / np.float32(mu_s + mu_a))
    spm = np.float32(1e4 / float(np.float32(p.microns_per_shell)) / float(np.float32(mu_a + mu_s)))
    return albedo, np.float32(np.float32(1.0) - albedo), spm


__all__ = [
    "Params", "params", "photon_batch", "photon_batch_fx", "photon_batch_device",
    "workspace_bytes", "set_plain_launch", "debug_rand", "tally_to_heat", "Batch", "BatchConfig",
    "expected_steps", "photon_batch_static", "report_fp64", "format_report_fp64", "tally_sums", "format_report", "derived", "TmcError",
    "MATH_EXACT", "MATH_FAST", "TALLY_DTYPE", "lib", "LIB_PATH",
]
