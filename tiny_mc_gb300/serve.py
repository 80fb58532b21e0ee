"""The served stream: requests with the batched sweep's parameter
distribution plus a target relative standard error (RSE) at shell 10 drawn
uniformly from [0.5 %, 5 %], a photon cap of 2^24, and Poisson arrivals at
rate lambda.  Seeded synthetic trace; no public dataset is involved.  Each
request owns a 2^32-photon id range, so its streams do not depend on the mix.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import Params, TALLY_DTYPE, _check, lib  # noqa: F401

REQUEST_DTYPE = np.dtype([
    ("shells", "<u4"), ("microns_per_shell", "<f4"), ("mu_a", "<f4"), ("mu_s", "<f4"),
    ("target_rse", "<f8"), ("max_photons", "<u8"), ("photon_id_base", "<u8"),
])
RESULT_DTYPE = np.dtype([
    ("photons", "<u8"), ("photon_steps", "<u8"), ("batches", "<u4"), ("batch_photons", "<u4"),
    ("rse", "<f8"), ("reached_target", "<i4"), ("reserved", "<i4"), ("latency_s", "<f8"),
])


class ServerConfig(ctypes.Structure):
    """``tmc_server_config``."""
    _fields_ = [("slots", ctypes.c_uint32), ("max_shells", ctypes.c_uint32),
                ("probe_shell", ctypes.c_uint32), ("min_batches", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("math", ctypes.c_uint32), ("block", ctypes.c_uint32),
                ("max_items_per_request", ctypes.c_uint32), ("stream", ctypes.c_uint32),
                ("steps_per_batch", ctypes.c_double), ("steps_per_item", ctypes.c_double),
                ("waves", ctypes.c_uint32), ("inflight_items", ctypes.c_uint32),
                ("persistent", ctypes.c_uint32)]


def make_trace(n: int = 100000, rate: float = 2000.0, seed: int = 0, rse=(0.005, 0.05),
               max_photons: int = 1 << 24, **sweep_kw):
    """(requests [n] REQUEST_DTYPE, arrival times [n] seconds)."""
    from .sweep import make_sweep
    sw = make_sweep(n, seed=seed, **sweep_kw)
    rng = np.random.default_rng(seed + 7919)
    req = np.zeros(n, REQUEST_DTYPE)
    for f in ("shells", "microns_per_shell", "mu_a", "mu_s"):
        req[f] = sw[f]
    req["target_rse"] = rng.uniform(rse[0], rse[1], n)
    req["max_photons"] = max_photons
    req["photon_id_base"] = np.arange(n, dtype=np.uint64) << np.uint64(32)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n))
    return req, arrivals


def _setup(L):
    if getattr(L, "_serve_ready", False):
        return
    vp, u64, i32 = ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int
    SC = ctypes.POINTER(ServerConfig)
    L.tmc_server_config_default.argtypes = [SC]
    L.tmc_server_config_default.restype = None
    L.tmc_server_create.argtypes = [ctypes.POINTER(ctypes.c_void_p), SC]
    L.tmc_server_create.restype = i32
    L.tmc_server_submit.argtypes = [vp, vp, ctypes.POINTER(u64)]
    L.tmc_server_submit.restype = i32
    L.tmc_server_progress.argtypes = [vp, vp, vp]
    L.tmc_server_progress.restype = i32
    L.tmc_server_poll.argtypes = [vp, u64, ctypes.POINTER(i32)]
    L.tmc_server_poll.restype = i32
    L.tmc_server_result.argtypes = [vp, u64, vp, vp]
    L.tmc_server_result.restype = i32
    L.tmc_server_stats.argtypes = [vp, vp, vp, vp]
    L.tmc_server_stats.restype = i32
    L.tmc_server_work.argtypes = [vp, ctypes.POINTER(u64)]
    L.tmc_server_work.restype = i32
    L.tmc_server_run_trace.argtypes = [vp, vp, vp, ctypes.c_uint32, ctypes.c_double, vp, vp]
    L.tmc_server_run_trace.restype = i32
    L.tmc_server_destroy.argtypes = [vp]
    L.tmc_server_destroy.restype = i32
    L.tmc_server_plan.argtypes = [SC, vp, vp, vp, vp]
    L.tmc_server_plan.restype = i32
    L.tmc_batch_means_rse.argtypes = [vp, ctypes.c_uint32, u64, vp, vp]
    L.tmc_batch_means_rse.restype = i32
    L._serve_ready = True


def default_config(**kw) -> ServerConfig:
    L = lib()
    _setup(L)
    c = ServerConfig()
    L.tmc_server_config_default(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def plan(request, config: ServerConfig | None = None, **kw):
    """``tmc_server_plan`` (host only): (photons per RSE batch, work items per
    batch, expected photon steps per photon) the server would use."""
    L = lib()
    _setup(L)
    c = config if config is not None else default_config(**kw)
    r = np.ascontiguousarray(np.asarray(request, REQUEST_DTYPE).reshape(1))
    b, k, e = ctypes.c_uint32(0), ctypes.c_uint32(0), ctypes.c_double(0.0)
    _check(L.tmc_server_plan(ctypes.byref(c), r.ctypes.data, ctypes.byref(b), ctypes.byref(k),
                             ctypes.byref(e)), "tmc_server_plan")
    return b.value, k.value, e.value


def batch_means_rse(probes: np.ndarray, items_per_batch: int, n_batches: int):
    """``tmc_batch_means_rse`` (host only): probes uint64 [items][2] (low, high
    64 bits of each item's 128-bit sum); returns (rse, mean)."""
    L = lib()
    _setup(L)
    p = np.ascontiguousarray(probes, np.uint64)
    rse, mean = ctypes.c_double(0.0), ctypes.c_double(0.0)
    _check(L.tmc_batch_means_rse(p.ctypes.data, items_per_batch, n_batches, ctypes.byref(rse),
                                 ctypes.byref(mean)), "tmc_batch_means_rse")
    return rse.value, mean.value


class Server:
    """``tmc_server``: submit / progress / poll / result, or run a whole trace."""

    def __init__(self, config: ServerConfig | None = None, **kw):
        L = lib()
        _setup(L)
        self.cfg = config if config is not None else default_config(**kw)
        h = ctypes.c_void_p()
        _check(L.tmc_server_create(ctypes.byref(h), ctypes.byref(self.cfg)), "tmc_server_create")
        self.handle = h

    def submit(self, request) -> int | None:
        """Request id, or None when no slot is free (TMC_E_BUSY)."""
        r = np.ascontiguousarray(np.asarray(request, REQUEST_DTYPE).reshape(1))
        rid = ctypes.c_uint64(0)
        st = lib().tmc_server_submit(self.handle, r.ctypes.data, ctypes.byref(rid))
        if st == -7:
            return None
        _check(st, "tmc_server_submit")
        return rid.value

    def progress(self):
        w, a = ctypes.c_uint32(0), ctypes.c_uint32(0)
        _check(lib().tmc_server_progress(self.handle, ctypes.byref(w), ctypes.byref(a)),
               "tmc_server_progress")
        return w.value, a.value

    def done(self, rid: int) -> bool:
        d = ctypes.c_int(0)
        _check(lib().tmc_server_poll(self.handle, rid, ctypes.byref(d)), "tmc_server_poll")
        return bool(d.value)

    def result(self, rid: int, shells: int):
        t = np.zeros(shells, TALLY_DTYPE)
        r = np.zeros(1, RESULT_DTYPE)
        _check(lib().tmc_server_result(self.handle, rid, t.ctypes.data, r.ctypes.data),
               "tmc_server_result")
        return t, r[0]

    def run(self, rid_shells: dict, timeout_s: float = 300.0):
        """Drive until every id in rid_shells is done; {id: (tally, result)}."""
        import time
        out = {}
        t0 = time.perf_counter()
        while len(out) < len(rid_shells):
            self.progress()
            for rid, sh in rid_shells.items():
                if rid not in out and self.done(rid):
                    out[rid] = self.result(rid, sh)
            if time.perf_counter() - t0 > timeout_s:
                raise TimeoutError("requests not finished")
            time.sleep(0.0002)
        return out

    def run_trace(self, requests: np.ndarray, arrivals: np.ndarray, time_limit_s: float = 0.0):
        req = np.ascontiguousarray(requests, REQUEST_DTYPE)
        arr = np.ascontiguousarray(arrivals, np.float64)
        res = np.zeros(len(req), RESULT_DTYPE)
        done = ctypes.c_uint32(0)
        _check(lib().tmc_server_run_trace(self.handle, req.ctypes.data, arr.ctypes.data, len(req),
                                          time_limit_s, res.ctypes.data, ctypes.byref(done)),
               "tmc_server_run_trace")
        return res, done.value

    def stats(self):
        p, s, w = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
        _check(lib().tmc_server_stats(self.handle, ctypes.byref(p), ctypes.byref(s), ctypes.byref(w)),
               "tmc_server_stats")
        return p.value, s.value, w.value

    def work(self) -> int:
        """Photon steps walked so far, running requests included."""
        w = ctypes.c_uint64(0)
        _check(lib().tmc_server_work(self.handle, ctypes.byref(w)), "tmc_server_work")
        return w.value

    def close(self):
        if getattr(self, "handle", None):
            lib().tmc_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
