"""Host-side checks of the request server (no GPU): trace generation and
configuration validation (rejected before any device work)."""
import ctypes

import numpy as np
import pytest


def test_trace_shape_and_rates():
    from tiny_mc_gb300.serve import make_trace
    req, arr = make_trace(20000, rate=2000.0, seed=0)
    assert len(req) == 20000 and np.all(np.diff(arr) > 0)
    assert abs(len(arr) / arr[-1] - 2000.0) / 2000.0 < 0.03      # Poisson rate
    assert req["target_rse"].min() >= 0.005 and req["target_rse"].max() <= 0.05
    assert np.all(req["max_photons"] == 1 << 24)
    assert np.all(np.diff(req["photon_id_base"].astype(np.int64)) == 1 << 32)
    assert set(np.unique(req["shells"])) == {101, 501}


@pytest.mark.parametrize("field,value", [("slots", 0), ("max_shells", 0), ("min_batches", 1),
                                         ("block", 100), ("math", 9), ("max_items_per_request", 0),
                                         ("waves", 65), ("steps_per_item", -1.0),
                                         ("steps_per_batch", 0.0)])
def test_invalid_server_config_rejected(tmc_mod, field, value):
    from tiny_mc_gb300.serve import default_config
    c = default_config(**{field: value})
    h = ctypes.c_void_p()
    assert tmc_mod.lib().tmc_server_create(ctypes.byref(h), ctypes.byref(c)) == -1


def test_default_server_config(tmc_mod):
    from tiny_mc_gb300.serve import default_config
    c = default_config()
    assert c.probe_shell == 10 and c.min_batches >= 2 and c.slots > 0
    assert c.waves == 0 and c.inflight_items == 0 and c.steps_per_item == 0.0   # 16, unbounded, unsplit
    assert ctypes.sizeof(c) == 64
