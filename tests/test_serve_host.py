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
                                         ("steps_per_batch", 0.0), ("persistent", 2)])
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
    assert c.persistent in (0, 1)
    assert ctypes.sizeof(c) == 72


# ------------------------------------------------ the server's host-side plan
def _req(mu_a, mu_s, shells=101, mps=50.0):
    from tiny_mc_gb300.serve import REQUEST_DTYPE
    r = np.zeros(1, REQUEST_DTYPE)[0]
    r["shells"], r["microns_per_shell"], r["mu_a"], r["mu_s"] = shells, mps, mu_a, mu_s
    r["target_rse"], r["max_photons"] = 0.01, 1 << 24
    return r


@pytest.mark.parametrize("stream,spi", [(0, 0.0), (1, 0.0), (0, float(1 << 21)), (1, float(1 << 20))])
def test_server_plan_rules(tmc_mod, stream, spi):
    """Photons per RSE batch: the largest power of two <= steps_per_batch /
    E[steps], within [lo, 65536] (lo = 2 x block, or 32 for the barrier-free
    kernel); items: a power-of-two split of at least lo photons each, about
    steps_per_item steps (at most twice it unless the item is at lo)."""
    from tiny_mc_gb300.serve import plan
    rng = np.random.default_rng(5)
    for _ in range(200):
        mu_a = float(np.float32(10 ** rng.uniform(-2, 1)))
        mu_s = float(np.float32(10 ** rng.uniform(0, 3)))
        b, k, e = plan(_req(mu_a, mu_s), stream=stream, steps_per_item=spi)
        lo = 32 if stream else 256
        want = 8388608.0 / max(1.0, e)
        assert b & (b - 1) == 0 and lo <= b <= 65536
        assert b == lo or b <= want
        assert b == 65536 or 2 * b > want
        assert k & (k - 1) == 0 and b % k == 0 and b // k >= lo
        if spi == 0.0:
            assert k == 1
        else:
            assert (b // k) * e <= 2 * spi or b // (2 * k) < lo
        ref = ctypes.c_double(0.0)
        assert tmc_mod.lib().tmc_expected_steps(ctypes.c_float(mu_a), ctypes.c_float(mu_s),
                                                ctypes.byref(ref)) == 0
        assert abs(e - ref.value) <= 1e-9 * ref.value


def test_server_plan_rejects_bad_requests(tmc_mod):
    from tiny_mc_gb300.serve import plan
    bad = _req(2.0, 20.0)
    bad["target_rse"] = 0.0
    with pytest.raises(tmc_mod.TmcError):
        plan(bad)
    with pytest.raises(tmc_mod.TmcError):
        plan(_req(2.0, 20.0, shells=1000))          # above max_shells (501)


def _exact_rse(vals):
    """The server's statistic from exact integer batch values (2^-40 units)."""
    import math
    xs = [float(v >> 64) * 2.0 ** 24 + float(v & (2 ** 64 - 1)) * 2.0 ** -40 for v in vals]
    tot = 0.0
    for x in xs:
        tot += x
    m = tot / len(xs)
    ss = 0.0
    for x in xs:
        ss += (x - m) * (x - m)
    return math.sqrt(ss / (len(xs) - 1) / len(xs)) / m, m


def _probes(parts):
    a = np.zeros((len(parts), 2), np.uint64)
    for i, v in enumerate(parts):
        a[i, 0] = v & (2 ** 64 - 1)
        a[i, 1] = v >> 64
    return a


@pytest.mark.parametrize("k", [1, 2, 8])
def test_batch_means_rse_exact_and_split_invariant(k):
    """Batch values summed exactly from their items' 128-bit probes (sums
    that wrap 2^64 included) give, to the last bit, the statistic of the
    unsplit batches, whatever the split."""
    import random
    from tiny_mc_gb300.serve import batch_means_rse
    rng = random.Random(11 + k)
    n = 37
    vals = [rng.randrange(1 << 60, 1 << 70) for _ in range(n)]
    parts = []
    for v in vals:
        cuts = sorted(rng.randrange(0, v) for _ in range(k - 1))
        edges = [0] + cuts + [v]
        parts += [edges[i + 1] - edges[i] for i in range(k)]
    assert max(vals) > 1 << 64                     # some batches wrap 64 bits
    rse, mean = batch_means_rse(_probes(parts), k, n)
    ref_rse, ref_mean = _exact_rse(vals)
    assert rse == ref_rse and mean == ref_mean
    whole, _ = batch_means_rse(_probes(vals), 1, n)
    assert whole == rse


def test_batch_means_rse_zero_mean_is_nan():
    from tiny_mc_gb300.serve import batch_means_rse
    rse, mean = batch_means_rse(np.zeros((4, 2), np.uint64), 1, 4)
    assert mean == 0.0 and rse != rse

