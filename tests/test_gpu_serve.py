"""The request server on the GPU: a request's result is the same alone and in
a mix of concurrent requests, equals the plain kernel over the same photons,
stops by its rule, and admission refuses requests when slots are full.  Each
check runs on the four ways the server can drive the GPU: waves of the
kernel with per-item barriers or of the barrier-free kernel, and a
persistent launch of either, fed from a work queue in mapped host memory."""
import math

import numpy as np
import pytest

from test_gpu_parity import as_array

pytestmark = pytest.mark.gpu


def req(mu_a=2.0, mu_s=20.0, shells=101, rse=0.02, cap=1 << 20, base=0):
    from tiny_mc_gb300.serve import REQUEST_DTYPE
    r = np.zeros(1, REQUEST_DTYPE)[0]
    r["shells"], r["microns_per_shell"], r["mu_a"], r["mu_s"] = shells, 50.0, mu_a, mu_s
    r["target_rse"], r["max_photons"], r["photon_id_base"] = rse, cap, base
    return r


# server modes: waves of the kernel with per-item barriers, waves of the
# barrier-free kernel, one persistent launch fed from a work queue
MODES = {"waves_batch": dict(stream=0), "waves_stream": dict(stream=1), "persistent": dict(persistent=1),
         "persistent_stream": dict(persistent=1, stream=1)}
OTHER = {"waves_batch": "persistent", "waves_stream": "waves_batch", "persistent": "persistent_stream",
         "persistent_stream": "waves_stream"}

MIX = [req(2.0, 20.0, 101, 0.02, base=1 << 32), req(0.5, 50.0, 501, 0.03, base=2 << 32),
       req(5.0, 5.0, 101, 0.01, base=3 << 32), req(1.0, 300.0, 501, 0.05, base=4 << 32),
       req(0.02, 2.0, 101, 0.04, cap=1 << 16, base=5 << 32)]


@pytest.mark.parametrize("mode", list(MODES))
def test_alone_equals_in_mix(tmc_mod, mode):
    from tiny_mc_gb300.serve import Server
    probe = req(1.0, 30.0, 101, 0.02, base=9 << 32)
    s = Server(slots=8, **MODES[OTHER[mode]])      # alone, driven the other way
    rid = s.submit(probe)
    alone = s.run({rid: 101})[rid]
    s.close()
    s = Server(slots=8, **MODES[mode])
    ids = {s.submit(r): int(r["shells"]) for r in MIX[:3]}
    rid = s.submit(probe)
    ids[rid] = 101
    ids.update({s.submit(r): int(r["shells"]) for r in MIX[3:]})
    out = s.run(ids)
    s.close()
    t_alone, r_alone = alone
    t_mix, r_mix = out[rid]
    assert np.array_equal(t_alone, t_mix)
    for f in ("photons", "photon_steps", "batches", "batch_photons", "reached_target"):
        assert r_alone[f] == r_mix[f], f
    assert r_alone["rse"] == r_mix["rse"]


@pytest.mark.parametrize("mode", list(MODES))
def test_result_equals_plain_kernel_and_rule(tmc_mod, mode):
    from tiny_mc_gb300.serve import Server
    s = Server(slots=8, **MODES[mode])
    ids = {s.submit(r): int(r["shells"]) for r in MIX}
    out = s.run(ids)
    s.close()
    for (rid, sh), r in zip(ids.items(), MIX):
        tally, res = out[rid]
        n = int(res["photons"])
        assert n == int(res["batches"]) * int(res["batch_photons"])
        p = tmc_mod.params(shells=sh, microns_per_shell=50.0, mu_a=float(r["mu_a"]), mu_s=float(r["mu_s"]),
                           seed=1, photon_id_base=int(r["photon_id_base"]), math="fast")
        ref, steps = tmc_mod.photon_batch_fx(n, p)
        assert np.array_equal(as_array(tally), as_array(ref))
        assert int(res["photon_steps"]) == steps
        b = int(res["batches"])
        if res["reached_target"]:
            assert res["rse"] <= r["target_rse"]
        else:
            assert n >= int(r["max_photons"]) or b * int(res["batch_photons"]) >= int(r["max_photons"])
        # decisions only at 16, 32, 64, ... batches, or at the cap
        cap_b = -(-int(r["max_photons"]) // int(res["batch_photons"]))
        assert b == cap_b or (b >= 16 and (b & (b - 1)) == 0)


@pytest.mark.parametrize("mode", list(MODES))
def test_item_split_does_not_change_results(tmc_mod, mode):
    """RSE batches split into several work items (walked by different blocks),
    fewer launches in flight and a small in-flight item budget give the same
    tallies, steps, batch counts and RSE to the last bit."""
    from tiny_mc_gb300.serve import Server
    out = []
    for spi, waves, items in ((0.0, 0, 0), (float(1 << 16), 4, 64)):
        s = Server(slots=8, steps_per_item=spi, waves=waves, inflight_items=items, **MODES[mode])
        ids = {s.submit(r): int(r["shells"]) for r in MIX}
        out.append(s.run(ids))
        s.close()
    assert sorted(out[0]) == sorted(out[1])     # ids 1..5 in submit order on both servers
    for rid in out[0]:
        (ta, xa), (tb, xb) = out[0][rid], out[1][rid]
        assert np.array_equal(ta, tb)
        for f in ("photons", "photon_steps", "batches", "batch_photons", "reached_target", "rse"):
            assert xa[f] == xb[f], f


def test_admission_refuses_when_full(tmc_mod):
    from tiny_mc_gb300.serve import Server
    s = Server(slots=2)
    a = s.submit(MIX[0])
    b = s.submit(MIX[1])
    assert a is not None and b is not None
    assert s.submit(MIX[2]) is None          # TMC_E_BUSY: the caller queues
    s.run({a: 101, b: 501})
    c = s.submit(MIX[2])                      # a slot freed up
    assert c is not None
    s.run({c: 101})
    s.close()


@pytest.mark.parametrize("mode", list(MODES))
def test_run_trace_small(tmc_mod, mode):
    from tiny_mc_gb300.serve import Server, make_trace
    req_, arr = make_trace(60, rate=400.0, seed=3, mu_a_range=(0.5, 10.0), mu_s_range=(1.0, 100.0),
                           rse=(0.02, 0.05), max_photons=1 << 18)
    s = Server(slots=16, **MODES[mode])
    res, done = s.run_trace(req_, arr, time_limit_s=120.0)
    assert done == 60
    assert np.all(res["latency_s"] > 0) and np.all(res["photons"] > 0)
    photons, steps, waves = s.stats()
    assert photons == int(res["photons"].sum()) and waves > 0
    s.close()


@pytest.mark.parametrize("mode,spi", [("waves_batch", 0.0), ("waves_stream", 0.0), ("persistent", 0.0),
                                      ("persistent_stream", 0.0), ("waves_batch", float(1 << 24)),
                                      ("waves_stream", float(1 << 22)), ("persistent", float(1 << 24)),
                                      ("persistent_stream", float(1 << 22))])
def test_rse_from_exact_batch_probes_with_wraps(tmc_mod, mode, spi):
    """One shell and albedo 0.9999 with 2048-photon batches: each batch's sum
    of w in the probe shell (~2e7 weight units) exceeds 2^64 fixed-point
    units, so the per-item probe must count its wraps.  The server's RSE must
    equal, to the last bit, the batch-means RSE recomputed from per-batch
    plain-kernel tallies of the same photons."""
    from tiny_mc_gb300.serve import Server
    r = req(mu_a=0.1, mu_s=1000.0, shells=1, rse=1e-9, cap=32 * 2048, base=77 << 32)
    s = Server(slots=4, steps_per_batch=float(1 << 28), steps_per_item=spi, **MODES[mode])
    rid = s.submit(r)
    tally, res = s.run({rid: 1})[rid]
    s.close()
    B = int(res["batch_photons"])
    assert B == 2048 and int(res["batches"]) == 32 and not res["reached_target"]
    xs = []
    for j in range(32):
        p = tmc_mod.params(shells=1, microns_per_shell=50.0, mu_a=0.1, mu_s=1000.0, seed=1,
                           photon_id_base=(77 << 32) + j * B, math="fast")
        t, _ = tmc_mod.photon_batch_fx(B, p)
        xs.append(float(int(t["w_hi"][0])) * 2.0 ** 24 + float(int(t["w_lo"][0])) * 2.0 ** -40)
    assert max(xs) > 2.0 ** 24          # the per-batch sums did wrap 64 bits
    k = len(xs)
    tot = 0.0
    for x in xs:          # in batch order, uncompensated, as the server sums
        tot += x
    m = tot / k
    ss = 0.0
    for x in xs:
        ss += (x - m) * (x - m)
    rse = math.sqrt(ss / (k - 1) / k) / m
    assert res["rse"] == rse
