"""The batched form on the GPU: every problem's tally in one persistent
launch is bit-identical to the plain kernel's for the same photons, for any
launch configuration, through CUDA-graph replay, and after autotuning."""
import numpy as np
import pytest

from test_gpu_parity import as_array

pytestmark = pytest.mark.gpu


def small_sweep(n=40, seed=5, scale=1 / 512, max_albedo=0.999):
    from tiny_mc_gb300.sweep import make_sweep
    sw = make_sweep(4 * n, seed=seed, photon_scale=scale, min_photons=16)
    albedo = sw["mu_s"] / (sw["mu_s"] + sw["mu_a"])
    sw = sw[albedo < max_albedo][:n].copy()
    # keep the ranges disjoint after the filter
    sw["photon_id_base"] = np.concatenate([[0], np.cumsum(sw["n_photons"][:-1])])
    return sw


def plain_tally(tmc, prob, seed, math):
    p = tmc.params(shells=int(prob["shells"]), microns_per_shell=float(prob["microns_per_shell"]),
                   mu_a=float(prob["mu_a"]), mu_s=float(prob["mu_s"]), seed=seed,
                   photon_id_base=int(prob["photon_id_base"]), math=math)
    t, steps = tmc.photon_batch_fx(int(prob["n_photons"]), p)
    return as_array(t), steps


@pytest.mark.parametrize("math,stream", [("exact", False), ("fast", False), ("exact", True),
                                         ("fast", True)])
def test_batch_equals_plain_per_problem(tmc_mod, math, stream):
    sw = small_sweep()
    b = tmc_mod.Batch(sw, seed=7, math=math)
    b.set_config(256, 8, False, stream)
    b.run()
    tallies, steps = b.read()
    for i in range(len(sw)):
        ref, ref_steps = plain_tally(tmc_mod, sw[i], 7, math)
        assert np.array_equal(as_array(b.tally_of(tallies, i)), ref), i
        assert int(steps[i]) == ref_steps
    b.close()


def test_batch_equals_oracle(tmc_mod, oracle_mod):
    sw = small_sweep(n=6, seed=11)
    b = tmc_mod.Batch(sw, seed=3, math="exact")
    b.run()
    tallies, steps = b.read()
    for i in range(len(sw)):
        q = sw[i]
        p = oracle_mod.oparams(int(q["shells"]), float(q["microns_per_shell"]), float(q["mu_a"]),
                               float(q["mu_s"]), 3)
        ref, _, ref_steps = oracle_mod.walk_fx(p, int(q["n_photons"]), id_base=int(q["photon_id_base"]))
        assert np.array_equal(as_array(b.tally_of(tallies, i)), ref)
        assert int(steps[i]) == ref_steps
    b.close()


@pytest.mark.parametrize("block,ipb,graph,stream", [
    (128, 1, False, False), (256, 64, False, False), (512, 8, True, False), (256, 8, True, False),
    (128, 1, False, True), (256, 64, True, True), (512, 16, False, True), (128, 8, True, True)])
def test_batch_config_invariance(tmc_mod, block, ipb, graph, stream):
    sw = small_sweep(n=30, seed=8)
    b = tmc_mod.Batch(sw, seed=2, math="fast")
    b.run()
    ref, ref_steps = b.read()
    b.set_config(block, ipb, graph, stream)
    for _ in range(2):                 # second pass replays the graph
        b.run()
        t, s = b.read()
        assert np.array_equal(t, ref) and np.array_equal(s, ref_steps)
    assert b.config() == {"block": block, "items_per_block": ipb, "use_graph": graph, "stream": stream}
    b.close()


def test_stream_kernel_heavy_tail_items(tmc_mod):
    """High-albedo problems split into many small items (the case the
    barrier-free kernel is for): tallies still equal the plain kernel's."""
    from tiny_mc_gb300.sweep import PROBLEM_DTYPE
    pr = np.zeros(6, PROBLEM_DTYPE)
    pr["shells"] = [101, 501, 1, 101, 501, 7]
    pr["microns_per_shell"] = 50.0
    pr["mu_a"] = [0.1, 1.0, 0.05, 2.0, 0.2, 5.0]
    pr["mu_s"] = [100.0, 200.0, 100.0, 20.0, 300.0, 1.0]
    pr["n_photons"] = [3000, 2000, 1500, 50000, 1000, 20000]
    pr["photon_id_base"] = np.concatenate([[0], np.cumsum(pr["n_photons"][:-1])])
    b = tmc_mod.Batch(pr, seed=5, math="fast")
    b.set_config(128, 64, False, True)
    b.run()
    t, s = b.read()
    for i in range(len(pr)):
        ref, steps = plain_tally(tmc_mod, pr[i], 5, "fast")
        assert np.array_equal(as_array(b.tally_of(t, i)), ref), i
        assert int(s[i]) == steps
    b.close()


def test_batch_autotune_keeps_results(tmc_mod):
    sw = small_sweep(n=24, seed=9)
    b = tmc_mod.Batch(sw, seed=4, math="fast")
    b.run()
    ref, _ = b.read()
    with pytest.raises(tmc_mod.TmcError):
        b.refine(4)                    # TMC_E_STATE: no autotune yet
    ms = b.autotune(scale=0.25, max_steps_per_photon=2e4)
    assert ms > 0
    cfg = b.config()
    assert cfg["block"] in (128, 256, 512) and cfg["items_per_block"] in (4, 8, 16, 64)
    b.run()
    t, _ = b.read()
    assert np.array_equal(t, ref)
    b.set_config(**{**b.config(), "use_graph": True})
    assert b.refine(4) > 0
    cfg = b.config()
    assert cfg["use_graph"] is True and cfg["block"] in (128, 256, 512)
    b.run()
    t, _ = b.read()
    assert np.array_equal(t, ref)
    b.close()


def test_batch_edge_cases(tmc_mod):
    from tiny_mc_gb300.sweep import PROBLEM_DTYPE
    empty = np.zeros(0, PROBLEM_DTYPE)
    b = tmc_mod.Batch(empty, seed=1)
    b.run()
    t, s = b.read()
    assert t.size == 0 and s.size == 0
    b.close()
    two = np.zeros(2, PROBLEM_DTYPE)
    two["shells"] = [5, 1]
    two["microns_per_shell"] = 50
    two["mu_a"] = [2.0, 1.0]
    two["mu_s"] = [20.0, 0.0]
    two["n_photons"] = [0, 100]
    b = tmc_mod.Batch(two, seed=1)
    b.run()
    t, s = b.read()
    assert not as_array(b.tally_of(t, 0)).any() and s[0] == 0
    ref, ref_steps = plain_tally(tmc_mod, two[1], 1, "exact")
    assert np.array_equal(as_array(b.tally_of(t, 1)), ref) and s[1] == ref_steps
    b.close()
    bad = two.copy()
    bad["mu_a"][0] = 0.0
    with pytest.raises(tmc_mod.TmcError):
        tmc_mod.Batch(bad)


def test_stream_wait_limit_reports_timeout(tmc_mod):
    """The barrier-free kernel's only wait (for a block to free an item
    buffer) is bounded: with the test hook holding every buffer, each block
    walks two items, its warps wait out a 0.5 s limit, set the error flag and
    return; the read reports TMC_E_TIMEOUT and the context stays usable."""
    import time
    from tiny_mc_gb300.sweep import PROBLEM_DTYPE
    pr = np.zeros(1, PROBLEM_DTYPE)
    pr["shells"], pr["microns_per_shell"], pr["mu_a"], pr["mu_s"] = 101, 50.0, 2.0, 20.0
    pr["n_photons"] = 1 << 22               # ~20 items per block: a third is always needed
    b = tmc_mod.Batch(pr, seed=1, math="fast")
    b.set_config(128, 64, False, True)
    b.run()
    ref, ref_s = b.read()
    b.test_wait(True, 0.5)
    t0 = time.time()
    b.run()
    with pytest.raises(tmc_mod.TmcError) as e:
        b.read()
    assert e.value.status == -4               # TMC_E_TIMEOUT
    assert time.time() - t0 < 60
    b.test_wait(False, 0.0)
    b.run()
    t, st = b.read()
    assert np.array_equal(t, ref) and np.array_equal(st, ref_s)
    b.close()

