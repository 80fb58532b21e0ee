"""Host-side logic of the batched form (no GPU): the sweep generator and the
planner's expected-steps estimate (photon.c's weight recursion)."""
import numpy as np
import pytest


def test_sweep_distribution():
    from tiny_mc_gb300.sweep import make_sweep
    sw = make_sweep(4096, seed=0)
    assert len(sw) == 4096
    assert sw["mu_a"].min() >= 0.01 * 0.999 and sw["mu_a"].max() <= 10.0 * 1.001
    assert sw["mu_s"].min() >= 1.0 * 0.999 and sw["mu_s"].max() <= 1000.0 * 1.001
    assert set(np.unique(sw["shells"])) == {101, 501}
    assert sw["n_photons"].min() >= 2 ** 12 and sw["n_photons"].max() < 2 ** 22
    # log-uniform: the medians sit at the geometric middle of the ranges
    assert abs(np.log10(np.median(sw["mu_a"])) - (-0.5)) < 0.1
    assert abs(np.log10(np.median(sw["mu_s"])) - 1.5) < 0.1
    # disjoint photon-id ranges
    ends = sw["photon_id_base"] + sw["n_photons"]
    assert np.all(sw["photon_id_base"][1:] == ends[:-1])
    # seeded: the same draw twice, a different one for another seed
    assert np.array_equal(make_sweep(64, seed=0), make_sweep(64, seed=0))
    assert not np.array_equal(make_sweep(64, seed=1)["mu_a"], make_sweep(64, seed=0)["mu_a"])


def test_scaled_sweep_keeps_the_mix():
    from tiny_mc_gb300.sweep import make_sweep
    a = make_sweep(256, seed=3)
    b = make_sweep(256, seed=3, photon_scale=1 / 64, min_photons=64)
    assert np.array_equal(a["mu_a"], b["mu_a"]) and np.array_equal(a["shells"], b["shells"])
    assert np.all(b["n_photons"] >= 64) and b["n_photons"].sum() < a["n_photons"].sum() / 32


@pytest.mark.parametrize("mu_a,mu_s,n", [(2.0, 20.0, 20000), (0.1, 100.0, 300), (10.0, 1.0, 20000),
                                         (1.0, 200.0, 1000)])
def test_expected_steps_matches_oracle(tmc_mod, oracle_mod, mu_a, mu_s, n):
    """The planner's expected steps per photon against the oracle's measured
    mean (it only steers load balance, so 5% is plenty)."""
    est = tmc_mod.expected_steps(mu_a, mu_s)
    _, _, steps = oracle_mod.walk_fx(oracle_mod.oparams(101, 50.0, mu_a, mu_s, 1), n)
    assert abs(est - steps / n) / (steps / n) < 0.05


def test_expected_steps_known_values(tmc_mod):
    # 75.667 steps per photon at params.h optics (73 to the first roulette,
    # 24 per survival), 7168 at the high-albedo optics
    assert abs(tmc_mod.expected_steps(2.0, 20.0) - 75.667) < 0.01
    assert abs(tmc_mod.expected_steps(0.1, 100.0) - 7168.0) < 1.0


# ----------------------------------------------------- the batch planner (host)
def _check_partition(pr, items):
    """Every problem's photon range [0, n) is covered exactly once."""
    for i in range(len(pr)):
        mine = items[items[:, 0] == i]
        mine = mine[np.argsort(mine[:, 1])]
        n = int(pr["n_photons"][i])
        if n == 0:
            assert len(mine) == 0
            continue
        assert int(mine[0, 1]) == 0
        assert np.all(mine[1:, 1] == mine[:-1, 1] + mine[:-1, 2])
        assert int(mine[-1, 1] + mine[-1, 2]) == n
        assert np.all(mine[:, 2] > 0) and np.all(mine[:, 2] < 1 << 30)


@pytest.mark.parametrize("grid,block,ipb", [(1520, 128, 8), (456, 512, 16), (7, 256, 1), (3000, 128, 64)])
def test_plan_items_partition_and_order(tmc_mod, grid, block, ipb):
    from tiny_mc_gb300.sweep import make_sweep
    pr = make_sweep(300, seed=4, photon_scale=1.0 / 64, min_photons=16)
    pr["n_photons"][::37] = 0                       # empty problems get no items
    items = tmc_mod.plan_items(pr, grid, block, ipb)
    _check_partition(pr, items)
    est = np.array([tmc_mod.expected_steps(float(a), float(b)) for a, b in zip(pr["mu_a"], pr["mu_s"])])
    work = est[items[:, 0].astype(int)] * items[:, 2]
    assert np.all(work[:-1] >= work[1:])            # heaviest first
    for i in range(len(pr)):                        # no item below one photon per lane, unless
        n = int(pr["n_photons"][i])                 # the problem is that small
        k = int(np.sum(items[:, 0] == i))
        assert k <= max(1, -(-n // block))


def test_plan_items_one_photon_per_lane_rule(tmc_mod):
    """A problem whose photons are so long that two in a row would reach the
    launch's expected steps per lane is split down to one photon per lane;
    otherwise items keep two photons per lane."""
    from tiny_mc_gb300.sweep import PROBLEM_DTYPE
    pr = np.zeros(2, PROBLEM_DTYPE)
    pr["shells"], pr["microns_per_shell"] = 101, 50.0
    pr["mu_a"], pr["mu_s"] = [0.01, 2.0], [1000.0, 20.0]      # ~7e5 and ~76 steps per photon
    grid, block = 100, 128
    pr["n_photons"] = [4096, 1000]
    items = tmc_mod.plan_items(pr, grid, block, 8)
    heavy = items[items[:, 0] == 0]
    assert len(heavy) == 4096 // block and np.all(heavy[:, 2] == block)
    pr["n_photons"] = [4096, 1 << 30]               # light work dominates: lanes have room
    items = tmc_mod.plan_items(pr, grid, block, 8)
    heavy = items[items[:, 0] == 0]
    assert len(heavy) == 4096 // (2 * block) and np.all(heavy[:, 2] == 2 * block)
    _check_partition(pr, items)


def test_plan_items_rejects_bad_input(tmc_mod):
    from tiny_mc_gb300.sweep import PROBLEM_DTYPE
    pr = np.zeros(1, PROBLEM_DTYPE)
    pr["shells"], pr["microns_per_shell"], pr["mu_a"], pr["mu_s"], pr["n_photons"] = 101, 50.0, 0.0, 20.0, 10
    with pytest.raises(tmc_mod.TmcError):
        tmc_mod.plan_items(pr, 10, 128, 8)          # mu_a = 0
    pr["mu_a"] = 2.0
    with pytest.raises(tmc_mod.TmcError):
        tmc_mod.plan_items(pr, 0, 128, 8)           # no grid

