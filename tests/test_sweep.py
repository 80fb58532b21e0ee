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
