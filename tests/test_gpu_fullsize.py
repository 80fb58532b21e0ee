"""Parity at the full workload sizes through properties that do not need the
oracle to finish: 2^30 photons at params.h optics and 2^28 photons at the
high-albedo optics (1001 shells of 10 um).

* Additivity: the exact 128-bit tally of the whole photon-id range equals the
  sum of the tallies of its sub-ranges (bit for bit), and so do the photon
  steps.
* Launch-shape invariance at full size.
* Energy conservation: the roulette (photon.c:45-49) is unbiased, so every
  launched unit of weight is eventually absorbed in the infinite medium.  The
  weight sequence of photon.c:32 and :48 is deterministic in float between
  roulette survivals, so the expected total deposit per photon (and the
  expected steps per photon) follow exactly from that float recursion and a
  geometric number of survivals; the measured means must match within 5
  batch-means sigma of the sub-range values.
"""
import numpy as np
import pytest

from test_gpu_parity import as_array

pytestmark = pytest.mark.gpu


def float_recursion_expectation(mu_a, mu_s):
    """(E[sum of deposits (1-a) w], E[steps]) per photon of photon.c's float
    weight recursion, deposits in the 2^-40 fixed point the tallies use."""
    f32 = np.float32
    a = f32(f32(mu_s) / f32(f32(mu_s) + f32(mu_a)))
    c = f32(f32(1.0) - a)
    e_fx, e_steps, prob, w = 0, 0.0, 1.0, f32(1.0)
    for _ in range(14):
        fx, k = 0, 0
        while True:
            fx += int(np.rint(np.float64(w) * 2.0 ** 40))
            k += 1
            w = f32(w * a)
            if w < f32(0.001):
                break
        e_fx += prob * fx
        e_steps += prob * k
        w = f32(w / f32(0.1))
        prob *= 0.1
    return float(c) * e_fx * 2.0 ** -40, e_steps


def sums128(t):
    return [(int(r[1]) << 64) | int(r[0]) for r in t], [(int(r[3]) << 64) | int(r[2]) for r in t]


@pytest.mark.parametrize("optics,n,parts", [
    (dict(shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0), 1 << 30, 64),
    (dict(shells=1001, microns_per_shell=10.0, mu_a=0.1, mu_s=100.0), 1 << 28, 16),
])
def test_full_size_properties(tmc_mod, optics, n, parts):
    p = tmc_mod.params(seed=1, math="fast", **optics)
    whole, steps = tmc_mod.photon_batch_fx(n, p)
    whole = as_array(whole)
    per = n // parts
    acc_w = [0] * optics["shells"]
    acc_w2 = [0] * optics["shells"]
    totals, steps_parts, steps_sum = [], [], 0
    _, c, _ = tmc_mod.derived(p)
    for k in range(parts):
        q = tmc_mod.params(seed=1, math="fast", photon_id_base=k * per, **optics)
        t, s = tmc_mod.photon_batch_fx(per, q)
        sw, sw2 = sums128(as_array(t))
        acc_w = [a + b for a, b in zip(acc_w, sw)]
        acc_w2 = [a + b for a, b in zip(acc_w2, sw2)]
        totals.append(float(c) * sum(sw) * 2.0 ** -40 / per)
        steps_parts.append(s / per)
        steps_sum += s
    W, W2 = sums128(whole)
    assert W == acc_w and W2 == acc_w2
    assert steps == steps_sum
    e_total, e_steps = float_recursion_expectation(optics["mu_a"], optics["mu_s"])
    totals = np.array(totals)
    se = totals.std(ddof=1) / np.sqrt(parts)
    assert abs(totals.mean() - e_total) < 5 * se, (totals.mean(), e_total, se)
    assert abs(e_total - 1.0) < 1e-5          # and that is (nearly) all the launched weight
    sp = np.array(steps_parts)
    assert abs(sp.mean() - e_steps) < 5 * sp.std(ddof=1) / np.sqrt(parts), (sp.mean(), e_steps)


def test_full_size_launch_shape_invariance(tmc_mod):
    p = tmc_mod.params(seed=1, math="fast")
    n = 1 << 30
    a, sa = tmc_mod.photon_batch_fx(n, p)
    tmc_mod.set_plain_launch(512, 1, 0)
    try:
        b, sb = tmc_mod.photon_batch_fx(n, p)
    finally:
        tmc_mod.set_plain_launch(0, 0, 0)
    assert np.array_equal(as_array(a), as_array(b)) and sa == sb
