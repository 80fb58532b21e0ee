"""tmc_photon_batch_static: the photon walk for callers that cannot allocate.

Callers whose device memory belongs to someone else (a framework's pool, a
loop that forbids allocation once running) cannot let the library cudaMalloc
its scratch.  tmc_photon_batch_static keeps that scratch in a fixed array
inside the library.  These tests call it through the C ABI and compare it
with tmc_photon_batch on two calls in a row (the second with other optics and
more shells, so it must not see the first call's leftovers), and check the
size limit.  The file is named to run last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    dict(n=50000, seed=31, shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0),
    dict(n=1500, seed=32, shells=1001, microns_per_shell=10.0, mu_a=0.1, mu_s=100.0),
]


def test_static_matches_photon_batch_on_two_calls(tmc_mod):
    lib = tmc_mod.lib()
    for case in CASES:
        c = dict(case)
        n = c.pop("n")
        p = tmc_mod.params(**c)
        ref = np.zeros(p.shells, np.float32), np.zeros(p.shells, np.float32)
        tmc_mod.photon_batch(ref[0], ref[1], n, p)
        got = np.zeros(p.shells, np.float32), np.zeros(p.shells, np.float32)
        st = lib.tmc_photon_batch_static(got[0].ctypes.data, got[1].ctypes.data, n,
                                         ctypes.byref(p), None)
        assert st == 0, lib.tmc_last_error()
        np.testing.assert_allclose(got[0], ref[0], rtol=1e-6, atol=0)
        np.testing.assert_allclose(got[1], ref[1], rtol=1e-6, atol=0)
        assert got[0].sum() > 0


def test_static_rejects_shells_above_limit(tmc_mod):
    p = tmc_mod.params(shells=tmc_mod.STATIC_MAX_SHELLS + 1)
    heat = np.zeros(p.shells, np.float32)
    heat2 = np.zeros(p.shells, np.float32)
    with pytest.raises(tmc_mod.TmcError) as e:
        tmc_mod.photon_batch_static(heat, heat2, 10, p)
    assert e.value.status == -1
    assert "TMC_STATIC_MAX_SHELLS" in str(e.value)
    assert not heat.any()
