"""tmc_photon_batch_static: the photon walk for callers that cannot allocate.

Callers whose device memory belongs to someone else (a framework's pool, a
loop that forbids allocation once running) cannot let the library cudaMalloc
its scratch.  tmc_photon_batch_static keeps that scratch in a fixed array
inside the library.  These tests call it through the C ABI and check that

* it gives exactly what tmc_photon_batch gives, on calls in a row whose optics
  and shell counts change (so a call must not see the last one's leftovers),
  up to the TMC_STATIC_MAX_SHELLS maximum;
* sizes above that maximum, null arrays and photon-id overflow are refused
  with their own error text;
* in a fresh process that calls nothing else, the device's free memory does
  not change across repeated calls once the first call has loaded the module.

The file is named to run last.
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CASES = [
    dict(n=50000, seed=31, shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0, math="fast"),
    dict(n=1500, seed=32, shells=1001, microns_per_shell=10.0, mu_a=0.1, mu_s=100.0, math="exact"),
    dict(n=20000, seed=33, shells=4096, microns_per_shell=2.0, mu_a=2.0, mu_s=20.0, math="exact"),
    dict(n=30000, seed=34, shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0, math="exact"),
]


def test_static_matches_photon_batch_on_calls_in_a_row(tmc_mod):
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
        # same walk, same FP64 finalisation, same rounding to float
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
        assert got[0].sum() > 0


def test_static_rejections_carry_their_own_text(tmc_mod):
    p = tmc_mod.params(shells=tmc_mod.STATIC_MAX_SHELLS + 1)
    heat = np.zeros(p.shells, np.float32)
    heat2 = np.zeros(p.shells, np.float32)
    with pytest.raises(tmc_mod.TmcError) as e:
        tmc_mod.photon_batch_static(heat, heat2, 10, p)
    assert e.value.status == -1
    assert "TMC_STATIC_MAX_SHELLS" in str(e.value)
    assert not heat.any()
    lib = tmc_mod.lib()
    p = tmc_mod.params()
    h = np.zeros(101, np.float32)
    assert lib.tmc_photon_batch_static(None, h.ctypes.data, 10, ctypes.byref(p), None) == -1
    assert b"NULL" in lib.tmc_last_error()
    p = tmc_mod.params(photon_id_base=(1 << 64) - 5)
    assert lib.tmc_photon_batch_static(h.ctypes.data, h.ctypes.data, 10, ctypes.byref(p), None) == -5
    assert b"overflow" in lib.tmc_last_error()


# Run in a fresh interpreter that touches the GPU only through
# tmc_photon_batch_static: one zero-photon call loads the module (the set-up a
# caller makes at start-up), one real call loads the walk kernel, then the
# device's free memory is read (driver API, on the context the runtime made
# current) before and after more calls.
_CHILD = r"""
import ctypes, json, sys
import numpy as np
sys.path.insert(0, ROOT)
import tiny_mc_gb300 as t
cu = ctypes.CDLL("libcuda.so.1")
def free_bytes():
    f, tot = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert cu.cuMemGetInfo_v2(ctypes.byref(f), ctypes.byref(tot)) == 0
    return f.value
def call(n, p):
    h, h2 = np.zeros(p.shells, np.float32), np.zeros(p.shells, np.float32)
    t.photon_batch_static(h, h2, n, p)
    return h, h2
p = t.params(seed=7, math="fast")
q = t.params(seed=8, shells=4096, microns_per_shell=2.0)
call(0, p)
first = call(40000, p)
call(0, q)
before = free_bytes()
again = [call(40000, p), call(3000, q), call(40000, p)]
after = free_bytes()
same = all(np.array_equal(a, b) for a, b in zip(first, again[0])) and \
       all(np.array_equal(a, b) for a, b in zip(first, again[2]))
print(json.dumps({"before": before, "after": after, "same": bool(same),
                  "total": float(first[0].sum())}))
"""


def test_static_allocates_nothing_after_its_first_call():
    code = _CHILD.replace("ROOT", repr(ROOT))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                         env={**os.environ, "PYTHONPATH": ROOT})
    assert out.returncode == 0, out.stderr
    r = json.loads(out.stdout.strip().splitlines()[-1])
    assert r["before"] == r["after"], r
    assert r["same"] and r["total"] > 0, r
