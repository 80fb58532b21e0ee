"""The C-ABI library loads, exports every symbol include/tmc.h declares, and
its host-only logic (defaults, validation, the tiny_mc report) is right.
No call here launches a kernel, so this runs without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT


def declared_functions(header):
    src = open(header).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(tmc_[a-z0-9_]+)\s*\(", src)))


def test_exports_every_declared_symbol(tmc_mod):
    names = declared_functions(os.path.join(ROOT, "include", "tmc.h"))
    assert len(names) >= 10
    out = subprocess.run(["nm", "-D", "--defined-only", tmc_mod.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tmc_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    lib = tmc_mod.lib()
    for n in names:
        assert hasattr(lib, n)


def test_params_default_is_params_h(tmc_mod):
    p = tmc_mod.Params()
    tmc_mod.lib().tmc_params_default(ctypes.byref(p))
    assert (p.shells, p.microns_per_shell, p.mu_a, p.mu_s) == (101, 50.0, 2.0, 20.0)
    assert p.seed == 1 and p.photon_id_base == 0 and p.math == tmc_mod.MATH_EXACT
    assert ctypes.sizeof(tmc_mod.Params) == 40
    assert tmc_mod.TALLY_DTYPE.itemsize == 32


@pytest.mark.parametrize("field,value", [
    ("shells", 0), ("mu_a", 0.0), ("mu_a", -1.0), ("mu_a", float("nan")), ("mu_s", -1.0),
    ("mu_s", float("inf")), ("microns_per_shell", 0.0), ("math", 7), ("reserved", 1),
    ("mu_a", 1e-9),   # float albedo rounds to 1: the weight would never decay
])
def test_invalid_params_rejected_before_any_launch(tmc_mod, field, value):
    p = tmc_mod.params()
    setattr(p, field, value)
    heat = np.zeros(101, np.float32)
    heat2 = np.zeros(101, np.float32)
    with pytest.raises(tmc_mod.TmcError) as e:
        tmc_mod.photon_batch(heat, heat2, 10, p)
    assert e.value.status == -1
    assert not heat.any()


def test_shell_count_limit(tmc_mod):
    """1 .. 2^24 shells: above that (float)(shells - 1), the clamp bound of
    photon.c:27-29 done in float, would no longer be exact."""
    import ctypes
    p = tmc_mod.params(shells=(1 << 24) + 1)
    heat = np.zeros(101, np.float32)
    st = tmc_mod.lib().tmc_photon_batch(heat.ctypes.data, heat.ctypes.data, 10, ctypes.byref(p))
    assert st == -1 and not heat.any()


def test_null_arrays_rejected(tmc_mod):
    p = tmc_mod.params()
    assert tmc_mod.lib().tmc_photon_batch(None, None, 1, ctypes.byref(p)) == -1
    assert tmc_mod.lib().tmc_photon_batch_fx(None, 1, ctypes.byref(p), None) == -1
    assert tmc_mod.lib().tmc_set_plain_launch(100, 0, 0) == -1
    assert tmc_mod.lib().tmc_set_plain_launch(0, 0, -1) == -1
    assert tmc_mod.lib().tmc_set_plain_launch(0, 0, 0) == 0


def test_strerror(tmc_mod):
    for code in range(-8, 1):
        assert tmc_mod.lib().tmc_strerror(code)


def test_report_reproduces_reference_stdout(tmc_mod):
    """tmc_format_report on the reference's own float arrays (srand(1), 32768
    photons) prints byte-for-byte the table the reference printed."""
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    golden = open(os.path.join(GOLDEN, "ref_params_h_seed1_stdout.txt")).read().splitlines(keepends=True)
    p = tmc_mod.params()
    table = tmc_mod.format_report(g["params_h_heat"], g["params_h_heat2"], 32768, p)
    assert table == "".join(golden[7:])


def test_tally_to_heat_host(tmc_mod):
    p = tmc_mod.params()
    t = np.zeros(p.shells, tmc_mod.TALLY_DTYPE)
    t["w_lo"][3] = 1 << 40          # sum_w = 1.0
    t["w_hi"][4] = 1                # sum_w = 2^24
    t["w2_lo"][3] = 1 << 39         # sum_w2 = 0.5
    heat, heat2 = tmc_mod.tally_to_heat(t, p)
    _, c, _ = tmc_mod.derived(p)
    assert heat[3] == float(c) and heat[4] == float(c) * 2.0 ** 24
    assert heat2[3] == float(c) * float(c) * 0.5
    assert heat[0] == 0.0


def test_python_mirror_rejects_bad_arrays(tmc_mod):
    p = tmc_mod.params()
    with pytest.raises(ValueError):
        tmc_mod.photon_batch(np.zeros(10, np.float32), np.zeros(101, np.float32), 1, p)
    with pytest.raises(ValueError):
        tmc_mod.photon_batch(np.zeros(101, np.float64), np.zeros(101, np.float32), 1, p)


def test_batch_and_server_entry_points_reject_null_handles(tmc_mod):
    """Checked before any CUDA call, so this runs without a GPU."""
    import ctypes
    from tiny_mc_gb300 import serve  # noqa: F401  (sets up the server prototypes)
    serve._setup(tmc_mod.lib())
    L = tmc_mod.lib()
    ms = ctypes.c_double(0.0)
    assert L.tmc_batch_run(None, None) == -1
    assert L.tmc_batch_autotune(None, 0.5, 0.0, ctypes.byref(ms)) == -1
    assert L.tmc_batch_refine(None, 4, ctypes.byref(ms)) == -1
    assert L.tmc_batch_test_wait(None, 1, 0.5) == -1
    assert L.tmc_batch_destroy(None) == 0
    assert L.tmc_server_submit(None, None, None) == -1
    assert L.tmc_server_progress(None, None, None) == -1
    assert L.tmc_server_run_trace(None, None, None, 0, 0.0, None, None) == -1
    assert L.tmc_server_destroy(None) == 0


def test_error_text_is_specific_and_per_thread(tmc_mod):
    import ctypes
    import threading
    L = tmc_mod.lib()
    h = np.zeros(101, np.float32)
    p = tmc_mod.params(shells=(1 << 24) + 1)
    assert L.tmc_photon_batch(h.ctypes.data, h.ctypes.data, 10, ctypes.byref(p)) == -1
    mine = L.tmc_last_error()
    assert b"shells" in mine

    def other():
        q = tmc_mod.params(mu_a=0.0)
        assert L.tmc_photon_batch(h.ctypes.data, h.ctypes.data, 10, ctypes.byref(q)) == -1
        assert b"mu_a" in L.tmc_last_error()

    t = threading.Thread(target=other)
    t.start()
    t.join()
    assert L.tmc_last_error() == mine          # another thread's failure left ours alone

