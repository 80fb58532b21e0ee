"""The next rows beside the path on the GPU: the viewer's colour map kernel
against the oracle's restatement, the progressive walk's snapshots against
one batch call, and the FP64 report against the same formula on the host."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from test_gpu_parity import as_array

pytestmark = pytest.mark.gpu


def test_colormap_kernel_matches_oracle(tmc_mod, oracle_mod):
    from tiny_mc_gb300.view import colormap
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    for heats, w, h in [(g["params_h_heat"], 800, 800), (g["high_albedo_heat"], 640, 480),
                        (np.linspace(0, 3000, 7).astype(np.float32), 1000, 900)]:
        red, rgba = colormap(heats, w, h)
        ored, orgba = oracle_mod.colormap(heats, w, h)
        assert np.max(np.abs(red - ored)) < 2e-6
        diff = np.abs(rgba.astype(int) - orgba.astype(int))
        assert diff.max() <= 1 and (diff == 0).mean() > 0.999


def test_progressive_snapshots_equal_one_call(tmc_mod):
    from tiny_mc_gb300.view import Progressive, colormap
    p = tmc_mod.params(seed=17, math="fast")
    g = Progressive(p)
    seen = []
    for _ in range(5):
        g.advance(20000)
        new, heat, heat2, n = g.snapshot(wait=False)
        if new:
            seen.append(n)
    new, heat, heat2, n = g.snapshot(wait=True)
    assert n == 100000 and (new or seen[-1] == 100000)
    assert seen == sorted(seen)
    ref = np.zeros(101, np.float32), np.zeros(101, np.float32)
    tmc_mod.photon_batch(ref[0], ref[1], 100000, p)
    assert np.array_equal(heat, ref[0]) and np.array_equal(heat2, ref[1])
    img = g.render(800, 800)
    _, want = colormap(heat, 800, 800)
    assert np.array_equal(img, want)
    g.close()


def test_report_fp64_matches_host_formula(tmc_mod):
    p = tmc_mod.params(seed=5)
    n = 1 << 16
    tally, _ = tmc_mod.photon_batch_fx(n, p)
    dens, err, extra = tmc_mod.report_fp64(tally, p, n)
    heat, heat2 = tmc_mod.tally_to_heat(tally, p)
    t = 4.0 * np.pi * 50.0 ** 3 * n / 1e12
    i = np.arange(100, dtype=np.float64)
    shell = i * i + i + 1.0 / 3.0
    assert np.allclose(dens, heat[:100] / t / shell, rtol=1e-12, atol=0)
    with np.errstate(invalid="ignore"):
        want = np.sqrt(heat2[:100] - heat[:100] ** 2 / n) / t / shell
    ok = np.isfinite(want)
    assert np.allclose(err[ok], want[ok], rtol=1e-9, atol=0)
    assert np.array_equal(np.isnan(err), np.isnan(want))
    assert extra == pytest.approx(heat[100] / n, rel=1e-12)
    text = tmc_mod.format_report_fp64(dens, err, extra, p)
    assert len(text.splitlines()) == 103


def test_dropin_driver_output(tmc_mod, tmp_path):
    """The drop-in tiny_mc prints the reference's layout: 7 header lines, the
    two timing lines, the two column titles, 100 rows and "# extra"; its heat
    column agrees with the reference's seed-1 run (libc rand, 32768 photons)
    within |z| <= 4 in every shell.  Sigma is batch means: the reference's
    32 batches of 1024 photons give the variance of a 32768-photon total, and
    the drop-in's run (same photon count, other streams) has the same, so the
    difference's variance is twice it."""
    import subprocess
    from tiny_mc_gb300 import _build
    golden = open(os.path.join(GOLDEN, "ref_params_h_seed1_stdout.txt")).read().splitlines()
    ref = np.array([[float(c) for c in ln.split("\t")] for ln in golden if not ln.startswith("#")])
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    bheat = g["params_h_bheat"].astype(np.float64)
    var_total = len(bheat) * bheat.var(0, ddof=1)
    i = np.arange(100, dtype=np.float64)
    vol = 4.0 * np.pi * 50.0 ** 3 * 32768 / 1e12 * (i * i + i + 1.0 / 3.0)
    sigma_density = np.sqrt(2.0 * var_total[:100]) / vol
    for extra_args in ([], ["exact", "fp64", str(tmp_path / "heat.ppm")]):
        out = subprocess.run([_build.DRIVER, "32768", "1"] + extra_args, capture_output=True, text=True,
                             check=True).stdout.splitlines()
        assert len(out) == 7 + 2 + 2 + 100 + 1
        assert out[3].startswith("# Scattering =   20.000/cm") and out[5].startswith("# Photons    =    32768")
        assert out[7].startswith("# ") and out[7].endswith("seconds")
        rows = np.array([[float(c) for c in ln.split("\t")] for ln in out[11:111]])
        assert np.array_equal(rows[:, 0], ref[:, 0])
        z = (rows[:, 1] - ref[:, 1]) / sigma_density
        assert np.abs(z).max() < 4.0, (np.abs(z).max(), int(np.abs(z).argmax()))
        assert out[-1].startswith("# extra\t")
    ppm = (tmp_path / "heat.ppm").read_bytes()
    assert ppm.startswith(b"P6\n800 800\n255\n") and len(ppm) == len(b"P6\n800 800\n255\n") + 800 * 800 * 3
