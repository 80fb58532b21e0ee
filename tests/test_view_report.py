"""The next rows beside the path, host side (no GPU): the FP64 report's
formatting and the oracle's restatement of the viewer's colour map."""
import os

import numpy as np

from conftest import GOLDEN


def parse_table(text):
    rows = [ln.split("\t") for ln in text.splitlines() if not ln.startswith("#")]
    return np.array([[float(c) for c in r] for r in rows])


def test_fp64_report_format_matches_float_report(tmc_mod):
    """The FP64 table of the reference's arrays agrees with the reference's
    own (float) table to its printed precision."""
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    p = tmc_mod.params()
    heat = g["params_h_heat"].astype(np.float64)
    heat2 = g["params_h_heat2"].astype(np.float64)
    n = 32768
    t = 4.0 * np.pi * 50.0 ** 3 * n / 1e12
    i = np.arange(100, dtype=np.float64)
    shell = i * i + i + 1.0 / 3.0
    dens = heat[:100] / t / shell
    with np.errstate(invalid="ignore"):
        err = np.sqrt(heat2[:100] - heat[:100] ** 2 / n) / t / shell
    text = tmc_mod.format_report_fp64(dens, err, heat[100] / n, p)
    golden = open(os.path.join(GOLDEN, "ref_params_h_seed1_stdout.txt")).read()
    a = parse_table(text)
    b = parse_table("".join(golden.splitlines(keepends=True)[7:]))
    assert a.shape == b.shape == (100, 3)
    assert np.array_equal(a[:, 0], b[:, 0])
    assert np.allclose(a[:, 1], b[:, 1], rtol=1e-5, atol=2e-5)
    ok = np.isfinite(b[:, 2]) & np.isfinite(a[:, 2])
    assert np.allclose(a[ok, 2], b[ok, 2], rtol=1e-4, atol=2e-5)
    assert text.splitlines()[-1].startswith("# extra\t")


def test_oracle_colormap_formula(oracle_mod):
    """The restated shader: centre pixel maps to shell 0, corners to the last
    shells; red follows 2/(1+exp(-0.004 h)) - 1."""
    heats = np.linspace(0.0, 2000.0, 101).astype(np.float32)
    red, rgba = oracle_mod.colormap(heats, 800, 800)
    assert red.shape == (800, 800) and rgba.shape == (800, 800, 4)
    c = red[399, 399]     # pixel centre (399.5, 399.5)/800 - 0.5 -> dr ~ 0.000625 -> shell 0
    assert abs(c - (2.0 / (1.0 + np.exp(-0.004 * 0.0)) - 1.0)) < 1e-6
    corner = red[0, 0]    # dr = 0.70622 -> shell int(0.99875 * 100) = 99
    assert abs(corner - (2.0 / (1.0 + np.exp(-0.004 * heats[99])) - 1.0)) < 1e-6
    assert np.all(rgba[..., 3] == 255) and np.all(rgba[..., 1:3] == 0)
    # radially symmetric
    assert np.array_equal(red, red[::-1, :]) and np.array_equal(red, red[:, ::-1])
