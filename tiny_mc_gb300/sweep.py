"""The batched sweep workload: independent problems with the parameter
distribution of the 4096-problem configuration (mu_a log-uniform in
[0.01, 10]/cm, mu_s log-uniform in [1, 1000]/cm, SHELLS uniform over
{101, 501}, MICRONS_PER_SHELL 50, photon counts log-uniform in [2^12, 2^22]),
drawn from a seeded generator.  No public dataset is involved.  Problems get
disjoint photon-id ranges, so every photon of the sweep has its own stream.
"""
from __future__ import annotations

import numpy as np

PROBLEM_DTYPE = np.dtype([
    ("shells", "<u4"), ("microns_per_shell", "<f4"), ("mu_a", "<f4"), ("mu_s", "<f4"),
    ("n_photons", "<u8"), ("photon_id_base", "<u8"),
])


def make_sweep(n: int = 4096, seed: int = 0, photon_scale: float = 1.0,
               min_photons: int = 1, log2_photons=(12.0, 22.0), mu_a_range=(0.01, 10.0),
               mu_s_range=(1.0, 1000.0), shells=(101, 501), microns_per_shell: float = 50.0):
    """Structured array of `n` problems (PROBLEM_DTYPE).  photon_scale
    multiplies every photon count (a reduced copy of the same mix)."""
    rng = np.random.default_rng(seed)
    mu_a = np.float32(10.0 ** rng.uniform(np.log10(mu_a_range[0]), np.log10(mu_a_range[1]), n))
    mu_s = np.float32(10.0 ** rng.uniform(np.log10(mu_s_range[0]), np.log10(mu_s_range[1]), n))
    sh = rng.choice(np.asarray(shells, np.uint32), n)
    photons = np.floor(2.0 ** rng.uniform(log2_photons[0], log2_photons[1], n))
    photons = np.maximum(min_photons, np.round(photons * photon_scale)).astype(np.uint64)
    out = np.zeros(n, PROBLEM_DTYPE)
    out["shells"] = sh
    out["microns_per_shell"] = microns_per_shell
    out["mu_a"] = mu_a
    out["mu_s"] = mu_s
    out["n_photons"] = photons
    base = np.zeros(n, np.uint64)
    if n > 1:
        base[1:] = np.cumsum(photons[:-1], dtype=np.uint64)
    out["photon_id_base"] = base
    return out
