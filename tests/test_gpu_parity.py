"""GPU parity: the CUDA walk (through the C ABI) against the CPU oracle.

Exact arithmetic (TMC_MATH_EXACT) must give integer tallies bit-identical to
the FP32 restatement of photon.c driven by the same Philox streams; the
restatement itself is pinned to the reference's photon.c (test_oracle.py).
Both arithmetic modes must agree with the FP64 oracle to 1e-4 per shell (every
shell with >= 1e4 deposits) at params.h optics, and with the reference's own
libc-rand run within |z| <= 4 (batch-means sigma).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

PARAMS_H = dict(shells=101, microns_per_shell=50.0, mu_a=2.0, mu_s=20.0)
HIGH_ALBEDO = dict(shells=1001, microns_per_shell=10.0, mu_a=0.1, mu_s=100.0)


def as_array(tally):
    return np.stack([tally["w_lo"], tally["w_hi"], tally["w2_lo"], tally["w2_hi"]], axis=1)


def gpu_fx(tmc, n, math="exact", seed=1, base=0, **optics):
    p = tmc.params(seed=seed, photon_id_base=base, math=math, **optics)
    tally, steps = tmc.photon_batch_fx(n, p)
    return as_array(tally), steps


def oracle_fx(o, n, seed=1, base=0, **optics):
    p = o.oparams(optics["shells"], optics["microns_per_shell"], optics["mu_a"], optics["mu_s"], seed)
    return o.walk_fx(p, n, id_base=base)


@pytest.fixture(autouse=True)
def default_launch(tmc_mod):
    tmc_mod.set_plain_launch(0, 0, 0)
    yield
    tmc_mod.set_plain_launch(0, 0, 0)


def test_device_rand_stream_matches_oracle(tmc_mod, oracle_mod):
    for seed, photon in [(1, 0), (1, 12345), (0xdeadbeefcafe, (7 << 32) | 3)]:
        got = tmc_mod.debug_rand(seed, photon, 1001)
        assert np.array_equal(got, oracle_mod.stream(seed, photon, 1001))


@pytest.mark.parametrize("seed,base,n", [(1, 0, 1 << 16), (12345, 1 << 40, 50000)])
def test_exact_bit_identical_params_h(tmc_mod, oracle_mod, seed, base, n):
    got, steps = gpu_fx(tmc_mod, n, seed=seed, base=base, **PARAMS_H)
    ref, dep, ref_steps = oracle_fx(oracle_mod, n, seed=seed, base=base, **PARAMS_H)
    assert steps == ref_steps
    assert np.array_equal(got, ref)


def test_exact_bit_identical_high_albedo(tmc_mod, oracle_mod):
    n = 2048
    got, steps = gpu_fx(tmc_mod, n, **HIGH_ALBEDO)
    ref, _, ref_steps = oracle_fx(oracle_mod, n, **HIGH_ALBEDO)
    assert steps == ref_steps
    assert np.array_equal(got, ref)


def test_exact_bit_identical_random_optics(tmc_mod, oracle_mod):
    rng = np.random.default_rng(7)
    for _ in range(8):
        mu_a = float(np.float32(10 ** rng.uniform(-0.5, 1)))
        mu_s = float(np.float32(10 ** rng.uniform(0, 2)))
        optics = dict(shells=int(rng.choice([1, 2, 101, 501])), microns_per_shell=float(rng.choice([10, 50, 125])),
                      mu_a=mu_a, mu_s=mu_s)
        n = int(rng.integers(100, 3000))
        seed = int(rng.integers(1, 1 << 62))
        base = int(rng.integers(0, 1 << 50))
        got, steps = gpu_fx(tmc_mod, n, seed=seed, base=base, **optics)
        ref, _, ref_steps = oracle_fx(oracle_mod, n, seed=seed, base=base, **optics)
        assert steps == ref_steps, optics
        assert np.array_equal(got, ref), optics


@pytest.mark.parametrize("name,n", [("one_shell", 8192), ("low_albedo", 65536), ("fine_shells", 8192)])
def test_exact_bit_identical_edge_optics(tmc_mod, oracle_mod, name, n):
    """The optics the oracle is also pinned at against the reference's own
    photon.c: one shell (every deposit clamped), a roulette every few steps,
    4001 shells of 1 um (many photons clamped into the last shell)."""
    shells, mps, mu_a, mu_s = oracle_mod.CONFIGS[name]
    optics = dict(shells=shells, microns_per_shell=mps, mu_a=mu_a, mu_s=mu_s)
    got, steps = gpu_fx(tmc_mod, n, seed=11, base=1 << 36, **optics)
    ref, _, ref_steps = oracle_fx(oracle_mod, n, seed=11, base=1 << 36, **optics)
    assert steps == ref_steps
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("shells,mps,n,nt", [(20000, 0.5, 4096, 0), (1 << 24, 0.001, 64, 1)])
def test_exact_bit_identical_wide_tallies(tmc_mod, oracle_mod, shells, mps, n, nt):
    """Shell counts whose histogram does not fit in shared memory: deposits go
    straight to the 128-bit global tally; up to the 2^24-shell maximum, where
    (float)(shells - 1) is still exact for the clamp of photon.c:27-29."""
    optics = dict(shells=shells, microns_per_shell=mps, mu_a=2.0, mu_s=20.0)
    got, steps = gpu_fx(tmc_mod, n, seed=5, **optics)
    p = oracle_mod.oparams(shells, mps, 2.0, 20.0, 5)
    ref, dep, ref_steps = oracle_mod.walk_fx(p, n, nthreads=nt)
    assert steps == ref_steps
    assert np.array_equal(got, ref)
    assert int((dep > 0).sum()) > 1000          # deposits spread over many shells


@pytest.mark.parametrize("n", [0, 1, 31, 32, 33, 255, 257, 4097])
def test_edge_photon_counts(tmc_mod, oracle_mod, n):
    got, steps = gpu_fx(tmc_mod, n, seed=3, **PARAMS_H)
    ref, _, ref_steps = oracle_fx(oracle_mod, n, seed=3, **PARAMS_H)
    assert steps == ref_steps
    assert np.array_equal(got, ref)


@pytest.mark.parametrize("block,bpsm,maxb", [(128, 0, 0), (256, 1, 0), (512, 0, 0), (512, 1, 3), (128, 2, 1)])
def test_launch_shape_invariance(tmc_mod, block, bpsm, maxb):
    base, _ = gpu_fx(tmc_mod, 40000, seed=11, **PARAMS_H)
    tmc_mod.set_plain_launch(block, bpsm, maxb)
    got, _ = gpu_fx(tmc_mod, 40000, seed=11, **PARAMS_H)
    assert np.array_equal(got, base)


def test_split_ranges_add_up(tmc_mod):
    whole, s0 = gpu_fx(tmc_mod, 30000, seed=5, **PARAMS_H)
    a, s1 = gpu_fx(tmc_mod, 12345, seed=5, base=0, **PARAMS_H)
    b, s2 = gpu_fx(tmc_mod, 30000 - 12345, seed=5, base=12345, **PARAMS_H)
    tot = [(int(a[i, 1]) << 64 | int(a[i, 0])) + (int(b[i, 1]) << 64 | int(b[i, 0])) for i in range(101)]
    assert tot == [int(whole[i, 1]) << 64 | int(whole[i, 0]) for i in range(101)]
    assert s1 + s2 == s0


@pytest.mark.parametrize("shells,mps", [(1, 50.0), (1001, 1e7)])
def test_carry_paths_128bit(tmc_mod, oracle_mod, shells, mps):
    """One block, high albedo, every deposit in shell 0 (one shell, or 1001
    shells of 10 m): the shell's sums reach several 2^64 fixed-point units
    (sum of w ~ 6.6e7 weight units = 3.9 * 2^64, sum of w^2 ~ 1.9 * 2^64).
    With one shell the kernel keeps a histogram per warp, which each warp adds
    into the global tally every 2^18 lane steps (a lane walks ~1.9e6 steps
    here, so every warp flushes several times mid-walk); with 1001 shells it
    keeps one per block, whose 64-bit shared sums wrap and carry into the
    global high words.  Both must equal the oracle bit for bit."""
    optics = dict(shells=shells, microns_per_shell=mps, mu_a=0.1, mu_s=400.0)
    n = 16384
    tmc_mod.set_plain_launch(256, 1, 1)
    got, steps = gpu_fx(tmc_mod, n, seed=9, **optics)
    ref, _, ref_steps = oracle_fx(oracle_mod, n, seed=9, **optics)
    assert ref[0, 1] >= 3 and ref[0, 3] >= 1      # high words in use
    assert steps == ref_steps
    assert np.array_equal(got, ref)


def test_photon_batch_float_accumulates(tmc_mod, oracle_mod):
    p = tmc_mod.params(seed=2, **PARAMS_H)
    heat = np.zeros(101, np.float32)
    heat2 = np.zeros(101, np.float32)
    tmc_mod.photon_batch(heat, heat2, 20000, p)
    first = heat.copy()
    tmc_mod.photon_batch(heat, heat2, 20000, p)       # same photons again: doubles
    assert np.allclose(heat, 2 * first, rtol=1e-6)
    ref, _, _ = oracle_fx(oracle_mod, 20000, seed=2, **PARAMS_H)
    h, h2 = oracle_mod.heat_from_tally(oracle_mod.cfg("params_h"), ref)
    assert np.allclose(first, h.astype(np.float32), rtol=1e-6)
    assert np.allclose(heat2, (2 * h2).astype(np.float32), rtol=1e-6)


def test_device_entry_point(tmc_mod):
    torch = pytest.importorskip("torch")
    p = tmc_mod.params(seed=4, **PARAMS_H)
    d = torch.zeros((101, 4), dtype=torch.int64, device="cuda")
    steps = torch.zeros(1, dtype=torch.int64, device="cuda")
    ws = torch.zeros(tmc_mod.workspace_bytes() // 8, dtype=torch.int64, device="cuda")
    s = torch.cuda.current_stream().cuda_stream
    p1 = tmc_mod.params(seed=4, photon_id_base=0, **PARAMS_H)
    p2 = tmc_mod.params(seed=4, photon_id_base=7000, **PARAMS_H)
    tmc_mod.photon_batch_device(d.data_ptr(), 7000, p1, steps.data_ptr(), ws.data_ptr(), s)
    tmc_mod.photon_batch_device(d.data_ptr(), 13000, p2, steps.data_ptr(), 0, s)
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(np.uint64)
    ref, ref_steps = gpu_fx(tmc_mod, 20000, seed=4, **PARAMS_H)
    assert np.array_equal(got, ref)
    assert int(steps.item()) == ref_steps
    del p


def test_device_form_shared_workspace_is_ordered(tmc_mod, oracle_mod):
    """tmc_photon_batch_device with no workspace uses the library's own photon
    claim counter, the one the host-array calls use too.  A device-form walk
    still running on a side stream (one block, so it lasts) must not have that
    counter reset under it by a host-array call made right after it on the
    library's stream: both tallies must equal the oracle's bit for bit."""
    torch = pytest.importorskip("torch")
    n_dev, n_host = 1 << 16, 4096
    d = torch.zeros((101, 4), dtype=torch.int64, device="cuda")
    side = torch.cuda.Stream()
    tmc_mod.set_plain_launch(512, 1, 1)
    p_dev = tmc_mod.params(seed=21, photon_id_base=0, **PARAMS_H)
    with torch.cuda.stream(side):
        tmc_mod.photon_batch_device(d.data_ptr(), n_dev, p_dev, 0, 0, side.cuda_stream)
    host, host_steps = gpu_fx(tmc_mod, n_host, seed=21, base=n_dev, **PARAMS_H)
    side.synchronize()
    dev = d.cpu().numpy().view(np.uint64)
    ref_dev, _, _ = oracle_fx(oracle_mod, n_dev, seed=21, base=0, **PARAMS_H)
    ref_host, _, ref_host_steps = oracle_fx(oracle_mod, n_host, seed=21, base=n_dev, **PARAMS_H)
    assert np.array_equal(dev, ref_dev)
    assert np.array_equal(host, ref_host) and host_steps == ref_host_steps


@pytest.mark.parametrize("math,n", [("exact", 1 << 20), ("fast", 1 << 20), ("exact", 1 << 24),
                                    ("fast", 1 << 24)])
def test_vs_fp64_oracle_params_h(tmc_mod, oracle_mod, math, n):
    """Gate (a): 1e-4 relative in every shell with >= 1e4 deposits, against
    the FP64 oracle on the same streams (params.h optics; 2^24 photons is the
    largest count the FP64 oracle walks in seconds on the host's cores)."""
    got, _ = gpu_fx(tmc_mod, n, math=math, **PARAMS_H)
    p = oracle_mod.cfg("params_h")
    h, _ = oracle_mod.heat_from_tally(p, got)
    h64, _, dep = oracle_mod.walk_f64(p, n)
    m = dep >= 10000
    assert m.sum() >= 100
    rel = np.abs(h[m] - h64[m]) / h64[m]
    print(f"{math} 2^{n.bit_length() - 1} photons vs FP64: max rel {rel.max():.3g} over {m.sum()} shells")
    assert rel.max() < 1e-4, rel.max()


def test_fast_vs_exact_high_albedo(tmc_mod, oracle_mod):
    """High albedo (7168 steps/photon, 0.001-mfp shells): the FP32 walk itself
    differs from FP64 by shell-boundary flips; the fast arithmetic must stay
    within the same envelope as the exact (= reference) arithmetic."""
    n = 1 << 14
    ex, _ = gpu_fx(tmc_mod, n, math="exact", **HIGH_ALBEDO)
    fa, _ = gpu_fx(tmc_mod, n, math="fast", **HIGH_ALBEDO)
    p = oracle_mod.cfg("high_albedo")
    he, _ = oracle_mod.heat_from_tally(p, ex)
    hf, _ = oracle_mod.heat_from_tally(p, fa)
    h64, _, dep = oracle_mod.walk_f64(p, n)
    m = dep >= 10000
    rel_e = np.abs(he[m] - h64[m]) / h64[m]
    rel_f = np.abs(hf[m] - h64[m]) / h64[m]
    print(f"high_albedo vs FP64: exact max {rel_e.max():.3g} median {np.median(rel_e):.3g}; "
          f"fast max {rel_f.max():.3g} median {np.median(rel_f):.3g}")
    assert rel_f.max() < 3 * rel_e.max() + 1e-4
    assert np.median(rel_f) < 3 * np.median(rel_e) + 1e-5


@pytest.mark.parametrize("math", ["exact", "fast"])
def test_native_rng_zscore(tmc_mod, math):
    """Gate (b): GPU (Philox) vs the reference's own libc-rand run (seed 1,
    32768 photons in 32 batches): per-shell |z| <= 4, batch-means sigma."""
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    ref = g["params_h_bheat"].astype(np.float64) / int(g["params_h_batch"])
    nb, per = 64, 1 << 14
    means = []
    for b in range(nb):
        t, _ = gpu_fx(tmc_mod, per, math=math, base=b * per, **PARAMS_H)
        h = tmc_mod.tally_to_heat(np.ascontiguousarray(t).view(tmc_mod.TALLY_DTYPE).reshape(-1),
                                  tmc_mod.params(**PARAMS_H))[0]
        means.append(h / per)
    means = np.array(means)
    se = np.sqrt(means.var(0, ddof=1) / nb + ref.var(0, ddof=1) / len(ref))
    z = (means.mean(0) - ref.mean(0)) / se
    assert np.all(np.abs(z[:-1]) < 4.0), np.abs(z).max()


@pytest.mark.parametrize("math", ["exact", "fast"])
def test_native_rng_zscore_high_albedo(tmc_mod, math):
    """Gate (b) at high-albedo optics (1001 shells of 10 um, ~7168 steps per
    photon): GPU (Philox, 64 batches of 2^12 photons) against the reference's
    own libc-rand run (seed 1, 4096 photons in 32 batches of 128), batch-means
    sigma.  The reference's 128-photon batches make each of the 1000 shells'
    sigma a 31-degree-of-freedom estimate, so |z| <= 4 is applied to the heat
    of 32-shell groups (one test per group, 32 groups), and per shell at 5.4,
    the threshold whose chance of being crossed once among 1000 shells under
    the null equals that of 4 sigma for a single shell (two-sided 6.3e-5)."""
    g = np.load(os.path.join(GOLDEN, "ref_native.npz"))
    ref = g["high_albedo_bheat"].astype(np.float64) / int(g["high_albedo_batch"])
    nb, per = 64, 1 << 12
    means = []
    for b in range(nb):
        t, _ = gpu_fx(tmc_mod, per, math=math, base=b * per, **HIGH_ALBEDO)
        h = tmc_mod.tally_to_heat(np.ascontiguousarray(t).view(tmc_mod.TALLY_DTYPE).reshape(-1),
                                  tmc_mod.params(**HIGH_ALBEDO))[0]
        means.append(h / per)
    means = np.array(means)
    se = np.sqrt(means.var(0, ddof=1) / nb + ref.var(0, ddof=1) / len(ref))
    z = (means.mean(0) - ref.mean(0)) / se
    gi = np.arange(1000) // 32
    grp = lambda a: np.stack([np.bincount(gi, weights=row[:1000]) for row in a])  # noqa: E731
    gm, gr = grp(means), grp(ref)
    zg = (gm.mean(0) - gr.mean(0)) / np.sqrt(gm.var(0, ddof=1) / nb + gr.var(0, ddof=1) / len(gr))
    print(f"high_albedo {math}: max |z| per 32-shell group {np.abs(zg).max():.2f}, "
          f"per shell {np.abs(z[:-1]).max():.2f}, last shell {z[-1]:.2f}")
    assert np.all(np.abs(zg) < 4.0)
    assert np.all(np.abs(z) < 5.4)
