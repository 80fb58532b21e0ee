"""Generate the golden fixtures in tests/golden/ from the reference itself.

Needs the reference tree (computacionparalela/tiny_mc) — $TMC_REFERENCE_TREE,
else a directory named "reference" beside this repository — and gcc.  It builds oracle/_ref/
(the reference's own sources compiled unchanged, see oracle/Makefile) and
records what those binaries print or compute:

  ref_params_h_seed1_stdout.txt  stdout of the reference's headless program at
                              -DSEED=1, the two timing lines (8-9) removed
  ref_native.npz              the reference's float heat/heat2 arrays after
                              srand(1) and N photons (tiny_mc.c:43-49), and
                              per-batch arrays of consecutive photon groups
                              (params_h: 32768 photons = 32 x 1024;
                              high_albedo: 4096 = 32 x 128; one_shell,
                              low_albedo: 8192 = 32 x 256; fine_shells: 8192
                              = 4 x 2048), as raw float32
  ref_injected.npz            per-photon FNV-1a hashes and summed float
                              arrays of the reference's photon() fed by the
                              oracle's Philox streams (seed 1), with the
                              oracle's logarithm (log0) and with libm logf
                              (log1): params_h photons 0..511, high_albedo
                              0..31, one_shell 0..511, low_albedo 0..2047,
                              fine_shells 0..511

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle  # noqa: E402


def main() -> None:
    oracle.build(ref=True)
    # 1. the reference binary's stdout
    out = subprocess.run([oracle.ref_binary()], capture_output=True, text=True, check=True).stdout
    lines = out.splitlines(keepends=True)
    del lines[7:9]
    with open(os.path.join(HERE, "ref_params_h_seed1_stdout.txt"), "w") as f:
        f.writelines(lines)

    # 2. native-RNG arrays and batches
    arrays = {}
    for name, n, batch in (("params_h", 32768, 1024), ("high_albedo", 4096, 128),
                           ("one_shell", 8192, 256), ("low_albedo", 8192, 256),
                           ("fine_shells", 8192, 2048)):
        h, h2 = oracle.ref_native_run(name, n, 1)
        bh, bh2 = oracle.ref_native_batches(name, n, 1, batch)
        arrays[f"{name}_n"] = np.array(n)
        arrays[f"{name}_batch"] = np.array(batch)
        arrays[f"{name}_heat"] = h
        arrays[f"{name}_heat2"] = h2
        arrays[f"{name}_bheat"] = bh
        arrays[f"{name}_bheat2"] = bh2
    np.savez_compressed(os.path.join(HERE, "ref_native.npz"), **arrays)

    # 3. the reference's photon() on injected Philox streams
    inj = {}
    for name, n in (("params_h", 512), ("high_albedo", 32), ("one_shell", 512),
                    ("low_albedo", 2048), ("fine_shells", 512)):
        for log_mode in (oracle.LOG_TMC, oracle.LOG_NATIVE):
            hashes, hs, h2s = oracle.ref_photon_hashes(name, n, seed=1, log_mode=log_mode)
            inj[f"{name}_log{log_mode}_hashes"] = hashes
            inj[f"{name}_log{log_mode}_heat"] = hs
            inj[f"{name}_log{log_mode}_heat2"] = h2s
    np.savez_compressed(os.path.join(HERE, "ref_injected.npz"), **inj)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
