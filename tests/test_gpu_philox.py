"""Cross-check of Philox-4x32-10 against cuRAND's implementation (called
through its public device API on the GPU): the oracle's C Philox, and through
it the library's device Philox (test_gpu_parity checks those are identical),
produce the same words as cuRAND for counter {i/4, 0, subseq, subseq>>32} and
key {seed, seed>>32}."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

SRC = os.path.join(ROOT, "tests", "gpu_helpers", "curand_philox.cu")
OUT = os.path.join(ROOT, "tests", "_build", "libcurand_philox.so")


@pytest.fixture(scope="module")
def curand_lib():
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < os.path.getmtime(SRC):
        from tiny_mc_gb300._build import _nvcc
        subprocess.run([_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-shared",
                        "-Xcompiler", "-fPIC", "-o", OUT, SRC], check=True)
    L = ctypes.CDLL(OUT)
    L.curand_words.argtypes = [ctypes.c_ulonglong, ctypes.c_ulonglong, ctypes.c_int, ctypes.c_void_p]
    return L


@pytest.mark.parametrize("seed,subseq", [(0, 0), (1, 0), (1, 12345), (0xdeadbeefcafe, (7 << 32) | 3)])
def test_oracle_philox_equals_curand(curand_lib, oracle_mod, seed, subseq):
    n = 64
    got = np.zeros(n, np.uint32)
    assert curand_lib.curand_words(seed, subseq, n, got.ctypes.data) == 0
    words = []
    for b in range(n // 4):
        words.extend(oracle_mod.philox([b, 0, subseq & 0xffffffff, subseq >> 32],
                                       [seed & 0xffffffff, seed >> 32]))
    assert np.array_equal(got, np.array(words, np.uint32))
