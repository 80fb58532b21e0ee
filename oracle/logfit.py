"""How the coefficients of the library's logarithm were chosen (TEST
INFRASTRUCTURE ONLY: a derivation, not part of the product path).

The exact arithmetic mode evaluates log x for x in [2^-31, 1] (the step length
of photon.c:21) as  k ln2 + f + f^2 R(f),  m = 2^-k x in [sqrt(1/2), sqrt(2)),
f = m - 1.  R(f) = (Q(f) - 1) / f where Q(f) = log1p(f) / f is replaced by its
interpolant at the 10 Chebyshev nodes of [sqrt(1/2) - 1, sqrt(2) - 1]
(degree 9, computed here with 60-digit arithmetic), whose constant term is 1;
the nine other coefficients, rounded to float, are R's.  Run:

    python oracle/logfit.py          # prints the coefficients (hex floats) and
                                     # the relative error of Q with them

The float evaluation itself (Horner with fma, tmo_logf in tmc_oracle.c) is
checked against the C library's double log by tmo_logf_max_ulp: over every
float of [2^-31, 1] the largest error is 0.86 ulp.
"""
from __future__ import annotations

import struct

import mpmath as mp


def coefficients(degree: int = 9):
    mp.mp.dps = 60
    a = mp.sqrt(mp.mpf(0.5)) - 1
    b = mp.sqrt(mp.mpf(2)) - 1

    def q(f):
        return mp.log1p(f) / f if f != 0 else mp.mpf(1)

    n = degree
    nodes = [(a + b) / 2 + (b - a) / 2 * mp.cos(mp.pi * (2 * k + 1) / (2 * (n + 1))) for k in range(n + 1)]
    v = mp.matrix([[x ** j for j in range(n + 1)] for x in nodes])
    c = mp.lu_solve(v, mp.matrix([q(x) for x in nodes]))
    as_f32 = [struct.unpack("f", struct.pack("f", float(c[j])))[0] for j in range(n + 1)]
    xs = [a + (b - a) * mp.mpf(i) / 2000 for i in range(2001)]
    err = max(abs(sum(mp.mpf(as_f32[j]) * x ** j for j in range(n + 1)) / q(x) - 1) for x in xs)
    return as_f32, float(err)


if __name__ == "__main__":
    cf, err = coefficients()
    print("Q coefficients (c0 .. c9):", [float.hex(x) for x in cf])
    print("R coefficients, Horner order (c9 .. c1):", [float.hex(x) for x in cf[:0:-1]])
    print("max relative error of Q with float coefficients:", err)
