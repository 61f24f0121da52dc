"""Regenerate the reference's random test integrals (dmrg/tests/intgen.cpp).

intgen.cpp draws every integral from a default-seeded std::mt19937 through
std::uniform_real_distribution<double>(0, 1) in a fixed loop order
(dmrg/tests/intgen.cpp:29-99) and prints 17 significant digits, so the FCIDUMP
it writes is reproduced exactly by restating:

* MT19937 (Matsumoto & Nishimura 1998), default seed 5489, 32-bit output;
* libstdc++'s generate_canonical<double, 53> on a 32-bit engine: two draws
  x0 + x1 * 2^32 scaled by 2^-64 (values that round to 1 map to the largest
  double below 1);
* the loop order and scale factors of intgen.cpp.

The reference ran this with N=6 and compared against the Block DMRG code
(dmrg/tests/check.sh): triplet -5.4268022570, singlet -5.3978872751.
"""
from __future__ import annotations

import math

import numpy as np


class MT19937:
    def __init__(self, seed: int = 5489):
        self.mt = [0] * 624
        self.mt[0] = seed & 0xFFFFFFFF
        for i in range(1, 624):
            self.mt[i] = (1812433253 * (self.mt[i - 1] ^ (self.mt[i - 1] >> 30)) + i) & 0xFFFFFFFF
        self.idx = 624

    def _twist(self):
        mt = self.mt
        for i in range(624):
            y = (mt[i] & 0x80000000) | (mt[(i + 1) % 624] & 0x7FFFFFFF)
            v = mt[(i + 397) % 624] ^ (y >> 1)
            if y & 1:
                v ^= 0x9908B0DF
            mt[i] = v
        self.idx = 0

    def __call__(self) -> int:
        if self.idx >= 624:
            self._twist()
        y = self.mt[self.idx]
        self.idx += 1
        y ^= y >> 11
        y ^= (y << 7) & 0x9D2C5680
        y ^= (y << 15) & 0xEFC60000
        y ^= y >> 18
        return y & 0xFFFFFFFF


def canonical(g: MT19937) -> float:
    s = float(g()) + float(g()) * 4294967296.0
    r = s / 18446744073709551616.0
    if r >= 1.0:
        r = math.nextafter(1.0, 0.0)
    return r


def intgen(N: int):
    """(h1, eri in chemists' notation, fcidump lines) exactly as intgen.cpp writes them."""
    g = MT19937()
    lines = []

    def put(scale, i, j, k, l):
        lines.append((scale * canonical(g), i, j, k, l))

    for i in range(N):
        put(1.0, i + 1, i + 1, i + 1, i + 1)
        for j in range(i):
            put(0.5, i + 1, i + 1, i + 1, j + 1)
            put(0.2, i + 1, i + 1, j + 1, j + 1)
            put(0.2, i + 1, j + 1, i + 1, j + 1)
            put(0.5, i + 1, j + 1, j + 1, j + 1)
            for k in range(j):
                put(0.2, i + 1, i + 1, j + 1, k + 1)
                put(0.2, i + 1, j + 1, i + 1, k + 1)
                put(0.2, i + 1, j + 1, j + 1, k + 1)
                put(0.2, j + 1, j + 1, i + 1, k + 1)
                put(0.2, i + 1, j + 1, k + 1, k + 1)
                put(0.2, i + 1, k + 1, j + 1, k + 1)
                for l in range(k):
                    put(0.1, i + 1, j + 1, k + 1, l + 1)
                    put(0.1, i + 1, k + 1, j + 1, l + 1)
                    put(0.1, i + 1, l + 1, j + 1, k + 1)
    for i in range(N):
        put(-1.0, i + 1, i + 1, 0, 0)
        for j in range(i):
            put(1.0, i + 1, j + 1, 0, 0)
    h = np.zeros((N, N))
    eri = np.zeros((N, N, N, N))
    for v, i, j, k, l in lines:
        if k == 0 and l == 0:
            h[i - 1, j - 1] = h[j - 1, i - 1] = v
        else:
            i, j, k, l = i - 1, j - 1, k - 1, l - 1
            for a, b, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                               (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                eri[a, b, c, d] = v
    return h, eri, lines
