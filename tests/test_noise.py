"""make_noise (src/canonicalize.hpp:11-24) on the host: the oracle's MT19937 against
the C++ standard's known answers, the library's noise sequence (the same standard
library engine and distribution the reference calls) bit-exact against the oracle's
restatement, and the oracle's block layout of the noise array."""
import numpy as np
import pytest

from oracle import dmrg as od
from tests.bondcase import repeated_sector_psi


def test_mt19937_known_answers():
    w = od.mt19937_words(10000)
    # first output of a default-constructed std::mt19937 and the 10000th, which the
    # C++ standard requires ([rand.predef])
    assert int(w[0]) == 3499211612
    assert int(w[9999]) == 4123659995
    # restarting gives the same stream (the reference reseeds on every call)
    assert np.array_equal(od.mt19937_words(700), w[:700])


def test_noise_sequence_is_generate_canonical_of_word_pairs():
    w = od.mt19937_words(8)
    seq = od.noise_sequence(4)
    for j in range(4):
        r = (float(w[2 * j]) + float(w[2 * j + 1]) * 2.0**32) / 2.0**64
        assert seq[j] == r * 2.0 - 1.0
    big = od.noise_sequence(50000)
    assert big.min() >= -1.0 and big.max() < 1.0
    assert abs(big.mean()) < 0.02


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300._lib import lib as _lib

    return _lib()


def test_library_noise_sequence_bit_exact(lib):
    from mpsxx_gb300 import core

    n = 300000  # covers the largest blocks of the benchmark wavefunctions
    a = od.noise_sequence(n)
    b = core.noise_sequence(n)
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    assert core.noise_sequence(0).size == 0


def test_oracle_make_noise_layout():
    psi = repeated_sector_psi()
    before = {t: b.copy() for t, b in psi.blocks.items()}
    od.make_noise(psi, 1e-9)  # below the threshold: unchanged
    assert sorted(psi.blocks) == sorted(before)
    assert all(np.array_equal(before[t], psi.blocks[t]) for t in before)
    noise = 1e-3
    od.make_noise(psi, noise)
    seq = od.noise_sequence(64)
    # (0, 1) and (1, 0) are allowed and their sectors are seen in stored blocks: added;
    # (2, 2) is allowed but its sectors appear in no stored block (net dimension 0)
    assert sorted(psi.blocks) == sorted(psi.tag(i) for i in [(0, 0), (0, 1), (1, 0), (1, 1)])
    for t, b in psi.blocks.items():
        n = b.size
        ref = before.get(t, None)
        expect = seq[:n].reshape(b.shape) * noise if ref is None else ref + noise * seq[:n].reshape(b.shape)
        assert np.array_equal(b, expect)


def test_canonicalize_with_noise_changes_truncation():
    from tests.bondcase import hubbard_bond

    case = hubbard_bond()
    U0, V0, k0 = od.canonicalize_merged(True, case["psi"].copy(), case["M"], 0.0)
    p = case["psi"].copy()
    U1, V1, k1 = od.canonicalize_merged(True, p, case["M"], 1e-3)
    assert k0 != k1
    # unique sector quantum numbers: each row sector pairs with one column sector, so
    # the noise array has exactly the stored blocks
    assert sorted(p.blocks) == sorted(case["psi"].blocks)
