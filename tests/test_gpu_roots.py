"""Multiple roots (needs a GPU): state-specific DMRG with the lower roots projected out
of H_eff (the projected Functor of src/diagonalize.hpp:200-277) reproduces the lowest
eigenvalues of exact diagonalisation where the bond dimension is exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    return core.Context(0)


def test_three_lowest_hubbard_roots_match_ed(ctx):
    from oracle import ed
    from mpsxx_gb300 import dmrg
    from mpsxx_gb300.mpogen import hubbard_mpo

    L = 6
    U = np.array([4.0, 3.0, 5.0, 4.5, 2.5, 3.5])
    t = -np.array([1.0, 0.9, 1.1, 1.0, 0.95])
    exact = ed.hubbard_ground_energy(L, t, U, 3, 3, k=3)
    es, _ = dmrg.dmrg_roots(ctx, hubbard_mpo(L, t, U), L, 0, 64, 1e-11, 12, 3, seed=5)
    print("roots", es, "exact", list(exact))
    assert np.max(np.abs(np.array(es) - exact)) < 1e-8
