"""One-site stage (src/optimize.hpp:37-145, src/dmrg.cpp:80-115) on the merged
hot path (needs a GPU): after the two-site stage, one-site sweeps reproduce the
exact energy when M is exact, and stay variational, above the two-site sweep energy
by at most the truncation scale, when M truncates."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    return core.Context(0)


@pytest.mark.parametrize("M", [256, 24])
def test_two_then_one_site_stages(ctx, M):
    from oracle import ed
    from mpsxx_gb300 import dmrg
    from mpsxx_gb300.mpogen import hubbard_mpo

    L = 8
    rng = np.random.default_rng(11)
    U = rng.uniform(2.0, 6.0, L)
    t = -rng.uniform(0.8, 1.2, L - 1)
    exact = ed.hubbard_ground_energy(L, t, U, L // 2, L // 2)[0]
    st, logs = dmrg.dmrg(ctx, hubbard_mpo(L, t, U), L, 0, M, 1e-10, 12, onesite=True)
    two = [g for g in logs if g.kind == "twosite"]
    one = [g for g in logs if g.kind == "onesite"]
    assert two and one
    e2, e1 = two[-1].energy, one[-1].energy
    print(f"M={M}: exact {exact:.12f} two-site {e2:.12f} one-site {e1:.12f}")
    assert e1 >= exact - 1e-9 and e2 >= exact - 1e-9
    if M == 256:
        assert abs(e1 - exact) < 1e-9 and abs(e2 - exact) < 1e-9
    else:
        # the two-site sweep energy is taken before truncation (4M states at the bond),
        # the one-site one inside M states: apart by the truncation error
        assert e2 - 1e-9 <= e1 < e2 + 1e-3
