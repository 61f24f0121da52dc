"""Parameter Jacobians of the MPO generators (host only): the MPOs are linear in
the Hamiltonian parameters, so d(block)/d(theta) must reproduce the change of every
block under a parameter step exactly (to rounding), and tracking must not change
the MPO itself."""
import numpy as np
import pytest

from mpsxx_gb300 import mpogen


def block_delta(a, b, eps):
    keys = set(a["blocks"]) | set(b["blocks"])
    z = np.zeros((1, 1, 1, 1))
    return {k: (b["blocks"].get(k, z) - a["blocks"].get(k, z)).item() / eps for k in keys}


def check_linear(sites, sites_p, jacs, par, eps):
    worst = 0.0
    hits = 0
    for a, b, j in zip(sites, sites_p, jacs):
        for k, d in block_delta(a, b, eps).items():
            pred = j.get(k, {}).get(par, 0.0)
            hits += pred != 0.0
            worst = max(worst, abs(d - pred))
    return worst, hits


def test_hubbard_jacobian_is_exact():
    L = 7
    rng = np.random.default_rng(1)
    t = -rng.uniform(0.8, 1.2, L - 1)
    U = rng.uniform(2.0, 6.0, L)
    sites, jacs = mpogen.hubbard_mpo(L, t, U, jacobian=True)
    plain = mpogen.hubbard_mpo(L, t, U)
    assert [s["blocks"].keys() for s in sites] == [s["blocks"].keys() for s in plain]
    eps = 1e-3
    for k in range(L):
        up = U.copy()
        up[k] += eps
        worst, hits = check_linear(sites, mpogen.hubbard_mpo(L, t, up), jacs, ("U", k), eps)
        assert hits >= 1 and worst < 1e-9
    for k in range(L - 1):
        tp = t.copy()
        tp[k] += eps
        worst, hits = check_linear(sites, mpogen.hubbard_mpo(L, tp, U), jacs, ("t", k), eps)
        assert hits >= 4 and worst < 1e-9


@pytest.mark.parametrize("pq", [(0, 0), (1, 3), (3, 1), (4, 2)])
def test_qc_h_jacobian_is_exact(pq):
    n = 5
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 2)
    sites, jacs = mpogen.qc_mpo(h1, eri, jacobian=True)
    plain = mpogen.qc_mpo(h1, eri)
    for a, b in zip(sites, plain):
        assert a["blocks"].keys() == b["blocks"].keys()
        assert all(np.array_equal(a["blocks"][k], b["blocks"][k]) for k in a["blocks"])
    eps = 1e-3
    h2 = h1.copy()
    h2[pq] += eps
    worst, hits = check_linear(sites, mpogen.qc_mpo(h2, eri), jacs, ("h",) + pq, eps)
    assert hits >= 1 and worst < 1e-9


def test_parameter_gradient_contracts_site_gradients():
    from mpsxx_gb300.dmrg import parameter_gradient

    jacs = [{3: {"a": 2.0}, 5: {"a": 1.0, "b": -1.0}}, {0: {"b": 4.0}}]
    tags = [np.array([3, 5, 9]), np.array([0, 1])]
    grads = [np.array([1.0, 10.0, 100.0]), np.array([0.5, 7.0])]
    d = parameter_gradient(grads, tags, jacs)
    assert d == {"a": 2.0 * 1.0 + 1.0 * 10.0, "b": -10.0 + 4.0 * 0.5}
