"""Energy gradient with respect to the MPO and the Hamiltonian parameters (needs a
GPU): the adjoint of the merged-operator scatter, pulled through the MPO generator.

Checked against central finite differences (step 1e-4) of exact-diagonalisation
energies on systems small enough for DMRG with bond dimension M to be exact, to
1e-6 relative; the split-precision gradient against the FP64 one to 1e-5 relative;
right environments recomputed from checkpoints against all-stored environments to
1e-12.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    c = core.Context(0)
    yield c
    core.set_precision(c, core.FP64)


def converge(ctx, sites, n_elec, M, tole, sweeps):
    from mpsxx_gb300 import core, dmrg

    mpo = [core.Tensor.from_dict(ctx, d) for d in sites]
    st = dmrg.make_initial_state(ctx, mpo, n_elec, 0, M)
    log = None
    for _ in range(sweeps):
        log = dmrg.make_sweep(ctx, st, tole)
    return st, log


def params_gradient(ctx, st, jacs, checkpoint):
    from mpsxx_gb300 import dmrg

    g = dmrg.gradient_sweep(ctx, st, checkpoint=checkpoint)
    tags = [m.blocks()[0] for m in st.mpo]
    return g, dmrg.parameter_gradient(g.site_grads, tags, jacs)


@pytest.fixture(scope="module")
def hubbard_case(ctx):
    from mpsxx_gb300.mpogen import hubbard_mpo

    L = 8
    rng = np.random.default_rng(3)
    U = rng.uniform(2.0, 6.0, L)
    t = -rng.uniform(0.8, 1.2, L - 1)
    sites, jacs = hubbard_mpo(L, t, U, jacobian=True)
    st, log = converge(ctx, sites, L, 256, 1e-12, 5)
    return dict(L=L, U=U, t=t, jacs=jacs, st=st, log=log)


def test_hubbard_gradient_matches_exact_finite_differences(ctx, hubbard_case):
    from oracle import ed

    c = hubbard_case
    L, U, t = c["L"], c["U"], c["t"]
    g, dE = params_gradient(ctx, c["st"], c["jacs"], checkpoint=3)
    e_ed = ed.hubbard_ground_energy(L, t, U, L // 2, L // 2)[0]
    assert abs(c["log"].energy - e_ed) < 1e-9
    assert max(abs(e - c["log"].energy) for e in g.bond_energies) < 1e-9
    assert g.env_recomputed > 0
    h = 1e-4
    worst = 0.0
    for k in range(L):
        up, um = U.copy(), U.copy()
        up[k] += h
        um[k] -= h
        fd = (ed.hubbard_ground_energy(L, t, up, L // 2, L // 2)[0] -
              ed.hubbard_ground_energy(L, t, um, L // 2, L // 2)[0]) / (2 * h)
        worst = max(worst, abs(dE[("U", k)] - fd) / max(1.0, abs(fd)))
    for k in range(L - 1):
        tp, tm = t.copy(), t.copy()
        tp[k] += h
        tm[k] -= h
        fd = (ed.hubbard_ground_energy(L, tp, U, L // 2, L // 2)[0] -
              ed.hubbard_ground_energy(L, tm, U, L // 2, L // 2)[0]) / (2 * h)
        worst = max(worst, abs(dE[("t", k)] - fd) / max(1.0, abs(fd)))
    print("hubbard L=8 adjoint vs exact FD: worst relative error", worst)
    assert worst < 1e-6


def test_checkpointed_environments_give_the_same_gradient(ctx, hubbard_case):
    c = hubbard_case
    g1, d1 = params_gradient(ctx, c["st"], c["jacs"], checkpoint=1)
    g4, d4 = params_gradient(ctx, c["st"], c["jacs"], checkpoint=4)
    assert g1.env_recomputed == 0 and g4.env_recomputed > 0
    assert g4.env_peak < g1.env_peak
    for k in d1:
        assert abs(d1[k] - d4[k]) < 1e-12 * max(1.0, abs(d1[k]))


def test_split_gradient_matches_fp64(ctx, hubbard_case):
    from mpsxx_gb300 import core

    c = hubbard_case
    _, d64 = params_gradient(ctx, c["st"], c["jacs"], checkpoint=4)
    core.set_precision(ctx, core.SPLIT_TF32)
    try:
        _, d32 = params_gradient(ctx, c["st"], c["jacs"], checkpoint=4)
    finally:
        core.set_precision(ctx, core.FP64)
    worst = max(abs(d32[k] - d64[k]) / max(1.0, abs(d64[k])) for k in d64)
    print("split vs fp64 gradient: worst relative difference", worst)
    assert worst < 1e-5


def test_qc_h_gradient_matches_exact_finite_differences(ctx):
    from oracle import ed
    from mpsxx_gb300 import mpogen

    n = 6
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 4)
    sites, jacs = mpogen.qc_mpo(h1, eri, jacobian=True)
    st, log = converge(ctx, sites, n, 64, 1e-12, 5)
    e_ed = ed.qc_ground_energy(h1, eri, n // 2, n // 2)[0]
    assert abs(log.energy - e_ed) < 1e-9
    _, dE = params_gradient(ctx, st, jacs, checkpoint=2)
    hstep = 1e-4
    worst = 0.0
    for p, q in [(0, 0), (2, 2), (0, 1), (1, 3), (2, 5), (4, 5)]:
        hp, hm = h1.copy(), h1.copy()
        for hh, sgn in ((hp, 1.0), (hm, -1.0)):
            hh[p, q] += sgn * hstep
            if p != q:
                hh[q, p] += sgn * hstep
        fd = (ed.qc_ground_energy(hp, eri, n // 2, n // 2)[0] - ed.qc_ground_energy(hm, eri, n // 2, n // 2)[0]) / (
            2 * hstep)
        adj = dE.get(("h", p, q), 0.0) + (dE.get(("h", q, p), 0.0) if p != q else 0.0)
        worst = max(worst, abs(adj - fd) / max(1.0, abs(fd)))
    print("qc n=6 dE/dh adjoint vs exact FD: worst relative error", worst)
    assert worst < 1e-6


def test_qc_gradient_through_the_reference_mpo_matches_exact_finite_differences(ctx):
    """The same check through the reference scheme's MPO generator (complementary
    operators), for h_pq and for (pq|rs) classes: every entry of an 8-fold class
    stepped together, the adjoint read at the class's canonical key."""
    from oracle import ed
    from mpsxx_gb300 import mpogen, mpogen_comp

    n = 6
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 4)
    sites, jacs = mpogen_comp.qc_mpo_complementary(h1, eri, jacobian=True)
    st, log = converge(ctx, sites, n, 64, 1e-12, 5)
    e_ed = ed.qc_ground_energy(h1, eri, n // 2, n // 2)[0]
    assert abs(log.energy - e_ed) < 1e-9
    _, dE = params_gradient(ctx, st, jacs, checkpoint=2)
    step = 1e-4

    def energy(h, v):
        return ed.qc_ground_energy(h, v, n // 2, n // 2)[0]

    worst = 0.0
    for p, q in [(0, 0), (2, 2), (1, 0), (3, 1), (5, 2), (5, 4)]:
        hp, hm = h1.copy(), h1.copy()
        for hh, sgn in ((hp, 1.0), (hm, -1.0)):
            hh[p, q] += sgn * step
            if p != q:
                hh[q, p] += sgn * step
        fd = (energy(hp, eri) - energy(hm, eri)) / (2 * step)
        adj = dE.get(("h", p, q), 0.0)
        worst = max(worst, abs(adj - fd) / max(1.0, abs(fd)))
    for p, q, r, s in [(2, 2, 2, 2), (3, 1, 2, 0), (4, 4, 1, 1), (5, 2, 5, 2), (3, 3, 3, 0)]:
        vp, vm = eri.copy(), eri.copy()
        for vv, sgn in ((vp, 1.0), (vm, -1.0)):
            for a, b, c, d in {(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                               (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)}:
                vv[a, b, c, d] += sgn * step
        fd = (energy(h1, vp) - energy(h1, vm)) / (2 * step)
        adj = dE.get(("eri", p, q, r, s), 0.0)
        worst = max(worst, abs(adj - fd) / max(1.0, abs(fd)))
    print("qc n=6, reference MPO: dE/dh and dE/d(pq|rs) adjoint vs exact FD, worst relative error", worst)
    assert worst < 1e-6


def test_autograd_harness_backward_is_the_adjoint(ctx):
    """torch.autograd through the C ABI: backward gives the adjoint gradient, and a
    central difference of the harness's own energies (warm restarts) agrees."""
    import torch

    from mpsxx_gb300.autograd import HubbardChain

    L = 6
    rng = np.random.default_rng(7)
    theta0 = np.concatenate([-rng.uniform(0.8, 1.2, L - 1), rng.uniform(2.0, 6.0, L)])
    model = HubbardChain(ctx, L, L, 64, tole=1e-12, max_sweeps=8, warm_sweeps=6, checkpoint=2)
    theta = torch.tensor(theta0, dtype=torch.float64, requires_grad=True)
    e = model(theta)
    (g,) = torch.autograd.grad(e, theta)
    h = 1e-4
    for k in (0, L - 1, 2 * L - 2):
        tp, tm = theta0.copy(), theta0.copy()
        tp[k] += h
        tm[k] -= h
        ep = model(torch.tensor(tp)).item()
        em = model(torch.tensor(tm)).item()
        fd = (ep - em) / (2 * h)
        assert abs(g[k].item() - fd) < 1e-6 * max(1.0, abs(fd)), (k, g[k].item(), fd)
