"""CUDA path vs the oracle on the same inputs, through the C ABI (needs a GPU).

Tolerances: FP64 kernels reorder sums relative to the oracle's BLAS, so block
data is compared at 1e-12 relative to the largest magnitude, energies at 1e-10 Eh.
"""
import json
import os

import numpy as np
import pytest

from tests.bondcase import hubbard_bond, to_dict

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    return core.Context(0)


def dev(ctx, a):
    from mpsxx_gb300 import core

    return core.Tensor.from_dict(ctx, to_dict(a))


def max_block_diff(ref_blocks, got_blocks):
    keys = set(ref_blocks) | set(got_blocks)
    scale = max([float(np.max(np.abs(b))) for b in ref_blocks.values() if b.size] + [1e-300])
    err = 0.0
    for k in keys:
        r = ref_blocks.get(k)
        g = got_blocks.get(k)
        if r is None:
            r = np.zeros_like(g)
        if g is None:
            g = np.zeros_like(r)
        err = max(err, float(np.max(np.abs(r - g))) if r.size else 0.0)
    return err / scale


def test_sigma_vector_matches_oracle(ctx):
    from oracle import dmrg as od
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    L, R, P = dev(ctx, case["mL"]), dev(ctx, case["mR"]), dev(ctx, case["full"])
    S = P.like()
    core.compute_sigma_vector(ctx, L, R, P, S)
    ref = oq.QSDArray()
    od.compute_sigma_vector(case["mL"], case["mR"], case["full"], ref)
    assert max_block_diff(ref.blocks, S.to_blocks()) < 1e-12
    # accumulate semantics (beta = 1): a second call doubles sigma
    core.compute_sigma_vector(ctx, L, R, P, S)
    assert max_block_diff({k: 2 * v for k, v in ref.blocks.items()}, S.to_blocks()) < 1e-12


def test_diagonal_matches_oracle(ctx):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    L, R, P = dev(ctx, case["mL"]), dev(ctx, case["mR"]), dev(ctx, case["full"])
    D = P.like()
    core.compute_diagonal_elements(ctx, L, R, D)
    ref = case["full"].empty_like()
    od.compute_diagonal_elements(case["mL"], case["mR"], ref)
    assert max_block_diff(ref.blocks, D.to_blocks()) < 1e-12


@pytest.mark.parametrize("forward", [True, False])
def test_merged_operator_matches_oracle(ctx, forward):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    st, i = case["st"], case["i"]
    if forward:
        mpo, opr = case["mpo"][i], st.lenv[i]
    else:
        mpo, opr = case["mpo"][i + 1], st.renv[i + 1]
    got = core.compute_merged_operator(ctx, forward, dev(ctx, mpo), dev(ctx, opr))
    ref = od.compute_merged_operator(forward, mpo, opr)
    q, d = got.shape()
    assert q == [list(x) for x in ref.qshape] and d == ref.dshape
    tags, _ = got.blocks()
    assert list(tags) == sorted(ref.blocks)
    assert max_block_diff(ref.blocks, got.to_blocks()) < 1e-13


# canonicalize routes: (Jacobi column limit, batched-eigensolver Gram limit); -1 = default
ROUTES = {"default": (-1, -1), "jacobi": (128, 0), "eigensolver": (0, 100000), "lanes": (0, 0)}


@pytest.mark.parametrize("route", sorted(ROUTES))
@pytest.mark.parametrize("forward", [True, False])
def test_canonicalize_and_renormalize_match_oracle(ctx, forward, route):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    M = case["M"]
    P = dev(ctx, case["psi"])
    ctx.set_svd_routes(*ROUTES[route])
    try:
        lm, rm = core.canonicalize(ctx, forward, P, M)
    finally:
        ctx.set_svd_routes()
    U, V, kept = od.canonicalize_merged(forward, case["psi"], M)
    # same new bond (sectors and kept dims)
    assert lm.shape()[0][1] == U.qshape[1] and lm.shape()[1][1] == U.dshape[1]
    # the product U (s) V^T is sign-free
    def prod(a, b):
        from oracle import qsd as oq
        c = oq.QSDArray()
        oq.gemm("N", "N", 1.0, a, b, 1.0, c, nc=2)
        return c.blocks
    from oracle import qsd as oq
    gl = oq.QSDArray(lm.q, *lm.shape())
    gl.blocks = lm.to_blocks()
    gr = oq.QSDArray(rm.q, *rm.shape())
    gr.blocks = rm.to_blocks()
    assert max_block_diff(prod(U, V), prod(gl, gr)) < 1e-12
    # renormalised operator from the same (oracle) singular vectors: the kernel
    # parity does not depend on the SVD's sign gauge
    if forward:
        Ud = dev(ctx, U)
        env = core.renormalize(ctx, True, dev(ctx, case["mL"]), Ud, Ud)
        ref = od.renormalize_merged(True, case["mL"], U, U)
    else:
        Vd = dev(ctx, V)
        env = core.renormalize(ctx, False, dev(ctx, case["mR"]), Vd, Vd)
        ref = od.renormalize_merged(False, case["mR"], V, V)
    tags, _ = env.blocks()
    assert list(tags) == sorted(ref.blocks)
    assert max_block_diff(ref.blocks, env.to_blocks()) < 1e-12


def test_davidson_matches_oracle(ctx):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    L, R = dev(ctx, case["mL"]), dev(ctx, case["mR"])
    P = dev(ctx, case["full"])
    D = P.like()
    core.compute_diagonal_elements(ctx, L, R, D)
    e_gpu, st = core.diagonalize(ctx, L, R, D, P, 1e-11)
    diag = case["full"].empty_like()
    od.compute_diagonal_elements(case["mL"], case["mR"], diag)
    psi = case["full"].copy()
    ost = od.DavidsonStats()
    e_ref = od.davidson(lambda c, v: od.compute_sigma_vector(case["mL"], case["mR"], c, v), diag, psi, 1e-11, ost)
    assert abs(e_gpu - e_ref) < 1e-10
    assert st["converged"] == 1


def test_dmrg_hubbard12_energies_match_oracle(ctx):
    """Hubbard L=12, U=4, half filling, M=64, tole 1e-10: every sweep energy within 1e-10 Eh."""
    from mpsxx_gb300 import dmrg
    from mpsxx_gb300.mpogen import hubbard_mpo

    gold = json.load(open(os.path.join(HERE, "golden", "hubbard12_u4_m64.json")))
    mpo = [__import__("mpsxx_gb300.core", fromlist=["Tensor"]).Tensor.from_dict(ctx, d)
           for d in hubbard_mpo(12, -1.0, 4.0)]
    st = dmrg.make_initial_state(ctx, mpo, 12, 0, 64)
    diffs = []
    for k, ref in enumerate(gold["sweeps"]):
        log = dmrg.make_sweep(ctx, st, gold["tole"])
        diffs.append(abs(log.energy - ref["energy"]))
    print("per-sweep |E_gpu - E_oracle|:", diffs)
    # the first sweeps start far from the ground state, where different FP64
    # summation orders move the Davidson stopping points: 1e-8 there, 1e-10 once converged
    assert all(d < 1e-8 for d in diffs[:2]), diffs
    assert all(d < 1e-10 for d in diffs[2:]), diffs
    assert log.energy >= gold["exact"] - 1e-10


@pytest.mark.parametrize("route", sorted(ROUTES))
@pytest.mark.parametrize("forward", [True, False])
def test_canonicalize_rank_deficient_blocks_stay_orthonormal(ctx, forward, route):
    """Blocks of rank 2 (and all-zero blocks), on every route: the singular vectors of
    the numerically zero singular values that the truncation keeps are completed to an
    orthonormal set, as LAPACK's gesvd does (the eigensolver route drops them), so the
    isometric factor is orthonormal block by block and U s V^T reproduces the
    wavefunction.  Tolerance 1e-12."""
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    rng = np.random.default_rng(7)
    psi = case["psi"].empty_like()
    for n, (t, b) in enumerate(sorted(case["psi"].blocks.items())):
        m, k = b.shape
        blk = 1.0e3 * (rng.standard_normal((m, 2)) @ rng.standard_normal((2, k)))
        psi.blocks[t] = np.zeros_like(b) if n % 5 == 4 else blk
    ctx.set_svd_routes(*ROUTES[route])
    try:
        lm, rm = core.canonicalize(ctx, forward, dev(ctx, psi), 0)
    finally:
        ctx.set_svd_routes()
    iso = lm if forward else rm
    checked = 0
    for blk in iso.to_blocks().values():
        g = blk.T @ blk if forward else blk @ blk.T
        assert np.max(np.abs(g - np.eye(g.shape[0]))) < 1e-12
        checked += g.shape[0] > 1
    assert checked > 0
    gl = oq.QSDArray(lm.q, *lm.shape())
    gl.blocks = lm.to_blocks()
    gr = oq.QSDArray(rm.q, *rm.shape())
    gr.blocks = rm.to_blocks()
    c = oq.QSDArray()
    oq.gemm("N", "N", 1.0, gl, gr, 1.0, c, nc=2)
    assert max_block_diff(psi.blocks, c.blocks) < 1e-12


# ---------------------------------------------------------------------------
# make_noise (src/canonicalize.hpp:11-24) and the truncations that use it.  The
# noise itself is bit-exact (same sequence, product and sum rounded separately);
# the noised SVDs are compared through their sign-free products.
# ---------------------------------------------------------------------------

NOISE = 1e-3


def oracle_of(t):
    from oracle import qsd as oq

    a = oq.QSDArray(t.q, *t.shape())
    a.blocks = t.to_blocks()
    return a


def product(a, b, nc):
    from oracle import qsd as oq

    c = oq.QSDArray()
    oq.gemm("N", "N", 1.0, a, b, 1.0, c, nc=nc)
    return c.blocks


def two_site(case):
    from oracle import qsd as oq

    st, i = case["st"], case["i"]
    t = oq.QSDArray()
    oq.gemm("N", "N", 1.0, st.wave[i], st.wave[i + 1], 1.0, t, nc=4)
    return t


def test_make_noise_bit_exact(ctx):
    from oracle import dmrg as od
    from tests.bondcase import repeated_sector_psi
    from mpsxx_gb300 import core

    case = hubbard_bond()
    # merged two-site wavefunction, a wavefunction whose noise array adds blocks, and
    # a four-index two-site tensor (the one-site stage's noise path)
    for a in (case["psi"], repeated_sector_psi(), two_site(case)):
        d = dev(ctx, a)
        core.make_noise(ctx, d, 1e-9)  # below the threshold: nothing happens
        assert max_block_diff(a.blocks, d.to_blocks()) == 0.0
        core.make_noise(ctx, d, NOISE)
        ref = a.copy()
        od.make_noise(ref, NOISE)
        got = d.to_blocks()
        assert sorted(got) == sorted(ref.blocks)
        for t, b in ref.blocks.items():
            assert np.array_equal(got[t], b), t


@pytest.mark.parametrize("forward", [True, False])
def test_canonicalize_with_noise_matches_oracle(ctx, forward):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    M = case["M"]
    P = dev(ctx, case["psi"])
    lm, rm = core.canonicalize(ctx, forward, P, M, NOISE)
    assert max_block_diff(case["psi"].blocks, P.to_blocks()) == 0.0  # wfnc is left as it was
    U, V, kept = od.canonicalize_merged(forward, case["psi"].copy(), M, NOISE)
    U0, V0, kept0 = od.canonicalize_merged(forward, case["psi"].copy(), M, 0.0)
    assert kept != kept0  # the noise reaches the truncation
    assert lm.shape()[0][1] == U.qshape[1] and lm.shape()[1][1] == U.dshape[1]
    assert max_block_diff(product(U, V, 2), product(oracle_of(lm), oracle_of(rm), 2)) < 1e-12


@pytest.mark.parametrize("forward", [True, False])
def test_onesite_noise_split_matches_oracle(ctx, forward):
    from oracle import dmrg as od
    from mpsxx_gb300 import dmrg as gd

    case = hubbard_bond()
    st, i, M = case["st"], case["i"], case["M"]
    wf = st.wave[i]
    nb = st.wave[i + 1] if forward else st.wave[i - 1]
    left, right, f = gd.split_onesite_noise(ctx, forward, dev(ctx, wf), dev(ctx, nb), M, NOISE)
    lo, ro = od.canonicalize_onesite_noise(forward, wf.copy(), nb.copy(), M, NOISE)
    gl, gr = oracle_of(left), oracle_of(right)
    assert gl.qshape == lo.qshape and gl.dshape == lo.dshape
    assert gr.qshape == ro.qshape and gr.dshape == ro.dshape
    assert max_block_diff(product(lo, ro, 4), product(gl, gr, 4)) < 1e-12


def test_bond_step_with_noise(ctx):
    from oracle import dmrg as od
    from mpsxx_gb300 import core

    case = hubbard_bond()
    st, i, M, mpo = case["st"], case["i"], case["M"], case["mpo"]
    args = [dev(ctx, x) for x in (mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1], st.wave[i], st.wave[i + 1])]
    e0, _, nl0, _, _ = core.optimize_twosite_merged(ctx, True, *args, 1e-11, M, 0.0)
    e1, _, nl1, nr1, _ = core.optimize_twosite_merged(ctx, True, *args, 1e-11, M, NOISE)
    res, _, _, _ = od.optimize_twosite_merged(True, mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1], st.wave[i],
                                              st.wave[i + 1], 1e-11, M, NOISE)
    # the noise follows the eigensolver: energies unchanged
    assert abs(e1 - e0) < 1e-12 and abs(e1 - res.energy) < 1e-10
    assert nl1.shape()[1][2] != nl0.shape()[1][2]  # a different truncation
    # the new left site is still left-normalised over (l, n)
    u = oracle_of(nl1)
    gram = {}
    for t, b in u.blocks.items():
        a = u.index(t)[2]
        m = b.reshape(-1, b.shape[2])
        gram[a] = gram.get(a, 0.0) + m.T @ m
    for a, g in gram.items():
        assert np.abs(g - np.eye(g.shape[0])).max() < 1e-12, a


# ---------------------------------------------------------------------------
# The other compute_sigma_vector overloads (src/compute_sigma_vector.hpp:9-35,
# 53-83, 98-109) against the oracle's literal restatement of the reference's
# Gemm/Contract sequences, allocated and accumulated.
# ---------------------------------------------------------------------------

def overlap_operators(w, seed=1):
    from oracle import qsd as oq

    rng = np.random.default_rng(seed)

    def S(qs, ds):
        a = oq.QSDArray((0, 0), [qs, [oq.qneg(q) for q in qs]], [ds, ds])
        for x in range(len(qs)):
            for y in range(len(qs)):
                if a.allowed((x, y)) and ds[x] and ds[y]:
                    a.blocks[a.tag((x, y))] = rng.standard_normal((ds[x], ds[y]))
        return a

    return S(w.qshape[0], w.dshape[0]), S(w.qshape[-1], w.dshape[-1])


@pytest.mark.parametrize("kind", ["onesite", "twosite", "overlap2", "overlap3", "overlap4"])
def test_sigma_overloads_match_oracle(ctx, kind):
    from oracle import dmrg as od
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    if kind == "onesite":
        w = st.wave[i]
        ref = od.compute_sigma_vector_onesite(mpo[i], st.lenv[i], st.renv[i], w, oq.QSDArray())
        ops = [dev(ctx, x) for x in (mpo[i], st.lenv[i], st.renv[i])]
        fn = core.compute_sigma_vector_onesite
    elif kind == "twosite":
        w = two_site(case)
        ref = od.compute_sigma_vector_twosite(mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1], w, oq.QSDArray())
        ops = [dev(ctx, x) for x in (mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1])]
        fn = core.compute_sigma_vector_twosite
    else:
        w = {"overlap2": case["psi"], "overlap3": st.wave[i], "overlap4": two_site(case)}[kind]
        lS, rS = overlap_operators(w)
        ref = od.compute_sigma_vector_overlap(lS, rS, w, oq.QSDArray())
        ops = [dev(ctx, lS), dev(ctx, rS)]
        fn = core.compute_sigma_vector_overlap
    W = dev(ctx, w)
    got = fn(ctx, *ops, W)
    assert max_block_diff(ref.blocks, got.to_blocks()) < 1e-12
    # accumulate into an existing tensor (wfn itself): missing blocks are added
    acc = dev(ctx, w)
    fn(ctx, *ops, W, acc)
    expect = w.copy()
    oq.axpy(1.0, ref, expect)
    assert max_block_diff(expect.blocks, acc.to_blocks()) < 1e-12


@pytest.mark.parametrize("forward", [True, False])
def test_renormalize_overloads_match_oracle(ctx, forward):
    from oracle import dmrg as od
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    if forward:
        k, opr, w = i, st.lenv[i], st.wave[i]
    else:
        k, opr, w = i + 1, st.renv[i + 1], st.wave[i + 1]
    # a ket distinct from the bra (the bra perturbed), so that a swap or a missing
    # conjugation of either would show
    rng0 = np.random.default_rng(17)
    ket = w.copy()
    for t in ket.blocks:
        ket.blocks[t] = ket.blocks[t] + 0.3 * rng0.standard_normal(ket.blocks[t].shape)
    ref = od.renormalize_mpo(forward, mpo[k], opr, w, ket)
    W, K = dev(ctx, w), dev(ctx, ket)
    got = core.renormalize_mpo(ctx, forward, dev(ctx, mpo[k]), dev(ctx, opr), W, K)
    assert max_block_diff(ref.blocks, got.to_blocks()) < 1e-12
    again = core.renormalize_mpo(ctx, forward, dev(ctx, mpo[k]), dev(ctx, opr), W, K, got)  # accumulates
    assert again is got
    assert max_block_diff({t: 2 * b for t, b in ref.blocks.items()}, got.to_blocks()) < 1e-12
    # overlap matrix, with a random S on the contracted sectors
    rng = np.random.default_rng(5)
    qs, ds = (w.qshape[0], w.dshape[0]) if forward else (w.qshape[2], w.dshape[2])
    S = oq.QSDArray((0, 0), [qs, [oq.qneg(q) for q in qs]], [ds, ds])
    for x in range(len(qs)):
        for y in range(len(qs)):
            if S.allowed((x, y)) and ds[x] and ds[y]:
                S.blocks[S.tag((x, y))] = rng.standard_normal((ds[x], ds[y]))
    ref = od.renormalize_overlap(forward, S, w, ket)
    got = core.renormalize_overlap(ctx, forward, dev(ctx, S), W, K)
    assert max_block_diff(ref.blocks, got.to_blocks()) < 1e-12


@pytest.mark.parametrize("kind", ["onesite", "twosite"])
def test_diagonal_overloads_match_oracle(ctx, kind):
    from oracle import dmrg as od
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    w = st.wave[i] if kind == "onesite" else two_site(case)
    ref = oq.QSDArray(w.q, w.qshape, w.dshape)
    D = dev(ctx, w)  # starts from w's data, which the reference's Copy(scr, diag, 1) drops
    if kind == "onesite":
        od.compute_diagonal_elements_onesite(mpo[i], st.lenv[i], st.renv[i], ref)
        core.compute_diagonal_elements_onesite(ctx, *[dev(ctx, x) for x in (mpo[i], st.lenv[i], st.renv[i])], D)
    else:
        od.compute_diagonal_elements_twosite(mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1], ref)
        core.compute_diagonal_elements_twosite(
            ctx, *[dev(ctx, x) for x in (mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1])], D)
    got = D.to_blocks()
    # w's previous values are gone: every block is the reference's, and blocks that no
    # term reaches (absent from the reference's result) are stored as zeros
    assert set(ref.blocks) <= set(got)
    assert all(not np.any(got[t]) for t in set(got) - set(ref.blocks))
    assert max_block_diff(ref.blocks, got) < 1e-12

