"""The oracle against exact answers and the reference's own golden vectors (CPU)."""
import hashlib
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def golden(name):
    return json.load(open(os.path.join(HERE, "golden", name)))


def oracle_dmrg(mpo_dicts, n_elec, two_sz, M, tole, sweeps):
    from oracle import dmrg as od
    from oracle import from_site_dict

    st, logs = od.dmrg([from_site_dict(s) for s in mpo_dicts], n_elec, two_sz, M, tole, sweeps)
    return logs[-1].energy


def test_hubbard_chain_matches_exact_diagonalisation():
    from oracle.ed import hubbard_ground_energy
    from mpsxx_gb300.mpogen import hubbard_mpo

    e = oracle_dmrg(hubbard_mpo(6, -1.0, 4.0), 6, 0, 64, 1e-10, 8)
    assert abs(e - hubbard_ground_energy(6, -1.0, 4.0, 3, 3)[0]) < 1e-10


def test_site_dependent_hubbard_matches_exact_diagonalisation():
    from oracle.ed import hubbard_ground_energy
    from mpsxx_gb300.mpogen import hubbard_mpo

    rng = np.random.default_rng(3)
    t = rng.uniform(0.8, 1.2, 5)
    U = rng.uniform(2.0, 6.0, 6)
    e = oracle_dmrg(hubbard_mpo(6, t, U), 6, 0, 64, 1e-10, 8)
    assert abs(e - hubbard_ground_energy(6, t, U, 3, 3)[0]) < 1e-10


@pytest.mark.parametrize("n,nel,two_sz", [(4, 4, 0), (5, 4, 2), (6, 6, 0)])
def test_qc_hamiltonian_matches_exact_diagonalisation(n, nel, two_sz):
    from oracle.ed import qc_ground_energy
    from mpsxx_gb300 import mpogen

    h, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 11 + n)
    e = oracle_dmrg(mpogen.qc_mpo(h, eri, 0.37), nel, two_sz, 256, 1e-10, 10)
    ref = qc_ground_energy(h, eri, (nel + two_sz) // 2, (nel - two_sz) // 2, ecore=0.37)[0]
    assert abs(e - ref) < 1e-9


def test_generic_mpo_builder_finds_the_hubbard_bond_dimension():
    from mpsxx_gb300 import mpogen

    n = 7
    h = np.zeros((n, n))
    for i in range(n - 1):
        h[i, i + 1] = h[i + 1, i] = -1.0
    eri = np.zeros((n, n, n, n))
    for i in range(n):
        eri[i, i, i, i] = 4.0
    assert mpogen.mpo_bond_dims(mpogen.qc_mpo(h, eri))[:-1] == [6] * (n - 1)


def test_hubbard12_reference_golden_energy():
    """dmrg/tests/HUBBARD12 (U=1, h_{i+1,i}=+1, 12 electrons), M=200: the reference's
    log holds -11.8406372775523305 (hub12_dmrg.out:15536); the oracle lands within
    1e-8 of it and both lie above the exact ground state."""
    from mpsxx_gb300.mpogen import hubbard_mpo

    g = golden("reference_energies.json")
    ref = float(g["HUBBARD12_M200_roots"]["energies"][0])
    exact = g["HUBBARD12_exact"]["energy"]
    e = oracle_dmrg(hubbard_mpo(12, 1.0, 1.0), 12, 0, 200, 1e-8, 10)
    assert abs(e - ref) < 1e-8
    assert e >= exact - 1e-12 and ref >= exact - 1e-12
    assert abs(e - g["HUBBARD12_M200_oracle"]["energy"]) < 1e-10


def test_reference_random_integral_generator_is_reproduced():
    """dmrg/tests/intgen.cpp restated: its 16-orbital FCIDUMP is reproduced bit-exactly
    (sha256 of the integral lines recorded from the reference's file)."""
    from tests.golden.intgen import intgen

    g = golden("reference_energies.json")["INTGEN16_FCIDUMP"]
    _, _, lines = intgen(16)
    txt = "".join(f"{v:24.16e}{i:4d}{j:4d}{k:4d}{l:4d}\n" for v, i, j, k, l in lines)
    assert hashlib.sha256(txt.encode()).hexdigest() == g["sha256"]
    assert len(lines) == g["lines"]


def test_hubbard12_u4_m64_fixture_first_sweeps():
    """Regression: the first two sweeps of the committed L=12, U=4, M=64 fixture."""
    from oracle import dmrg as od
    from oracle import from_site_dict
    from mpsxx_gb300.mpogen import hubbard_mpo

    g = golden("hubbard12_u4_m64.json")
    st = od.make_initial_state([from_site_dict(s) for s in hubbard_mpo(12, -1.0, 4.0)], 12, 0, 64)
    for k in range(2):
        log = od.make_sweep(st, g["tole"])
        assert abs(log.energy - g["sweeps"][k]["energy"]) < 1e-12


def test_fcidump_round_trip_and_energy(tmp_path):
    """FCIDUMP writer/reader (src/parsing_integral.cpp:105-154 conventions): the unique
    8-fold entries written and unfolded back reproduce the integrals exactly, and the
    MPO built from the file has the same ED-checked DMRG energy as from the arrays."""
    import numpy as np

    from mpsxx_gb300 import mpogen
    from oracle import ed

    n = 5
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 7)
    path = tmp_path / "FCIDUMP"
    mpogen.write_fcidump(str(path), h1, eri, nelec=4, ms2=0, ecore=0.75)
    d = mpogen.read_fcidump(str(path))
    assert (d["norb"], d["nelec"], d["ms2"], d["ecore"]) == (n, 4, 0, 0.75)
    assert np.array_equal(d["h1"], h1)
    assert np.array_equal(d["eri"], eri)
    e = ed.qc_ground_energy(d["h1"], d["eri"], 2, 2, ecore=d["ecore"])[0]
    assert abs(e - (ed.qc_ground_energy(h1, eri, 2, 2)[0] + 0.75)) < 1e-12


def _merged_sigma(mL, mR, psi):
    from oracle import dmrg as od

    full = psi.empty_like()
    full.allocate(0.0)
    for k, b in psi.blocks.items():
        full.blocks[k] = b
    sg = full.empty_like()
    od.compute_sigma_vector(mL, mR, full, sg)
    return sg


def _max_diff(a, b):
    keys = set(a.blocks) | set(b.blocks)
    return max(float(np.abs(a.blocks.get(k, 0.0) - b.blocks.get(k, 0.0)).max()) for k in keys)


def test_rank_overloads_equal_the_merged_product():
    """The one-site and four-index two-site compute_sigma_vector overloads, restated
    literally (the reference's Gemm/Contract sequences), equal the merged product on
    every allowed merged block expanded back: the route the library takes for them."""
    from oracle import dmrg as od
    from oracle import qsd as oq
    from tests.bondcase import hubbard_bond

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    w = st.wave[i]
    lit = od.compute_sigma_vector_onesite(mpo[i], st.lenv[i], st.renv[i], w, oq.QSDArray())
    rows = oq.MergeInfo(w.qshape[:2], w.dshape[:2])
    mL = od.compute_merged_operator(True, mpo[i], st.lenv[i])
    merged = oq.expand_rows(rows, _merged_sigma(mL, st.renv[i], oq.merge_rows(rows, w)))
    assert _max_diff(lit, merged) < 1e-13
    t = oq.QSDArray()
    oq.gemm("N", "N", 1.0, st.wave[i], st.wave[i + 1], 1.0, t, nc=4)
    lit = od.compute_sigma_vector_twosite(mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1], t, oq.QSDArray())
    rows = oq.MergeInfo(t.qshape[:2], t.dshape[:2])
    cols = oq.MergeInfo(t.qshape[2:], t.dshape[2:])
    mR = od.compute_merged_operator(False, mpo[i + 1], st.renv[i + 1])
    sg = _merged_sigma(mL, mR, oq.merge_rows(rows, oq.merge_cols(t, cols)))
    assert _max_diff(lit, oq.expand_cols(oq.expand_rows(rows, sg), cols)) < 1e-13


def test_renormalize_and_diagonal_overloads_equal_the_merged_forms():
    """renormalize with the site MPO (forward and backward) and the one-site / four-index
    diagonals, restated literally, equal the merged forms the library runs them as."""
    from oracle import dmrg as od
    from oracle import qsd as oq
    from tests.bondcase import hubbard_bond

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    w, w2 = st.wave[i], st.wave[i + 1]
    mL = od.compute_merged_operator(True, mpo[i], st.lenv[i])
    mR = od.compute_merged_operator(False, mpo[i + 1], st.renv[i + 1])
    rows = oq.MergeInfo(w.qshape[:2], w.dshape[:2])
    U = oq.merge_rows(rows, w)
    assert _max_diff(od.renormalize_mpo(True, mpo[i], st.lenv[i], w, w), od.renormalize_merged(True, mL, U, U)) < 1e-13
    cols = oq.MergeInfo(w2.qshape[1:], w2.dshape[1:])
    V = oq.merge_cols(w2, cols)
    assert _max_diff(od.renormalize_mpo(False, mpo[i + 1], st.renv[i + 1], w2, w2),
                     od.renormalize_merged(False, mR, V, V)) < 1e-13
    d = oq.QSDArray(w.q, w.qshape, w.dshape)
    od.compute_diagonal_elements_onesite(mpo[i], st.lenv[i], st.renv[i], d)
    dm = U.empty_like()
    dm.allocate(0.0)
    od.compute_diagonal_elements(mL, st.renv[i], dm)
    assert _max_diff(d, oq.expand_rows(rows, dm)) < 1e-13


def _dense(a):
    offs = [np.concatenate([[0], np.cumsum(d)]).astype(int) for d in a.dshape]
    out = np.zeros([int(o[-1]) for o in offs])
    for t, b in a.blocks.items():
        idx = a.index(t)
        out[tuple(slice(offs[k][i], offs[k][i + 1]) for k, i in enumerate(idx))] = b
    return out


def test_guesswave_restatement():
    """compute_guesswave (src/compute_guesswave.hpp:11-38) restated: forward (L^T C) R and
    backward L (C R^T) on dense copies of random tensors, and the gauge move of a
    canonical state: an isometry against itself gives back the other site unchanged."""
    from oracle import dmrg as od
    from oracle import qsd as oq

    from tests.bondcase import guesswave_case

    L, C, R, rand_like = guesswave_case()
    Lr, Lc, Cr = rand_like(L), rand_like(L), rand_like(C)
    f = od.compute_guesswave(True, Lr, Lc, Cr, oq.QSDArray())
    ref = np.einsum("lnp,lnr,rmq->pmq", _dense(Lr), _dense(Lc), _dense(Cr))
    assert np.abs(_dense(f) - ref).max() < 1e-12 * np.abs(ref).max()
    Rr, Rc = rand_like(R), rand_like(R)
    b = od.compute_guesswave(False, Rr, Rc, Cr, oq.QSDArray())
    ref = np.einsum("asx,xy->asy", _dense(Cr), np.einsum("xnr,ynr->xy", _dense(Rc), _dense(Rr)))
    assert np.abs(_dense(b) - ref).max() < 1e-12 * np.abs(ref).max()
    assert _max_diff(od.compute_guesswave(True, L, L, C, oq.QSDArray()), C) < 1e-12
    assert _max_diff(od.compute_guesswave(False, R, R, C, oq.QSDArray()), C) < 1e-12
    acc = C.copy()  # accumulates into a non-empty wfn1
    od.compute_guesswave(True, L, L, C, acc)
    assert _max_diff(acc, _twice(C)) < 1e-12


def _twice(a):
    t = a.copy()
    for k in t.blocks:
        t.blocks[k] = 2.0 * t.blocks[k]
    return t


def _perturbed(a, seed):
    """a plus 0.3 x seeded normal values on every block a holds (same layout)."""
    rng = np.random.default_rng(seed)
    b = a.copy()
    for k in b.blocks:
        b.blocks[k] = b.blocks[k] + 0.3 * rng.standard_normal(b.blocks[k].shape)
    return b


def test_renormalize_with_distinct_bra_and_ket_equals_dense_products():
    """renormalize with the site MPO and of an overlap matrix, bra != ket: forward
    opr1[a,v,b] = sum bra[l,n,a] opr0[l,w,k] W[w,n,m,v] ket[k,m,b] and backward
    opr1[a,w,b] = sum bra[a,n,r] opr0[r,v,s] W[w,n,m,v] ket[b,m,s] (src/renormalize.hpp:
    10-54) on dense copies; a swap of bra and ket changes the result."""
    from oracle import dmrg as od
    from oracle import qsd as oq
    from tests.bondcase import hubbard_bond

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    for forward, k, opr, w in ((True, i, st.lenv[i], st.wave[i]), (False, i + 1, st.renv[i + 1], st.wave[i + 1])):
        bra, ket = w, _perturbed(w, 11 + k)
        got = _dense(od.renormalize_mpo(forward, mpo[k], opr, bra, ket))
        W, O, B, K = _dense(mpo[k]), _dense(opr), _dense(bra), _dense(ket)
        if forward:
            ref = np.einsum("lna,lwk,wnmv,kmb->avb", B, O, W, K)
        else:
            ref = np.einsum("anr,rvs,wnmv,bms->awb", B, O, W, K)
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()
        swapped = _dense(od.renormalize_mpo(forward, mpo[k], opr, ket, bra))
        assert np.abs(swapped - ref).max() > 1e-6 * np.abs(ref).max()
        # overlap matrix: forward S1[a,b] = sum S0[l,k] bra[l,n,a] ket[k,n,b]
        rng = np.random.default_rng(3 + k)
        qs, ds = (w.qshape[0], w.dshape[0]) if forward else (w.qshape[2], w.dshape[2])
        S = oq.QSDArray((0, 0), [qs, [oq.qneg(q) for q in qs]], [ds, ds])
        for x in range(len(qs)):
            for y in range(len(qs)):
                if S.allowed((x, y)) and ds[x] and ds[y]:
                    S.blocks[S.tag((x, y))] = rng.standard_normal((ds[x], ds[y]))
        got = _dense(od.renormalize_overlap(forward, S, bra, ket))
        if forward:
            ref = np.einsum("lk,lna,knb->ab", _dense(S), B, K)
        else:
            ref = np.einsum("rs,anr,bns->ab", _dense(S), B, K)
        assert np.abs(got - ref).max() < 1e-12 * np.abs(ref).max()


def test_single_group_diagonal_overwrites_like_copy():
    """The one-site and four-index diagonals end with Copy(scr, diag, 1)
    (src/compute_diagonal_elements.hpp:31,58): blocks diag held before are dropped."""
    from oracle import dmrg as od
    from oracle import qsd as oq
    from tests.bondcase import hubbard_bond

    case = hubbard_bond()
    st, i, mpo = case["st"], case["i"], case["mpo"]
    w = st.wave[i]
    fresh = oq.QSDArray(w.q, w.qshape, w.dshape)
    od.compute_diagonal_elements_onesite(mpo[i], st.lenv[i], st.renv[i], fresh)
    reused = _perturbed(w, 4)
    od.compute_diagonal_elements_onesite(mpo[i], st.lenv[i], st.renv[i], reused)
    assert set(reused.blocks) == set(fresh.blocks)
    assert _max_diff(reused, fresh) == 0.0
