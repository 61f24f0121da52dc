"""The restated complementary-operator MPO generator (mpsxx_gb300/mpogen_comp.py)
against the MPOs the reference's own mpogen.x wrote (tests/golden/make_ref_fixtures.py):
every site of the QC n=8 Hamiltonian (K=16, seed 1) and the two sites of the C2
middle bond (n=20, K=40, seed 1) with the bond dimensions and block counts of all
C2 sites — equal sectors, equal block tags and bit-identical values."""
import json
import os

import numpy as np

from oracle import ref_io

REF = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref")


def _same(ref: dict, mine: dict):
    assert [list(map(tuple, x)) for x in ref["qshape"]] == [list(map(tuple, x)) for x in mine["qshape"]]
    assert [list(x) for x in ref["dshape"]] == [list(x) for x in mine["dshape"]]
    assert tuple(ref["q"]) == tuple(mine["q"])
    assert sorted(ref["blocks"]) == sorted(mine["blocks"])
    for t, b in ref["blocks"].items():
        assert float(b.ravel()[0]) == float(mine["blocks"][t].ravel()[0]), t


def test_qc8_mpo_equals_the_reference_bitwise():
    from mpsxx_gb300 import mpogen, mpogen_comp

    h1, eri = mpogen.synthetic_qc_integrals(8, 16, 1)
    mine = mpogen_comp.qc_mpo_complementary(h1, eri)
    z = np.load(os.path.join(REF, "mpo_qc8.npz"))
    assert len(mine) == 8
    for i in range(8):
        _same(ref_io.unpack_tensor(z, f"site{i}"), mine[i])


def test_c2_mpo_equals_the_reference():
    """W = 862 at the middle bond (9,10), the bound 2 + 4n - 2L + 8L^2 of the scheme."""
    from mpsxx_gb300 import mpogen, mpogen_comp

    h1, eri = mpogen.synthetic_qc_integrals(20, 40, 1)
    mine = mpogen_comp.qc_mpo_complementary(h1, eri)
    with open(os.path.join(REF, "runs.json")) as f:
        rec = json.load(f)["c2_mpo"]
    assert [len(s["qshape"][3]) for s in mine[:-1]] == rec["bond_dims"]
    assert [len(s["blocks"]) for s in mine] == rec["nnz"]
    assert mpogen.mpo_bond_dims(mine)[9] == 862 == 2 + 4 * 20 - 2 * 10 + 8 * 10 * 10
    z = np.load(os.path.join(REF, "mpo_c2_bond.npz"))
    for i in (9, 10):
        _same(ref_io.unpack_tensor(z, f"site{i}"), mine[i])


def test_complementary_mpo_matches_exact_diagonalisation():
    """The generated operator is the Hamiltonian: its DMRG energy with exact bond
    dimension equals exact diagonalisation (QC n=5, 4 electrons)."""
    from mpsxx_gb300 import mpogen, mpogen_comp
    from oracle import dmrg as od
    from oracle import ed
    from oracle import from_site_dict

    h1, eri = mpogen.synthetic_qc_integrals(5, 10, 3)
    mpo = [from_site_dict(s) for s in mpogen_comp.qc_mpo_complementary(h1, eri)]
    st = od.make_initial_state(mpo, 4, 0, 64)
    for _ in range(4):
        e = od.make_sweep(st, 1e-12).energy
    assert abs(e - float(np.min(ed.qc_ground_energy(h1, eri, 2, 2)))) < 1e-9


def _sym_eri_bump(eri, p, q, r, s, eps):
    out = eri.copy()
    for a, b, c, d in {(p, q, r, s), (q, p, r, s), (p, q, s, r), (q, p, s, r),
                       (r, s, p, q), (s, r, p, q), (r, s, q, p), (s, r, q, p)}:
        out[a, b, c, d] += eps
    return out


def test_complementary_mpo_jacobian_matches_finite_differences():
    """Every block of the reference scheme's MPO is linear in the integrals it reads,
    so the generator's Jacobian must equal central differences of the generated
    blocks under symmetric perturbations of h_pq and of a (pq|rs) class (n=6)."""
    from mpsxx_gb300 import mpogen, mpogen_comp

    n = 6
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 5)
    sites, jacs = mpogen_comp.qc_mpo_complementary(h1, eri, jacobian=True)
    plain = mpogen_comp.qc_mpo_complementary(h1, eri)
    assert all(a["blocks"].keys() == b["blocks"].keys() for a, b in zip(sites, plain))
    eps = 1e-3
    params = [("h", 0, 0), ("h", 3, 1), ("h", 5, 4), ("eri", 2, 2, 2, 2), ("eri", 3, 1, 2, 0), ("eri", 4, 4, 1, 1),
              ("eri", 5, 2, 5, 2), ("eri", 3, 3, 3, 0), ("eri", 5, 4, 3, 2)]
    worst, seen = 0.0, 0
    for par in params:
        if par[0] == "h":
            _, p, q = par
            hp, hm = h1.copy(), h1.copy()
            for hh, sg in ((hp, 1.0), (hm, -1.0)):
                hh[p, q] += sg * eps
                if p != q:
                    hh[q, p] += sg * eps
            wp = mpogen_comp.qc_mpo_complementary(hp, eri)
            wm = mpogen_comp.qc_mpo_complementary(hm, eri)
        else:
            wp = mpogen_comp.qc_mpo_complementary(h1, _sym_eri_bump(eri, *par[1:], eps))
            wm = mpogen_comp.qc_mpo_complementary(h1, _sym_eri_bump(eri, *par[1:], -eps))
        for i in range(n):
            assert wp[i]["blocks"].keys() == wm[i]["blocks"].keys() == sites[i]["blocks"].keys()
            for tag in sites[i]["blocks"]:
                fd = (wp[i]["blocks"][tag].item() - wm[i]["blocks"][tag].item()) / (2 * eps)
                jv = jacs[i].get(tag, {}).get(par, 0.0)
                worst = max(worst, abs(fd - jv))
                seen += jv != 0.0
    print("complementary MPO jacobian vs central differences: worst", worst, "non-zero entries", seen)
    assert seen > 0
    assert worst < 1e-9
