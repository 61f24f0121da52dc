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
