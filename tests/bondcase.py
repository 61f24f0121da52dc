"""Shared fixture builder: a consistent two-site bond taken from an oracle sweep."""
from __future__ import annotations

import functools

from oracle import dmrg as od
from oracle import from_site_dict
from oracle import qsd as oq
from mpsxx_gb300.mpogen import hubbard_mpo


@functools.lru_cache(maxsize=None)
def hubbard_bond(L: int = 10, M: int = 32, bond: int = 4, U: float = 4.0):
    mpo = [from_site_dict(s) for s in hubbard_mpo(L, -1.0, U)]
    st = od.make_initial_state(mpo, L, 0, M)
    od.make_sweep(st, 1e-8)
    for i in range(bond):
        res, env, nl, nr = od.optimize_twosite_merged(True, mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1],
                                                      st.wave[i], st.wave[i + 1], 1e-9, M)
        st.lenv[i + 1] = env
        st.wave[i] = nl
        st.wave[i + 1] = nr
    i = bond
    mL = od.compute_merged_operator(True, mpo[i], st.lenv[i])
    mR = od.compute_merged_operator(False, mpo[i + 1], st.renv[i + 1])
    ql, qr = od.wave_merge_infos(mpo[i], mpo[i + 1], st.lenv[i], st.renv[i + 1])
    t = oq.QSDArray()
    oq.gemm("N", "N", 1.0, st.wave[i], st.wave[i + 1], 1.0, t, nc=4)
    psi = oq.merge_cols(oq.merge_rows(ql, t), qr)
    full = psi.empty_like()
    full.allocate(0.0)
    for k, b in psi.blocks.items():
        full.blocks[k] = b
    return dict(mpo=mpo, st=st, i=i, mL=mL, mR=mR, psi=psi, full=full, M=M)


def repeated_sector_psi() -> oq.QSDArray:
    """A wavefunction whose sectors repeat quantum numbers, so four blocks are allowed
    among rows 0-1 and columns 0-1; two are stored, and they show the dimension of
    each of those sectors (row 2 / column 2 allow one more block but appear in none)."""
    import numpy as np

    qrow = [(0, 0), (0, 0), (1, 1)]
    qcol = [(2, 0), (2, 0), (1, -1)]
    psi = oq.QSDArray((2, 0), [qrow, qcol], [[2, 3, 4], [5, 3, 2]])
    rng = np.random.default_rng(3)
    psi.blocks[psi.tag((0, 0))] = rng.standard_normal((2, 5))
    psi.blocks[psi.tag((1, 1))] = rng.standard_normal((3, 3))
    return psi


def to_dict(a: oq.QSDArray) -> dict:
    return {"q": a.q, "qshape": a.qshape, "dshape": a.dshape, "blocks": a.blocks}


def guesswave_case(seed=3):
    """Site tensors of a Hubbard bond (left-normalised L(i-1), centre C(i), right-normalised
    R(i+1)) and random tensors with the same block layouts."""
    import numpy as np

    case = hubbard_bond()
    st, i = case["st"], case["i"]
    rng = np.random.default_rng(seed)

    def rand_like(a):
        r = a.copy()
        for t in r.blocks:
            r.blocks[t] = rng.standard_normal(r.blocks[t].shape)
        return r

    return st.wave[i - 1], st.wave[i], st.wave[i + 1], rand_like
