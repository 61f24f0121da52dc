"""Exact diagonalisation in a fixed (N, 2Sz) sector (test infrastructure only).

Independent of the MPO machinery: the Hamiltonian is built from integrals on
bit strings (alpha modes then beta modes, Jordan-Wigner signs), so it pins the
oracle's energies from outside the reference's algorithm.
"""
from __future__ import annotations

import itertools
from math import comb

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


def _configs(n: int, k: int):
    out = []
    for occ in itertools.combinations(range(n), k):
        b = 0
        for o in occ:
            b |= 1 << o
        out.append(b)
    return np.array(sorted(out), dtype=np.int64)


def _popcount_below(b: int, i: int) -> int:
    return bin(b & ((1 << i) - 1)).count("1")


def _one_body_spin(h: np.ndarray, cfgs: np.ndarray) -> sp.csr_matrix:
    """Matrix of sum_pq h_pq a+_p a_q within one spin species."""
    n = h.shape[0]
    index = {int(c): i for i, c in enumerate(cfgs)}
    rows, cols, vals = [], [], []
    for j, c in enumerate(cfgs):
        c = int(c)
        for q in range(n):
            if not (c >> q) & 1:
                continue
            c1 = c & ~(1 << q)
            s1 = _popcount_below(c, q)
            for p in range(n):
                if h[p, q] == 0.0 or (c1 >> p) & 1:
                    continue
                c2 = c1 | (1 << p)
                s2 = _popcount_below(c1, p)
                rows.append(index[c2])
                cols.append(j)
                vals.append(h[p, q] * (-1) ** (s1 + s2))
    m = len(cfgs)
    return sp.csr_matrix((vals, (rows, cols)), shape=(m, m))


def hubbard_ground_energy(L: int, t, U, n_up: int, n_dn: int, k: int = 1) -> np.ndarray:
    """Lowest eigenvalues of the open-chain Hubbard model (h_{i,i+1} = t_i)."""
    tt = np.broadcast_to(np.asarray(t, dtype=np.float64), (L - 1,))
    uu = np.broadcast_to(np.asarray(U, dtype=np.float64), (L,))
    h = np.zeros((L, L))
    for i in range(L - 1):
        h[i, i + 1] = h[i + 1, i] = tt[i]
    cu = _configs(L, n_up)
    cd = _configs(L, n_dn)
    hu = _one_body_spin(h, cu)
    hd = _one_body_spin(h, cd)
    Iu = sp.identity(len(cu), format="csr")
    Id = sp.identity(len(cd), format="csr")
    H = sp.kron(hu, Id, format="csr") + sp.kron(Iu, hd, format="csr")
    occ_u = ((cu[:, None] >> np.arange(L)[None, :]) & 1).astype(np.float64)
    occ_d = ((cd[:, None] >> np.arange(L)[None, :]) & 1).astype(np.float64)
    diag = (occ_u * uu[None, :]) @ occ_d.T  # [nu, nd]
    H = H + sp.diags(diag.ravel())
    if H.shape[0] <= 2000:
        w = np.linalg.eigvalsh(H.toarray())
        return w[:k]
    w = spla.eigsh(H, k=k, which="SA", tol=1e-13, return_eigenvectors=False)
    return np.sort(w)


def qc_ground_energy(h1: np.ndarray, eri: np.ndarray, n_up: int, n_dn: int, ecore: float = 0.0,
                     k: int = 1) -> np.ndarray:
    """Lowest eigenvalues of H = sum h_pq E_pq + 1/2 sum (pq|rs) a+_p a+_r a_s a_q (spin-free
    integrals, chemists' notation), by dense/sparse matrix in the spin-orbital sector.
    Intended for small n (<= 8)."""
    n = h1.shape[0]
    # spin orbitals: alpha 0..n-1, beta n..2n-1
    nso = 2 * n
    cfgs = []
    for ou in itertools.combinations(range(n), n_up):
        for od in itertools.combinations(range(n), n_dn):
            b = 0
            for o in ou:
                b |= 1 << o
            for o in od:
                b |= 1 << (n + o)
            cfgs.append(b)
    cfgs = sorted(cfgs)
    index = {c: i for i, c in enumerate(cfgs)}
    m = len(cfgs)

    def apply_ann(c, q):
        if not (c >> q) & 1:
            return None, 0
        return c & ~(1 << q), _popcount_below(c, q)

    def apply_cre(c, p):
        if (c >> p) & 1:
            return None, 0
        return c | (1 << p), _popcount_below(c, p)

    H = np.zeros((m, m)) if m <= 6000 else None
    rows, cols, vals = [], [], []
    for j, c in enumerate(cfgs):
        acc = {}
        # one-body
        for sp_ in range(2):
            for q in range(n):
                c1, s1 = apply_ann(c, q + sp_ * n)
                if c1 is None:
                    continue
                for p in range(n):
                    if h1[p, q] == 0.0:
                        continue
                    c2, s2 = apply_cre(c1, p + sp_ * n)
                    if c2 is None:
                        continue
                    acc[c2] = acc.get(c2, 0.0) + h1[p, q] * (-1) ** (s1 + s2)
        # two-body: 1/2 (pq|rs) a+_{p s} a+_{r t} a_{s t} a_{q s}
        for s_ in range(2):
            for t_ in range(2):
                for q in range(n):
                    c1, s1 = apply_ann(c, q + s_ * n)
                    if c1 is None:
                        continue
                    for s in range(n):
                        c2, s2 = apply_ann(c1, s + t_ * n)
                        if c2 is None:
                            continue
                        for r in range(n):
                            c3, s3 = apply_cre(c2, r + t_ * n)
                            if c3 is None:
                                continue
                            for p in range(n):
                                v = eri[p, q, r, s]
                                if v == 0.0:
                                    continue
                                c4, s4 = apply_cre(c3, p + s_ * n)
                                if c4 is None:
                                    continue
                                acc[c4] = acc.get(c4, 0.0) + 0.5 * v * (-1) ** (s1 + s2 + s3 + s4)
        for c4, v in acc.items():
            rows.append(index[c4])
            cols.append(j)
            vals.append(v)
    Hs = sp.csr_matrix((vals, (rows, cols)), shape=(m, m))
    Hs = Hs + ecore * sp.identity(m)
    if m <= 6000:
        return np.linalg.eigvalsh(Hs.toarray())[:k]
    return np.sort(spla.eigsh(Hs, k=k, which="SA", tol=1e-13, return_eigenvectors=False))
