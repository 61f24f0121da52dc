"""Matrix-product-operator generators (host side, NumPy).

The MPO is an input of the two-site hot path, built once on the host.  Each
site operator ``W[w, s, s', w']`` follows the reference's conventions:

* physical basis ``vac(0,0), alpha(1,+1), beta(1,-1), pair(2,0)`` with
  ``|pair> = b^+ a^+ |0>`` (``src/mpsite.h:26-32``, ``src/prime_operators.cpp:20-131``);
* quantum shapes ``(q_left, q_site, -q_site, q_right)`` with total zero, where
  ``q_left[w]`` is the charge of left-block operator ``w`` and
  ``q_right[w'] = -charge`` of the next left-block operator;
* every block is 1x1x1x1 and a block gets a factor -1 when the left operator and
  the bra site state are both fermion-odd (``src/prime_operators.h:167-187``);
  with that rule, ``W`` maps left operator ``O_w`` to ``O_w * o_site``.

Every generator returns a list of plain site dictionaries
``{"q", "qshape", "dshape", "blocks"}`` (blocks keyed by the row-major sparse
tag), the neutral exchange format both the device path and the oracle consume.
"""
from __future__ import annotations

from typing import Dict, List, Sequence, Tuple

import numpy as np

VAC, ALPHA, BETA, PAIR = 0, 1, 2, 3
SITE_Q = [(0, 0), (1, 1), (1, -1), (2, 0)]

# one-site operators as {(bra, ket): value} (src/prime_operators.cpp:12-131)
OPS: Dict[str, Dict[Tuple[int, int], float]] = {
    "I": {(VAC, VAC): 1.0, (ALPHA, ALPHA): 1.0, (BETA, BETA): 1.0, (PAIR, PAIR): 1.0},
    "Ca": {(ALPHA, VAC): 1.0, (PAIR, BETA): -1.0},
    "Da": {(VAC, ALPHA): 1.0, (BETA, PAIR): -1.0},
    "Cb": {(BETA, VAC): 1.0, (PAIR, ALPHA): 1.0},
    "Db": {(VAC, BETA): 1.0, (ALPHA, PAIR): 1.0},
    "NaNb": {(PAIR, PAIR): 1.0},
}
OP_Q = {"I": (0, 0), "Ca": (1, 1), "Da": (-1, -1), "Cb": (1, -1), "Db": (-1, 1), "NaNb": (0, 0)}


def _op_matrix(name: str) -> np.ndarray:
    m = np.zeros((4, 4))
    for (b, k), v in OPS[name].items():
        m[b, k] = v
    return m


def op_matrix(name: str) -> np.ndarray:
    """Dense 4x4 matrix of a named one-site operator (bra, ket)."""
    return _op_matrix(name)


def _neg(q):
    return (-q[0], -q[1])


class SiteMPO:
    """Accumulates the 1x1x1x1 blocks of one site operator W[w,s,s',w']."""

    def __init__(self, q_left: Sequence[Tuple[int, int]], q_right_ops: Sequence[Tuple[int, int]]):
        self.ql = [tuple(q) for q in q_left]
        # right bond quantum shape is minus the charge of the next left operators
        self.qr = [_neg(tuple(q)) for q in q_right_ops]
        self.entries: Dict[Tuple[int, int, int, int], float] = {}

    def add(self, w: int, mat: np.ndarray, w2: int, coef: float = 1.0):
        """W[w,:,:,w2] += coef * (sign-adjusted) mat."""
        if coef == 0.0:
            return
        lpar = self.ql[w][0] & 1
        for s in range(4):
            for sp in range(4):
                v = mat[s, sp]
                if v == 0.0:
                    continue
                if lpar and (SITE_Q[s][0] & 1):
                    v = -v
                key = (w, s, sp, w2)
                self.entries[key] = self.entries.get(key, 0.0) + coef * v

    def to_dict(self) -> dict:
        nl, nr = len(self.ql), len(self.qr)
        qshape = [self.ql, list(SITE_Q), [_neg(q) for q in SITE_Q], self.qr]
        dshape = [[1] * nl, [1] * 4, [1] * 4, [1] * nr]
        strides = (4 * 4 * nr, 4 * nr, nr, 1)
        blocks = {}
        for (w, s, sp, w2), v in sorted(self.entries.items()):
            if v == 0.0:
                continue
            q = tuple(a + b for a, b in zip(self.ql[w], SITE_Q[s]))
            q = (q[0] - SITE_Q[sp][0] + self.qr[w2][0], q[1] - SITE_Q[sp][1] + self.qr[w2][1])
            if q != (0, 0):
                raise ValueError("MPO element violates quantum-number conservation")
            tag = w * strides[0] + s * strides[1] + sp * strides[2] + w2
            blocks[tag] = np.full((1, 1, 1, 1), v)
        return {"q": (0, 0), "qshape": qshape, "dshape": dshape, "blocks": blocks}


def hubbard_mpo(L: int, t, U) -> List[dict]:
    """Open-chain Hubbard MPO.

    H = sum_i t_i sum_s (c+_{i s} c_{i+1 s} + h.c.) + sum_i U_i n_{i up} n_{i dn}
    (``t_i`` is the one-electron integral h_{i,i+1}; scalars broadcast).
    Left-block operators at an inner bond: I, H, c+_a, c+_b, c_a, c_b of the last
    site, so the bond dimension is 6.
    """
    tt = np.broadcast_to(np.asarray(t, dtype=np.float64), (max(L - 1, 1),)).copy()
    uu = np.broadcast_to(np.asarray(U, dtype=np.float64), (L,)).copy()
    Ca, Da, Cb, Db, I, NN = (_op_matrix(n) for n in ("Ca", "Da", "Cb", "Db", "I", "NaNb"))
    inner = [(0, 0), (0, 0), (1, 1), (1, -1), (-1, -1), (-1, 1)]  # I, H, Ca, Cb, Da, Db
    sites = []
    for k in range(L):
        left = [(0, 0)] if k == 0 else inner
        right = [(0, 0)] if k == L - 1 else inner
        W = SiteMPO(left, right)
        last = k == L - 1
        iH_r = 0 if last else 1
        # identity propagation
        if not last:
            W.add(0, I, 0)
        if k > 0:
            W.add(1, I, iH_r)  # H * 1
        W.add(0, NN, iH_r, uu[k])  # on-site U
        if k > 0:
            h = tt[k - 1]
            # c+_{k-1 s} c_{k s}
            W.add(2, Da, iH_r, h)
            W.add(3, Db, iH_r, h)
            # c+_{k s} c_{k-1 s} = - c_{k-1 s} c+_{k s}
            W.add(4, Ca, iH_r, -h)
            W.add(5, Cb, iH_r, -h)
        if not last:
            W.add(0, Ca, 2)
            W.add(0, Cb, 3)
            W.add(0, Da, 4)
            W.add(0, Db, 5)
        sites.append(W.to_dict())
    return sites


def mpo_bond_dims(mpo: List[dict]) -> List[int]:
    return [len(s["qshape"][3]) for s in mpo]
