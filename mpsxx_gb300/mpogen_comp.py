"""The complementary-operator MPO of a quantum-chemistry Hamiltonian, built the way
the mpsxx reference's generator builds it (``src/gen_qc_operators.cpp:18-202``,
``src/boundary_opinfo.cpp:48-140``, ``src/get_product_ops.cpp:41-346``,
``src/gen_site_operator.cpp:9-169``, ``src/integral_component.cpp:6-304``): the
default ``mpogen.x`` run, one operator group, no swap sweep.

At the boundary after site i, with L = i+1 sites on the left and R = N-L on the
right, the left block carries I, H, the single operators C/D of the left orbitals,
the complementary single operators (Q_k = the left block's share of the terms with
one operator on orbital k) of the right orbitals, and the normal double operators
of the left orbitals: 2 + 4N - 2L + 8L^2 operators.  Every site tensor is built
by pairing each left-block operator with each one-site operator, keeping products
that are operators of the next boundary, with coefficients from the integrals;
operators no term reaches are then removed, forward and backward.

Operators are identified by the reference's 32-bit operator codes (a type field,
two spin/creation fields and two 12-bit orbital indices): the sector order of each
bond follows their enumeration order there, the order in which a site's terms are
summed follows their numerical order, so the result equals the reference's MPO in
block structure and values.  The swap-sweep variant (``mpogen.x -x``) is not
restated.

Site tensors are returned in the neutral exchange format of ``mpogen``:
``{"q", "qshape", "dshape", "blocks": {tag: ndarray (1,1,1,1)}}``.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .mpogen import SITE_Q

# ---------------------------------------------------------------------------
# operator codes (src/bit_operator_type.h:13-78)
# ---------------------------------------------------------------------------
ZERO = 0x00000000
IDEN = 0x40000000
HAM = 0xC0000000
TYPE = 0xF0000000
NORMAL = 0x7FFFFFFF
COMP = 0x80000000
MASK = 0x7C003000
FIRST = 0x0FFFC000
SECOND = 0x00003FFF
INDEX = 0x03FFCFFF
DOUBLE = 0x30000000
SINGLE = 0x20000000
SINGLE_2 = 0x10000000
SINGLE_COMP = 0xA0000000
CONJ_S = 0x08000000
CRE_A, CRE_B, DES_A, DES_B = 0x2C000000, 0x28000000, 0x24000000, 0x20000000
CRE_A_CRE_A, CRE_A_CRE_B, CRE_B_CRE_A, CRE_B_CRE_B = 0x3C003000, 0x3C002000, 0x38003000, 0x38002000
CRE_A_DES_A, CRE_A_DES_B, CRE_B_DES_A, CRE_B_DES_B = 0x3C001000, 0x3C000000, 0x38001000, 0x38000000
DES_A_CRE_A, DES_A_CRE_B, DES_B_CRE_A, DES_B_CRE_B = 0x34003000, 0x34002000, 0x30003000, 0x30002000
DES_A_DES_A, DES_A_DES_B, DES_B_DES_A, DES_B_DES_B = 0x34001000, 0x34000000, 0x30001000, 0x30000000
FIELD_SHIFT = 12
INDEX_SHIFT = 14
U32 = 0xFFFFFFFF

# the physical states of a site (src/mpsite.h)
VAC, ALPHA, BETA, PAIR = 0, 1, 2, 3

# one-site operators: (bra, ket, value) (src/prime_operators.cpp:12-131)
PRIME = {
    "I": ((VAC, VAC, 1.0), (ALPHA, ALPHA, 1.0), (BETA, BETA, 1.0), (PAIR, PAIR, 1.0)),
    "Ca": ((ALPHA, VAC, 1.0), (PAIR, BETA, -1.0)),
    "Da": ((VAC, ALPHA, 1.0), (BETA, PAIR, -1.0)),
    "Cb": ((BETA, VAC, 1.0), (PAIR, ALPHA, 1.0)),
    "Db": ((VAC, BETA, 1.0), (ALPHA, PAIR, 1.0)),
    "CaCb": ((PAIR, VAC, -1.0),),
    "DaDb": ((VAC, PAIR, 1.0),),
    "CaDa": ((ALPHA, ALPHA, 1.0), (PAIR, PAIR, 1.0)),
    "CaDb": ((ALPHA, BETA, 1.0),),
    "CbDa": ((BETA, ALPHA, 1.0),),
    "CbDb": ((BETA, BETA, 1.0), (PAIR, PAIR, 1.0)),
    "CaCbDb": ((PAIR, BETA, -1.0),),
    "CbCaDa": ((PAIR, ALPHA, 1.0),),
    "CaDaDb": ((ALPHA, PAIR, 1.0),),
    "CbDbDa": ((BETA, PAIR, -1.0),),
    "CaDaCbDb": ((PAIR, PAIR, 1.0),),
}


def get_quantum(op: int) -> Tuple[int, int]:
    """(particle number, 2 Sz) of an operator code (src/bit_operator_type.cpp:5-24)."""
    p = s = 0
    if (op & IDEN) == 0:
        if op & SINGLE:
            o1 = (op & MASK & FIRST) >> INDEX_SHIFT >> FIELD_SHIFT
            if o1 & 2:
                p += 1
                s += 1 if o1 & 1 else -1
            else:
                p -= 1
                s += -1 if o1 & 1 else 1
        if op & SINGLE_2:
            o2 = (op & MASK & SECOND) >> FIELD_SHIFT
            if o2 & 2:
                p += 1
                s += 1 if o2 & 1 else -1
            else:
                p -= 1
                s += -1 if o2 & 1 else 1
    return (p, s)


def _first(op: int) -> int:
    return (op & INDEX & FIRST) >> INDEX_SHIFT


# ---------------------------------------------------------------------------
# operators at a boundary (src/boundary_opinfo.cpp:5-140): {code: sector}
# ---------------------------------------------------------------------------
def site_ops(i: int) -> Dict[int, int]:
    """The one-site operators of orbital i, numbered in the reference's order."""
    codes = [IDEN, HAM | (i << INDEX_SHIFT), CRE_A | (i << INDEX_SHIFT), CRE_B | (i << INDEX_SHIFT),
             DES_A | (i << INDEX_SHIFT), DES_B | (i << INDEX_SHIFT), COMP | CRE_A | (i << INDEX_SHIFT),
             COMP | CRE_B | (i << INDEX_SHIFT), COMP | DES_A | (i << INDEX_SHIFT), COMP | DES_B | (i << INDEX_SHIFT)]
    codes += [t | (i << INDEX_SHIFT) | i for t in (CRE_A_DES_A, CRE_B_DES_B, CRE_A_CRE_B, CRE_A_DES_B, DES_A_CRE_B,
                                                    DES_A_DES_B)]
    return {c & U32: k for k, c in enumerate(codes)}


def boundary_ops(L: int, N: int) -> Dict[int, int]:
    """Left-block operators after L sites (forward direction, no swap sweep)."""
    R = N - L
    ops: Dict[int, int] = {}

    def add(c):
        if c not in ops:
            ops[c] = len(ops)

    if R > 0:
        add(IDEN)
    if L > 0:
        add(HAM)
    if L == 0 or R == 0:
        return ops
    for i in range(L):
        for t in (CRE_A, CRE_B, DES_A, DES_B):
            add(t | (i << INDEX_SHIFT))
    for i in range(L, N):
        for t in (CRE_A, CRE_B, DES_A, DES_B):
            add((COMP | t | (i << INDEX_SHIFT)) & U32)
    for i in range(L):
        for t in (CRE_A_DES_A, CRE_B_DES_B, CRE_A_CRE_B, CRE_A_DES_B, DES_A_CRE_B, DES_A_DES_B):
            add(t | (i << INDEX_SHIFT) | i)
        for j in range(i):
            for t in (CRE_A_CRE_A, CRE_A_CRE_B, CRE_B_CRE_A, CRE_B_CRE_B, CRE_A_DES_A, CRE_A_DES_B, CRE_B_DES_A,
                      CRE_B_DES_B, DES_A_CRE_A, DES_A_CRE_B, DES_B_CRE_A, DES_B_CRE_B, DES_A_DES_A, DES_A_DES_B,
                      DES_B_DES_A, DES_B_DES_B):
                add(t | (j << INDEX_SHIFT) | i)
    return ops


# ---------------------------------------------------------------------------
# product of a left-block and a one-site operator (src/get_product_ops.cpp:41-346,
# the branches without swap sweep)
# ---------------------------------------------------------------------------
def product_ops(l_op: int, s_op: int, r_indxs: Sequence[int]) -> List[int]:
    lt, st = l_op & NORMAL & TYPE, s_op & NORMAL & TYPE
    if s_op == IDEN:
        if lt == DOUBLE:
            return [l_op]
        if lt == SINGLE:
            if l_op & COMP:
                return [l_op] if _first(l_op) in r_indxs else []
            return [l_op]
        if l_op & IDEN:
            return [l_op]
        return []
    if l_op == IDEN:
        if st == DOUBLE:
            return [s_op]
        if st == SINGLE:
            if s_op & COMP:
                base = s_op & (~INDEX & U32)
                return [base | (ix << INDEX_SHIFT) for ix in r_indxs]
            return [s_op]
        if s_op & IDEN:
            return [s_op & TYPE]
        return []
    if lt == SINGLE and st == SINGLE:
        if (l_op & COMP) == 0 and (s_op & COMP) == 0:
            if _first(l_op) > _first(s_op):
                return [DOUBLE | (s_op & FIRST) | ((l_op & FIRST) >> INDEX_SHIFT)]
            return [DOUBLE | (l_op & FIRST) | ((s_op & FIRST) >> INDEX_SHIFT)]
        if (l_op & COMP) and ((l_op ^ CONJ_S) & NORMAL) == s_op:
            return [HAM]
        if (l_op & COMP) == 0 and ((s_op ^ CONJ_S) & MASK) == (l_op & MASK):
            return [HAM]
        return []

    def comp_of(d_op, x_op):
        q = get_quantum(d_op)
        qx = get_quantum(x_op)
        if abs(q[0] + qx[0]) == 1 and abs(q[1] + qx[1]) == 1:
            r = (d_op & FIRST) ^ ((d_op & SECOND) << INDEX_SHIFT) ^ (x_op & FIRST)
            r = ((COMP | SINGLE | (r & MASK & FIRST)) ^ CONJ_S) & U32
            return [r | (ix << INDEX_SHIFT) for ix in r_indxs]
        return []

    if lt == DOUBLE and st == SINGLE and (s_op & COMP) == 0:
        return comp_of(l_op, s_op)
    if st == DOUBLE and lt == SINGLE and (l_op & COMP) == 0:
        return comp_of(s_op, l_op)
    if lt == DOUBLE and st == DOUBLE:
        ql, qs = get_quantum(l_op), get_quantum(s_op)
        if ql[0] + qs[0] == 0 and ql[1] + qs[1] == 0:
            return [HAM]
    return []


# ---------------------------------------------------------------------------
# integral coefficients (src/integral_component.cpp:6-304)
# ---------------------------------------------------------------------------
# Non-zero entries of the reference's 256-entry table from the spin/creation pattern of
# four operators (2 bits each, first operator highest) to the integral combination:
# 1: v(i,j,l,k)  2: v(i,j,k,l)  3: v(i,k,j,l); +4: negated; +8: minus v(i,j,k,l),
# v(i,k,j,l), v(i,j,l,k) respectively (src/integral_component.cpp:127-160).
INT2E_TYPE = {
    0x0A: 9, 0x1B: 6, 0x1E: 1, 0x22: 11, 0x27: 3, 0x28: 10, 0x2D: 7, 0x36: 5, 0x39: 2, 0x4B: 1, 0x4E: 6, 0x5F: 9,
    0x63: 5, 0x6C: 2, 0x72: 3, 0x77: 11, 0x78: 7, 0x7D: 10, 0x82: 10, 0x87: 7, 0x88: 11, 0x8D: 3, 0x93: 2, 0x9C: 5,
    0xA0: 9, 0xB1: 6, 0xB4: 1, 0xC6: 2, 0xC9: 5, 0xD2: 7, 0xD7: 10, 0xD8: 3, 0xDD: 11, 0xE1: 1, 0xE4: 6, 0xF5: 9,
}


def _int1e_index(l_op: int, s_op: int, r_op: int) -> Tuple[int, List[int]]:
    """(type code, [i, j]) of the one-electron entry an operator triple reads."""
    idx, itype = [], 0
    for op in (l_op, s_op):
        if (op & NORMAL & TYPE) == SINGLE:
            idx.append(_first(op))
            itype |= (op & MASK & FIRST) >> (INDEX_SHIFT + FIELD_SHIFT + 2 * len(idx) - 4)
    if (s_op & TYPE) == HAM:
        i = _first(s_op)
        idx += [i, i]
        itype = 0xD
    if (r_op & NORMAL & TYPE) == SINGLE:
        idx.append(_first(r_op))
        itype |= (r_op & MASK & FIRST) >> (INDEX_SHIFT + FIELD_SHIFT + 2 * len(idx) - 4)
    assert len(idx) == 2
    return itype, idx


def int1e_component(l_op: int, s_op: int, r_op: int, h: np.ndarray) -> float:
    itype, idx = _int1e_index(l_op, s_op, r_op)
    if itype in (0xD, 0x8):
        return float(h[idx[0], idx[1]])
    if itype in (0x7, 0x2):
        return -float(h[idx[0], idx[1]])
    return 0.0


def int1e_derivative(l_op: int, s_op: int, r_op: int) -> Dict[object, float]:
    """d(int1e_component)/d(parameter): the entry h[i, j] read is the lower-triangle
    element h1[max(i, j), min(i, j)] (the one the FCIDUMP holds), key ("h", p, q)."""
    itype, (i, j) = _int1e_index(l_op, s_op, r_op)
    sign = 1.0 if itype in (0xD, 0x8) else -1.0 if itype in (0x7, 0x2) else 0.0
    return {("h", max(i, j), min(i, j)): sign} if sign else {}


def _add_ops(op: int, idx: list, itype: int, single_mask: int) -> int:
    t = op & single_mask & TYPE
    if t == SINGLE:
        idx.append(_first(op))
        itype |= (op & MASK & FIRST) >> (INDEX_SHIFT + FIELD_SHIFT + 2 * len(idx) - 8)
    elif t == DOUBLE:
        idx.append(_first(op))
        itype |= (op & MASK & FIRST) >> (INDEX_SHIFT + FIELD_SHIFT + 2 * len(idx) - 8)
        idx.append(op & INDEX & SECOND)
        itype |= (op & MASK & SECOND) >> (FIELD_SHIFT + 2 * len(idx) - 8)
    return itype


def _int2e_index(l_op: int, s_op: int, r_op: int) -> Tuple[int, List[int]]:
    """(combination code from INT2E_TYPE, [i, j, k, l]) of the two-electron entries an
    operator triple reads."""
    idx: list = []
    itype = _add_ops(l_op, idx, 0, NORMAL)
    st = s_op & TYPE
    if st in (SINGLE, DOUBLE):
        itype = _add_ops(s_op, idx, itype, U32)
    elif st == SINGLE_COMP:
        oc = (s_op & MASK & FIRST) >> (INDEX_SHIFT + FIELD_SHIFT)
        k = _first(s_op)
        seq = (oc, oc ^ 1, oc ^ 3) if oc & 2 else (oc ^ 3, oc ^ 1, oc)
        for o in seq:
            idx.append(k)
            itype |= o << (8 - 2 * len(idx))
    elif st == HAM:
        k = _first(s_op)
        idx += [k, k, k, k]
        itype = 0xD8
    itype = _add_ops(r_op, idx, itype, NORMAL)
    assert len(idx) == 4 and itype < 256
    return INT2E_TYPE.get(itype, 0), idx


def _int2e_terms(m: int, idx: List[int]) -> List[Tuple[float, Tuple[int, int, int, int]]]:
    """The signed entries of v (reference layout) that combination m adds up."""
    i, j, k, l = idx
    first = {1: (i, j, l, k), 2: (i, j, k, l), 3: (i, k, j, l)}.get(m % 4)
    if first is None:
        return []
    second = {1: (i, j, k, l), 2: (i, k, j, l), 3: (i, j, l, k)}[m % 4]
    sign = -1.0 if m & 4 else 1.0
    out = [(sign, first)]
    if m & 8:
        out.append((-sign, second))
    return out


def int2e_component(l_op: int, s_op: int, r_op: int, v: np.ndarray) -> float:
    """v[i,j,k,l] in the reference's layout: v[i,k,j,l] holds (ij|kl)."""
    m, idx = _int2e_index(l_op, s_op, r_op)
    i, j, k, l = idx
    val = 0.0
    if m % 4 == 1:
        val += v[i, j, l, k]
        if m & 8:
            val -= v[i, j, k, l]
    elif m % 4 == 2:
        val += v[i, j, k, l]
        if m & 8:
            val -= v[i, k, j, l]
    elif m % 4 == 3:
        val += v[i, k, j, l]
        if m & 8:
            val -= v[i, j, l, k]
    return float(-val if m & 4 else val)


def _canonical_eri(p: int, q: int, r: int, s: int) -> Tuple[int, int, int, int]:
    """The canonical index of (pq|rs) under 8-fold symmetry (p >= q, r >= s, pq >= rs)."""
    a, b = max(p, q), min(p, q)
    c, d = max(r, s), min(r, s)
    if a * (a + 1) // 2 + b < c * (c + 1) // 2 + d:
        a, b, c, d = c, d, a, b
    return a, b, c, d


def int2e_derivative(l_op: int, s_op: int, r_op: int) -> Dict[object, float]:
    """d(int2e_component)/d(parameter), key ("eri", canonical p, q, r, s): the entry
    v[a, b, c, d] is (ac|bd), which the reference fills from the canonical element."""
    out: Dict[object, float] = {}
    for sign, (a, b, c, d) in _int2e_terms(*_int2e_index(l_op, s_op, r_op)):
        key = ("eri",) + _canonical_eri(a, c, b, d)
        out[key] = out.get(key, 0.0) + sign
    return {k: x for k, x in out.items() if x != 0.0}


# ---------------------------------------------------------------------------
# one site tensor (src/gen_site_operator.cpp:9-169, src/prime_operators.h:167-187)
# ---------------------------------------------------------------------------
class _Site:
    def __init__(self, lq: Sequence[Tuple[int, int]], rq: Sequence[Tuple[int, int]], track: bool = False):
        self.lq, self.rq = lq, rq  # left sector charges; right sector charges (before negation)
        self.blocks: Dict[Tuple[int, int, int, int], float] = {}
        # with track: d(block)/d(parameter) per block, parameters as int1e_derivative /
        # int2e_derivative name them
        self.jac: Optional[Dict[Tuple[int, int, int, int], Dict[object, float]]] = {} if track else None

    def prime(self, name: str, li: int, ri: int, scale: float, dscale: Optional[Dict[object, float]] = None):
        if abs(scale) < 1.0e-16:
            return
        odd_l = self.lq[li][0] & 1
        for bra, ket, x in PRIME[name]:
            flip = odd_l and SITE_Q[bra][0] & 1
            val = -scale * x if flip else scale * x
            key = (li, bra, ket, ri)
            if key in self.blocks:
                self.blocks[key] = self.blocks[key] + val
            else:
                self.blocks[key] = val
            if self.jac is not None and dscale:
                jk = self.jac.setdefault(key, {})
                f = -x if flip else x
                for par, dv in dscale.items():
                    jk[par] = jk.get(par, 0.0) + f * dv

    def remap(self, fn):
        """Re-key blocks (and their derivatives) by fn(key) -> new key or None (dropped)."""
        keep = {k: fn(k) for k in self.blocks}
        self.blocks = {nk: x for k, x in self.blocks.items() if (nk := keep[k]) is not None}
        if self.jac is not None:
            self.jac = {nk: d for k, d in self.jac.items() if (nk := keep.get(k)) is not None}


def gen_site_operator(site: _Site, l_op: int, li: int, s_op: int, r_op: int, ri: int, ecore: float,
                      h: np.ndarray, v: np.ndarray):
    track = site.jac is not None

    def i1(l, s_, r):
        return int1e_component(l, s_, r, h), (int1e_derivative(l, s_, r) if track else None)

    def i2(l, s_, r):
        return int2e_component(l, s_, r, v), (int2e_derivative(l, s_, r) if track else None)

    st = s_op & TYPE
    if st == IDEN:
        v2, d2 = 1.0, None
        if (l_op & TYPE) == DOUBLE and (r_op & TYPE) == DOUBLE and (l_op & INDEX) != (r_op & INDEX):
            v2, d2 = i2(l_op, s_op, r_op)
        site.prime("I", li, ri, v2, d2)
    elif st == HAM:
        if not (s_op & INDEX) and abs(ecore) > 1.0e-16:
            site.prime("I", li, ri, ecore)
        v1, d1 = i1(l_op, s_op, r_op)
        v2, d2 = i2(l_op, s_op, r_op)
        site.prime("CaDa", li, ri, v1, d1)
        site.prime("CbDb", li, ri, v1, d1)
        site.prime("CaDaCbDb", li, ri, v2, d2)
    elif st == SINGLE:
        v2, d2 = 1.0, None
        if (l_op & NORMAL & TYPE) == SINGLE and (r_op & TYPE) == DOUBLE:
            conj = (COMP | CONJ_S) if (l_op & COMP) else 0
            lc = (l_op ^ conj) & U32
            if (DOUBLE | (lc & FIRST) | ((s_op & FIRST) >> INDEX_SHIFT)) != r_op and \
                    (DOUBLE | ((lc & FIRST) >> INDEX_SHIFT) | (s_op & FIRST)) != r_op:
                v2, d2 = i2(lc, s_op, r_op)
        elif (l_op & TYPE) == DOUBLE and (r_op & NORMAL & TYPE) == SINGLE:
            conj = (COMP | CONJ_S) if (r_op & COMP) else 0
            rc = (r_op ^ conj) & U32
            if (DOUBLE | (s_op & FIRST) | ((rc & FIRST) >> INDEX_SHIFT)) != l_op and \
                    (DOUBLE | ((s_op & FIRST) >> INDEX_SHIFT) | (rc & FIRST)) != l_op:
                v2, d2 = i2(l_op, s_op, rc)
        name = {CRE_A: "Ca", CRE_B: "Cb", DES_A: "Da", DES_B: "Db"}.get(s_op & MASK)
        if name:
            site.prime(name, li, ri, v2, d2)
    elif st == SINGLE_COMP:
        v1 = v2 = 0.0
        d1 = d2 = None
        if (l_op & NORMAL & TYPE) == SINGLE:
            conj = (COMP | CONJ_S) if (l_op & COMP) else 0
            lc = (l_op ^ conj) & U32
            v1, d1 = i1(lc, s_op, r_op)
            v2, d2 = i2(lc, s_op, r_op)
            v1 *= 0.5
        elif (r_op & NORMAL & TYPE) == SINGLE:
            conj = (COMP | CONJ_S) if (r_op & COMP) else 0
            rc = (r_op ^ conj) & U32
            v1, d1 = i1(l_op, s_op, rc)
            v2, d2 = i2(l_op, s_op, rc)
            v1 *= 0.5
        if d1:
            d1 = {k: 0.5 * x for k, x in d1.items()}
        pair = {CRE_A: ("Ca", "CaCbDb"), CRE_B: ("Cb", "CbCaDa"), DES_A: ("Da", "CbDbDa"),
                DES_B: ("Db", "CaDaDb")}.get(s_op & MASK)
        if pair:
            site.prime(pair[0], li, ri, v1, d1)
            site.prime(pair[1], li, ri, v2, d2)
    elif st == DOUBLE:
        v2, d2 = 1.0, None
        lt, rt = l_op & TYPE, r_op & TYPE
        if lt == SINGLE and rt == SINGLE:
            v2, d2 = i2(l_op, s_op, r_op)
        elif lt == SINGLE and rt == SINGLE_COMP:
            v2, d2 = i2(l_op, s_op, (r_op ^ COMP ^ CONJ_S) & U32)
        elif rt == SINGLE and lt == SINGLE_COMP:
            v2, d2 = i2((l_op ^ COMP ^ CONJ_S) & U32, s_op, r_op)
        elif lt == DOUBLE and (l_op & INDEX) != (s_op & INDEX):
            v2, d2 = i2(l_op, s_op, r_op)
        elif rt == DOUBLE and (r_op & INDEX) != (s_op & INDEX):
            v2, d2 = i2(l_op, s_op, r_op)
        m = s_op & MASK
        if m == CRE_A_DES_A:
            site.prime("CaDa", li, ri, v2, d2)
        elif m == CRE_B_DES_B:
            site.prime("CbDb", li, ri, v2, d2)
        elif m == CRE_A_CRE_B:
            site.prime("CaCb", li, ri, v2, d2)
        elif m == CRE_A_DES_B:
            site.prime("CaDb", li, ri, v2, d2)
        elif m == DES_A_CRE_B:
            site.prime("CbDa", li, ri, -v2, {k: -x for k, x in d2.items()} if d2 else None)
        elif m == DES_A_DES_B:
            site.prime("DaDb", li, ri, v2, d2)


# ---------------------------------------------------------------------------
# the generator (src/gen_qc_operators.cpp:18-202)
# ---------------------------------------------------------------------------
def reference_integrals(h1: np.ndarray, eri: np.ndarray, tol: float = 1.0e-16):
    """The reference's integral arrays from chemist-order (pq|rs): oneint = h1 and
    twoint[i,k,j,l] = (ij|kl) (src/parsing_integral.cpp:105-154), entries below tol
    dropped as the operator-group selection does (src/make_qc_mpos.cpp:56-117)."""
    n = h1.shape[0]
    # one value per symmetry class, taken at the FCIDUMP's canonical index (i >= j,
    # k >= l, ij >= kl; h_ij at i >= j), as the reference's parser fills all of them
    h = np.tril(h1) + np.tril(h1, -1).T
    i, j, k, l = np.indices((n, n, n, n))
    a, b = np.maximum(i, j), np.minimum(i, j)
    c, d = np.maximum(k, l), np.minimum(k, l)
    swap = a * (a + 1) // 2 + b < c * (c + 1) // 2 + d
    e = eri[np.where(swap, c, a), np.where(swap, d, b), np.where(swap, a, c), np.where(swap, b, d)]
    h = np.where(np.abs(h) >= tol, h, 0.0)
    v = np.ascontiguousarray(np.transpose(e, (0, 2, 1, 3)))
    v = np.where(np.abs(v) >= tol, v, 0.0)
    return h, v


def qc_mpo_complementary(h1: np.ndarray, eri: np.ndarray, ecore: float = 0.0, jacobian: bool = False):
    """The reference generator's MPO for H = sum h_pq a+_p a_q + 1/2 sum (pq|rs) ...
    (integrals in chemist order, 8-fold symmetric), one dict per site.

    With ``jacobian`` also, per site, {block tag: {parameter: d(block)/d(parameter)}}:
    every block is a linear combination of the integrals the reference reads, which
    are h1[p, q] with p >= q (key ("h", p, q)) and the canonical (pq|rs) of each
    8-fold class (key ("eri", p, q, r, s), p >= q, r >= s, pq >= rs).  A derivative
    is with respect to the symmetric parameter, i.e. all its equal entries at once."""
    N = h1.shape[0]
    h, v = reference_integrals(h1, eri)
    l_ops = boundary_ops(0, N)
    r_indxs = list(range(N - 1, 0, -1))
    sites: List[Tuple[dict, dict, _Site]] = []
    for i in range(N):
        s_ops = site_ops(i)
        r_ops = boundary_ops(i + 1, N)
        lq = [None] * len(l_ops)
        for c, k in l_ops.items():
            lq[k] = get_quantum(c)
        rq = [None] * len(r_ops)
        for c, k in r_ops.items():
            rq[k] = get_quantum(c)
        site = _Site(lq, rq, track=jacobian)
        s_sorted = sorted(s_ops)
        for l_op in sorted(l_ops):
            li = l_ops[l_op]
            for s_op in s_sorted:
                for p in product_ops(l_op, s_op, r_indxs):
                    ri = r_ops.get(p)
                    if ri is not None:
                        gen_site_operator(site, l_op, li, s_op, p, ri, ecore, h, v)
        # forward removal: right sectors no block reaches (BoundaryOpInfo::clean)
        used = sorted({k[3] for k in site.blocks})
        remap = {old: new for new, old in enumerate(used)}
        site.remap(lambda k: (k[0], k[1], k[2], remap[k[3]]))
        site.rq = [rq[o] for o in used]
        kept = {c: remap[k] for c, k in r_ops.items() if k in remap}
        sites.append(site)
        l_ops = kept
        if r_indxs:
            r_indxs.pop()
    # backward removal: left sectors that no longer connect to the right
    r_keep = [0]
    for i in range(N - 1, -1, -1):
        s = sites[i]
        keep_r = {old: new for new, old in enumerate(r_keep)}
        s.remap(lambda k: (k[0], k[1], k[2], keep_r[k[3]]) if k[3] in keep_r else None)
        used_l = sorted({k[0] for k in s.blocks})
        remap_l = {old: new for new, old in enumerate(used_l)}
        s.remap(lambda k: (remap_l[k[0]], k[1], k[2], k[3]))
        s.rq = [s.rq[o] for o in r_keep]
        s.lq = [s.lq[o] for o in used_l]
        r_keep = used_l
    out, jacs = [], []
    neg = lambda q: (-q[0], -q[1])  # noqa: E731
    for s in sites:
        qshape = [list(s.lq), list(SITE_Q), [neg(q) for q in SITE_Q], [neg(q) for q in s.rq]]
        dshape = [[1] * len(x) for x in qshape]
        n1, n2, n3 = len(qshape[1]), len(qshape[2]), len(qshape[3])
        tag = lambda k: ((k[0] * n1 + k[1]) * n2 + k[2]) * n3 + k[3]  # noqa: E731
        blocks = {}
        for key, x in s.blocks.items():
            blocks[tag(key)] = np.full((1, 1, 1, 1), x)
        out.append({"q": (0, 0), "qshape": qshape, "dshape": dshape, "blocks": dict(sorted(blocks.items()))})
        if jacobian:
            jacs.append({tag(key): {p: x for p, x in d.items() if x != 0.0}
                         for key, d in s.jac.items() if key in s.blocks and any(x != 0.0 for x in d.values())})
    if jacobian:
        return out, jacs
    return out
