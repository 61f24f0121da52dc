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

from typing import Dict, List, Optional, Sequence, Tuple

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
        # d(entry)/d(parameter) of the Hamiltonian parameters the entries depend on
        self.jac: Dict[Tuple[int, int, int, int], Dict[object, float]] = {}

    def add(self, w: int, mat: np.ndarray, w2: int, coef: float = 1.0, dcoef: Optional[Dict[object, float]] = None):
        """W[w,:,:,w2] += coef * (sign-adjusted) mat.  ``dcoef`` maps parameters to
        d(coef)/d(parameter); the entries' derivatives are accumulated alongside."""
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
                if dcoef:
                    jk = self.jac.setdefault(key, {})
                    for par, dv in dcoef.items():
                        jk[par] = jk.get(par, 0.0) + dv * v

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

    def jacobian(self) -> Dict[int, Dict[object, float]]:
        """{block tag: {parameter: d(block)/d(parameter)}} over the stored blocks."""
        nr = len(self.qr)
        strides = (4 * 4 * nr, 4 * nr, nr, 1)
        out = {}
        for key, d in self.jac.items():
            if self.entries.get(key, 0.0) == 0.0:
                continue
            w, s, sp, w2 = key
            tag = w * strides[0] + s * strides[1] + sp * strides[2] + w2
            nz = {par: v for par, v in d.items() if v != 0.0}
            if nz:
                out[tag] = nz
        return out


def hubbard_mpo(L: int, t, U, jacobian: bool = False):
    """Open-chain Hubbard MPO.

    H = sum_i t_i sum_s (c+_{i s} c_{i+1 s} + h.c.) + sum_i U_i n_{i up} n_{i dn}
    (``t_i`` is the one-electron integral h_{i,i+1}; scalars broadcast).
    Left-block operators at an inner bond: I, H, c+_a, c+_b, c_a, c_b of the last
    site, so the bond dimension is 6.  With ``jacobian`` also returns, per site,
    {block tag: {("t", i) or ("U", i): d(block)/d(parameter)}} (the MPO is linear in
    the parameters; a parameter that is exactly zero has no block to carry it).
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
        W.add(0, NN, iH_r, uu[k], {("U", k): 1.0})  # on-site U
        if k > 0:
            h = tt[k - 1]
            dt = {("t", k - 1): 1.0}
            dmt = {("t", k - 1): -1.0}
            # c+_{k-1 s} c_{k s}
            W.add(2, Da, iH_r, h, dt)
            W.add(3, Db, iH_r, h, dt)
            # c+_{k s} c_{k-1 s} = - c_{k-1 s} c+_{k s}
            W.add(4, Ca, iH_r, -h, dmt)
            W.add(5, Cb, iH_r, -h, dmt)
        if not last:
            W.add(0, Ca, 2)
            W.add(0, Cb, 3)
            W.add(0, Da, 4)
            W.add(0, Db, 5)
        sites.append(W)
    if jacobian:
        return [W.to_dict() for W in sites], [W.jacobian() for W in sites]
    return [W.to_dict() for W in sites]


def mpo_bond_dims(mpo: List[dict]) -> List[int]:
    return [len(s["qshape"][3]) for s in mpo]


# ---------------------------------------------------------------------------
# Generic sum-of-products -> MPO (quantum-chemistry Hamiltonians)
# ---------------------------------------------------------------------------
#
# A term is a product of spin-orbital creation/annihilation operators.  Each term
# is brought to site order (sign from the fermionic reordering), operators on the
# same site are fused into one 4x4 site operator, and the MPO is grown from the
# left: at site k every term is (left bond operator a, site operator o, rest of
# the string); the bipartite graph between distinct (a, o) and distinct rests is
# covered by a minimum vertex cover (Konig's theorem).  A covered (a, o) becomes a
# new bond operator "a * o"; a covered rest r becomes the complementary operator
# sum_c c (a * o) over its uncovered edges.  Both are exact, so the MPO represents
# the Hamiltonian exactly; the cover keeps the bond dimension minimal for the cut.

ELEM = {"Ca": _op_matrix("Ca"), "Cb": _op_matrix("Cb"), "Da": _op_matrix("Da"), "Db": _op_matrix("Db")}
ELEM_Q = {"Ca": (1, 1), "Cb": (1, -1), "Da": (-1, -1), "Db": (-1, 1)}


class _SiteOps:
    """Canonical site operators: matrix normalised so its first non-zero is +1."""

    def __init__(self):
        self.mats: List[np.ndarray] = [_op_matrix("I")]
        self.q: List[Tuple[int, int]] = [(0, 0)]
        self.index: Dict[bytes, int] = {self.mats[0].tobytes(): 0}
        self.cache: Dict[Tuple[str, ...], Tuple[int, float]] = {(): (0, 1.0)}

    def get(self, seq: Tuple[str, ...]):
        hit = self.cache.get(seq)
        if hit is not None:
            return hit
        m = np.eye(4)
        q = (0, 0)
        for e in seq:
            m = m @ ELEM[e]
            q = (q[0] + ELEM_Q[e][0], q[1] + ELEM_Q[e][1])
        nz = np.flatnonzero(np.abs(m) > 0)
        if nz.size == 0:
            self.cache[seq] = (-1, 0.0)
            return self.cache[seq]
        scale = float(m.flat[nz[0]])
        mn = m / scale
        key = mn.tobytes()
        idx = self.index.get(key)
        if idx is None:
            idx = len(self.mats)
            self.index[key] = idx
            self.mats.append(mn)
            self.q.append(q)
        self.cache[seq] = (idx, scale)
        return idx, scale


def _site_order(ops):
    """Stable sort of (site, elem) by site with the fermionic sign of the permutation."""
    ops = list(ops)
    sign = 1.0
    # insertion sort counting transpositions of operators on different sites
    for i in range(1, len(ops)):
        j = i
        while j > 0 and ops[j - 1][0] > ops[j][0]:
            ops[j - 1], ops[j] = ops[j], ops[j - 1]
            sign = -sign
            j -= 1
    return ops, sign


def _fuse(ops, sops: _SiteOps):
    """Site-ordered elementary ops -> ((site, siteop), ...) and a scale."""
    out = []
    scale = 1.0
    i = 0
    while i < len(ops):
        s = ops[i][0]
        seq = []
        while i < len(ops) and ops[i][0] == s:
            seq.append(ops[i][1])
            i += 1
        idx, sc = sops.get(tuple(seq))
        if idx < 0:
            return None, 0.0
        scale *= sc
        if idx != 0:
            out.append((s, idx))
    return tuple(out), scale


def _lin_add(acc: Dict[object, float], lin: Optional[Dict[object, float]], f: float = 1.0):
    if lin:
        for par, v in lin.items():
            acc[par] = acc.get(par, 0.0) + f * v


def terms_to_strings(nsite: int, terms, sops: _SiteOps, track: bool = False):
    """[(coef, [(site, elem), ...][, dcoef]), ...] -> {((site, siteop), ...): coef}.
    With ``track`` also {string: {parameter: d(coef)/d(parameter)}} from the terms'
    optional third element {parameter: d(coef)/d(parameter)}."""
    acc: Dict[tuple, float] = {}
    lins: Dict[tuple, Dict[object, float]] = {}
    for term in terms:
        coef, ops = term[0], term[1]
        if coef == 0.0:
            continue
        so, sign = _site_order(ops)
        key, sc = _fuse(so, sops)
        if key is None:
            continue
        acc[key] = acc.get(key, 0.0) + coef * sign * sc
        if track and len(term) > 2:
            _lin_add(lins.setdefault(key, {}), term[2], sign * sc)
    strings = {k: v for k, v in acc.items() if v != 0.0}
    if track:
        return strings, {k: lins[k] for k in strings if k in lins}
    return strings


def _min_vertex_cover(nl: int, nr: int, edges_l: np.ndarray, edges_r: np.ndarray):
    """Minimum vertex cover of a bipartite graph (Konig), returns (left mask, right mask)."""
    import scipy.sparse as sp
    from scipy.sparse.csgraph import maximum_bipartite_matching

    g = sp.csr_matrix((np.ones(edges_l.size, dtype=np.int8), (edges_l, edges_r)), shape=(nl, nr))
    g.sum_duplicates()
    match_r = maximum_bipartite_matching(g, perm_type="column")  # left -> right or -1
    match_l_of_r = np.full(nr, -1, dtype=np.int64)
    for u, v in enumerate(match_r):
        if v >= 0:
            match_l_of_r[v] = u
    indptr, indices = g.indptr, g.indices
    visited_l = np.zeros(nl, dtype=bool)
    visited_r = np.zeros(nr, dtype=bool)
    stack = [u for u in range(nl) if match_r[u] < 0]
    for u in stack:
        visited_l[u] = True
    while stack:
        u = stack.pop()
        for v in indices[indptr[u]:indptr[u + 1]]:
            if visited_r[v] or match_r[u] == v:
                continue
            visited_r[v] = True
            w = match_l_of_r[v]
            if w >= 0 and not visited_l[w]:
                visited_l[w] = True
                stack.append(w)
    return ~visited_l, visited_r


def mpo_from_strings(nsite: int, strings: Dict[tuple, float], sops: _SiteOps,
                     lins: Optional[Dict[tuple, Dict[object, float]]] = None):
    """Exact MPO of sum_s coef_s * prod_k o_{s,k} (site-ordered, fused strings).
    With ``lins`` ({string: {parameter: d(coef)/d(parameter)}}) the parameter
    derivatives are carried through the construction (every coefficient lands in
    exactly one MPO entry, the rest of its path being identity-like 1's) and the
    per-site {block tag: {parameter: derivative}} maps are returned as well."""
    track = lins is not None
    # current terms: (alpha, rest) -> coef, rest = ((site, op), ...) with sites >= k
    cur: Dict[Tuple[int, tuple], float] = {}
    curlin: Dict[Tuple[int, tuple], Dict[object, float]] = {}
    for key, c in strings.items():
        k2 = (0, key)
        cur[k2] = cur.get(k2, 0.0) + c
        if track and key in lins:
            _lin_add(curlin.setdefault(k2, {}), lins[key])
    jacs = []
    q_left = [(0, 0)]
    sites = []
    for k in range(nsite):
        lnodes: Dict[Tuple[int, int], int] = {}
        rnodes: Dict[tuple, int] = {}
        el, er, ec, elin = [], [], [], []
        for (alpha, rest), c in cur.items():
            if rest and rest[0][0] == k:
                o, r = rest[0][1], rest[1:]
            else:
                o, r = 0, rest
            lk = (alpha, o)
            li = lnodes.setdefault(lk, len(lnodes))
            ri = rnodes.setdefault(r, len(rnodes))
            el.append(li)
            er.append(ri)
            ec.append(c)
            if track:
                elin.append(curlin.get((alpha, rest)))
        el = np.asarray(el, dtype=np.int64)
        er = np.asarray(er, dtype=np.int64)
        ec = np.asarray(ec, dtype=np.float64)
        llist = list(lnodes.keys())
        rlist = list(rnodes.keys())
        if k == nsite - 1:
            cover_l = np.zeros(len(llist), dtype=bool)
            cover_r = np.ones(len(rlist), dtype=bool)
        else:
            cover_l, cover_r = _min_vertex_cover(len(llist), len(rlist), el, er)
        # new bond operators: covered left nodes first (in node order), then covered rests
        new_ops: List[Tuple[str, object]] = []
        beta_of_l = {}
        for li in np.flatnonzero(cover_l):
            beta_of_l[int(li)] = len(new_ops)
            new_ops.append(("l", int(li)))
        beta_of_r = {}
        for ri in np.flatnonzero(cover_r):
            beta_of_r[int(ri)] = len(new_ops)
            new_ops.append(("r", int(ri)))
        # charges of new operators
        def lq(li):
            a, o = llist[li]
            qa = q_left[a]
            qo = sops.q[o]
            return (qa[0] + qo[0], qa[1] + qo[1])

        q_new = []
        wentries: Dict[Tuple[int, int, int], float] = {}
        wlin: Dict[Tuple[int, int, int], Dict[object, float]] = {}
        nxt: Dict[Tuple[int, tuple], float] = {}
        nxtlin: Dict[Tuple[int, tuple], Dict[object, float]] = {}
        for kind, idx in new_ops:
            if kind == "l":
                q_new.append(lq(idx))
        # covered rests: charge from any incident edge
        r_charge = {}
        for e in range(el.size):
            li, ri = int(el[e]), int(er[e])
            if li in beta_of_l:
                b = beta_of_l[li]
                a, o = llist[li]
                wentries[(a, o, b)] = 1.0
                key = (b, rlist[ri])
                nxt[key] = nxt.get(key, 0.0) + ec[e]
                if track and elin[e]:
                    _lin_add(nxtlin.setdefault(key, {}), elin[e])
            else:
                b = beta_of_r[ri]
                a, o = llist[li]
                wentries[(a, o, b)] = wentries.get((a, o, b), 0.0) + ec[e]
                if track and elin[e]:
                    _lin_add(wlin.setdefault((a, o, b), {}), elin[e])
                r_charge[ri] = lq(li)
                key = (b, rlist[ri])
                nxt[key] = 1.0
        for kind, idx in new_ops:
            if kind == "r":
                q_new.append(r_charge[idx])
        W = SiteMPO(q_left, q_new)
        for (a, o, b), c in wentries.items():
            if c != 0.0:
                W.add(a, sops.mats[o], b, c, wlin.get((a, o, b)))
        sites.append(W.to_dict())
        if track:
            jacs.append(W.jacobian())
        q_left = q_new
        cur = {}
        curlin = {}
        for (b, r), c in nxt.items():
            if c != 0.0:
                cur[(b, r)] = c
                if track and (b, r) in nxtlin:
                    curlin[(b, r)] = nxtlin[(b, r)]
    if track:
        return sites, jacs
    return sites


def qc_terms(h1: np.ndarray, eri: np.ndarray, ecore: float = 0.0, tol: float = 0.0, track_h: bool = False):
    """H = E0 + sum h_pq a+_ps a_qs + 1/2 sum (pq|rs) a+_ps a+_rt a_st a_qs (chemists' notation).
    With ``track_h`` the one-electron terms carry {("h", p, q): 1} (derivative of
    their coefficient with respect to the matrix element h1[p, q])."""
    n = h1.shape[0]
    C = ("Ca", "Cb")
    D = ("Da", "Db")
    terms = []
    if ecore != 0.0:
        terms.append((ecore, []))
    for p in range(n):
        for q in range(n):
            v = h1[p, q]
            if abs(v) <= tol:
                continue
            for s in range(2):
                if track_h:
                    terms.append((v, [(p, C[s]), (q, D[s])], {("h", p, q): 1.0}))
                else:
                    terms.append((v, [(p, C[s]), (q, D[s])]))
    nz = np.argwhere(np.abs(eri) > tol)
    for p, q, r, s in nz:
        v = 0.5 * eri[p, q, r, s]
        for a in range(2):
            for b in range(2):
                if p == r and a == b:
                    continue
                if s == q and a == b:
                    continue
                terms.append((v, [(p, C[a]), (r, C[b]), (s, D[b]), (q, D[a])]))
    return terms


def qc_mpo(h1: np.ndarray, eri: np.ndarray, ecore: float = 0.0, jacobian: bool = False):
    """Exact quantum-chemistry MPO with spatial-orbital sites.  With ``jacobian``
    also the per-site {block tag: {("h", p, q): d(block)/d(h1[p, q])}} maps."""
    sops = _SiteOps()
    if jacobian:
        strings, lins = terms_to_strings(h1.shape[0], qc_terms(h1, eri, ecore, track_h=True), sops, track=True)
        return mpo_from_strings(h1.shape[0], strings, sops, lins)
    strings = terms_to_strings(h1.shape[0], qc_terms(h1, eri, ecore), sops)
    return mpo_from_strings(h1.shape[0], strings, sops)


def synthetic_qc_integrals(n: int, K: int, seed: int):
    """Synthetic integrals: h_pp ~ U(-3,-0.5) sorted ascending, h_pq ~ N(0,0.1^2) e^{-|p-q|/4}
    symmetrised; (pq|rs) = sum_K L^K_pq L^K_rs with L^K_pq ~ N(0,0.1^2) e^{-|p-q|/4}
    symmetrised and +0.3 on L^p_pp (p < min(n, K)): 8-fold symmetric and PSD."""
    rng = np.random.default_rng(seed)
    idx = np.arange(n)
    decay = np.exp(-np.abs(idx[:, None] - idx[None, :]) / 4.0)
    hd = np.sort(rng.uniform(-3.0, -0.5, size=n))
    off = rng.normal(0.0, 0.1, size=(n, n)) * decay
    h = 0.5 * (off + off.T)
    h[idx, idx] = hd
    Lk = rng.normal(0.0, 0.1, size=(K, n, n)) * decay[None]
    Lk = 0.5 * (Lk + Lk.transpose(0, 2, 1))
    for p in range(min(n, K)):
        Lk[p, p, p] += 0.3
    eri = np.einsum("kpq,krs->pqrs", Lk, Lk)
    return h, eri


def write_fcidump(path: str, h1: np.ndarray, eri: np.ndarray, nelec: int, ms2: int = 0, ecore: float = 0.0,
                  tol: float = 0.0):
    """FCIDUMP writer: the unique 8-fold entries (i >= j, k >= l, ij >= kl, 1-based),
    one-electron entries with k = l = 0 and the core energy on the 0 0 0 0 line."""
    n = h1.shape[0]
    lines = [f" &FCI NORB={n},NELEC={nelec},MS2={ms2},", "  ORBSYM=" + "1," * n, "  ISYM=1,", " &END"]
    for i in range(n):
        for j in range(i + 1):
            ij = i * (i + 1) // 2 + j
            for k in range(n):
                for l in range(k + 1):
                    if k * (k + 1) // 2 + l > ij:
                        continue
                    v = eri[i, j, k, l]
                    if abs(v) > tol:
                        lines.append(f"{v:28.20e} {i + 1:4d} {j + 1:4d} {k + 1:4d} {l + 1:4d}")
    for i in range(n):
        for j in range(i + 1):
            if abs(h1[i, j]) > tol:
                lines.append(f"{h1[i, j]:28.20e} {i + 1:4d} {j + 1:4d} {0:4d} {0:4d}")
    lines.append(f"{ecore:28.20e} {0:4d} {0:4d} {0:4d} {0:4d}")
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def read_fcidump(path: str):
    """FCIDUMP reader: unique integrals unfolded with 8-fold symmetry, core energy from
    the 0 0 0 0 line (same convention as src/parsing_integral.cpp:105-154)."""
    import re

    with open(path) as f:
        txt = f.read()
    head, body = re.split(r"(?:&END|/)\s*\n", txt, maxsplit=1)
    norb = int(re.search(r"NORB\s*=\s*(\d+)", head).group(1))
    nelec = int(re.search(r"NELEC\s*=\s*(\d+)", head).group(1))
    ms2m = re.search(r"MS2\s*=\s*(-?\d+)", head)
    ms2 = int(ms2m.group(1)) if ms2m else 0
    h = np.zeros((norb, norb))
    g = np.zeros((norb, norb, norb, norb))
    e0 = 0.0
    for line in body.splitlines():
        f_ = line.split()
        if len(f_) < 5:
            continue
        v = float(f_[0])
        i, j, k, l = (int(x) for x in f_[1:5])
        if i == 0 and j == 0 and k == 0 and l == 0:
            e0 = v
        elif k == 0 and l == 0:
            h[i - 1, j - 1] = h[j - 1, i - 1] = v
        else:
            i, j, k, l = i - 1, j - 1, k - 1, l - 1
            for a, b, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                               (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)):
                g[a, b, c, d] = v
    return {"norb": norb, "nelec": nelec, "ms2": ms2, "h1": h, "eri": g, "ecore": e0}
