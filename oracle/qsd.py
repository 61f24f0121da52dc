"""CPU oracle: block-sparse quantum-number tensors (test infrastructure only).

This module is a NumPy restatement of the reference's BTAS ``QSTArray`` /
``STArray`` semantics that the two-site DMRG hot path relies on.  It is the
checker for the CUDA path: only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it.  Nothing in the product package
routes through it.

Restated semantics (reference paths are relative to the mpsxx project root):

* quantum number ``fermion(p, s)`` = (particle number, 2*Sz), added
  component-wise, ordered by (p, then s), parity = p odd
  (``src/fermion.h:11-106``);
* a block with sparse index ``(i_0..i_{N-1})`` may be non-zero iff
  ``q_total == sum_k qshape[k][i_k]`` (``include/btas/QSPARSE/QSTArray.h:34-36``);
* blocks are keyed by their row-major tag over the sector counts
  (``include/btas/SPARSE/STArray.h:189-200,338-348``); ``allocate`` creates every
  allowed block of non-zero size (``STArray.h:219-237``);
* ``conjugate`` negates every quantum number (``QSTArray.h:293-300``);
* ``transposed_view(K)`` re-tags blocks ``[i1..iK|iK+1..iN] -> [iK+1..iN|i1..iK]``
  without moving data (``STArray.h:558-577``);
* ``Gemm`` fixes the result quantum shape with ``gemm_contract_qshape``
  (``include/btas/QSPARSE/btas_contract_qshape.h:60-108``), sizes an empty result
  or scales an existing one by beta (``include/btas/QSPARSE/QSTBLAS.h:182-226``),
  and enumerates block tasks with ``ST_Gemm_thread``
  (``include/btas/SPARSE/STBLAS.h:297-359``): for every row block i of the left
  view and column block j of the right view whose result block is allowed, the
  ordered pairs (a_ik, b_jk) with equal contracted tag, each pair a dense
  row-major GEMM accumulated serially into its own result block
  (``include/btas/SPARSE/T_arguments.h:517-600``, ``include/btas/DENSE/TBLAS.h:209-245``).

Parity pins: exact diagonalisation (``tests/test_oracle.py``) and the reference
itself — task lists, bond operations and sweep energies of its own runs
(``tests/test_reference_fixtures.py``, fixtures in ``tests/golden/ref/``).
"""
from __future__ import annotations

import itertools
import math
from typing import Dict, List, Sequence, Tuple

import numpy as np

Q = Tuple[int, int]
ZERO: Q = (0, 0)

NoTrans = "N"
Trans = "T"


def qadd(a: Q, b: Q) -> Q:
    return (a[0] + b[0], a[1] + b[1])


def qneg(a: Q) -> Q:
    return (-a[0], -a[1])


def qparity(a: Q) -> bool:
    return bool(a[0] & 1)


def qsum(qs) -> Q:
    p = 0
    s = 0
    for q in qs:
        p += q[0]
        s += q[1]
    return (p, s)


class QSDArray:
    """Block-sparse tensor: sectors per index, dims per sector, blocks by tag."""

    def __init__(self, q: Q = ZERO, qshape=None, dshape=None):
        self.q: Q = tuple(q)
        self.qshape: List[List[Q]] = [list(map(tuple, x)) for x in (qshape or [])]
        if dshape is None:
            dshape = [[0] * len(x) for x in self.qshape]
        self.dshape: List[List[int]] = [list(map(int, x)) for x in dshape]
        self.blocks: Dict[int, np.ndarray] = {}
        self._update_strides()

    # -- shape bookkeeping -------------------------------------------------
    def _update_strides(self):
        self.shape = tuple(len(x) for x in self.qshape)
        st = [0] * len(self.shape)
        s = 1
        for i in range(len(self.shape) - 1, -1, -1):
            st[i] = s
            s *= self.shape[i]
        self.strides = tuple(st)
        self.nsparse = s if self.shape else 0

    @property
    def rank(self) -> int:
        return len(self.qshape)

    def size(self) -> int:
        """Number of sparse positions (0 for a cleared array)."""
        return self.nsparse if self.rank else 0

    def index(self, tag: int) -> Tuple[int, ...]:
        out = []
        for st in self.strides:
            out.append(tag // st)
            tag %= st
        return tuple(out)

    def tag(self, index: Sequence[int]) -> int:
        return int(sum(i * s for i, s in zip(index, self.strides)))

    def allowed(self, index: Sequence[int]) -> bool:
        return self.q == qsum(self.qshape[k][i] for k, i in enumerate(index))

    def block_dims(self, index: Sequence[int]) -> Tuple[int, ...]:
        return tuple(self.dshape[k][i] for k, i in enumerate(index))

    def copy(self) -> "QSDArray":
        out = QSDArray(self.q, self.qshape, self.dshape)
        out.blocks = {t: b.copy() for t, b in self.blocks.items()}
        return out

    def empty_like(self) -> "QSDArray":
        return QSDArray(self.q, self.qshape, self.dshape)

    def conjugate(self) -> "QSDArray":
        """Reference semantics: shares the blocks, flips every quantum number."""
        out = QSDArray(qneg(self.q), [[qneg(q) for q in x] for x in self.qshape], self.dshape)
        out.blocks = self.blocks
        return out

    def clear(self):
        self.q = ZERO
        self.qshape = []
        self.dshape = []
        self.blocks = {}
        self._update_strides()

    def allocate(self, fill: float = 0.0):
        """Create every allowed block of non-zero size (``STArray.h:219-237``)."""
        self.blocks = {}
        for idx in itertools.product(*[range(n) for n in self.shape]):
            if self.allowed(idx):
                dims = self.block_dims(idx)
                if int(np.prod(dims)) > 0:
                    self.blocks[self.tag(idx)] = np.full(dims, fill, dtype=np.float64)
        return self

    def reserve(self, tag: int) -> np.ndarray:
        blk = self.blocks.get(tag)
        if blk is None:
            idx = self.index(tag)
            if not self.allowed(idx):
                raise RuntimeError("reserve: block not allowed by quantum numbers")
            blk = np.zeros(self.block_dims(idx), dtype=np.float64)
            self.blocks[tag] = blk
        return blk

    def sorted_tags(self) -> List[int]:
        return sorted(self.blocks)

    def nnz(self) -> int:
        return int(sum(b.size for b in self.blocks.values()))

    def check_dshape(self):
        for t, b in self.blocks.items():
            assert b.shape == self.block_dims(self.index(t))


# ----------------------------------------------------------------------------
# Level-1 operations (QSTBLAS.h:57-252, STBLAS.h:94-145,373-453,626-638)
# ----------------------------------------------------------------------------

def dotc(x: QSDArray, y: QSDArray) -> float:
    """Sum over blocks present in both, in map (tag) order."""
    s = 0.0
    for t in sorted(x.blocks):
        yb = y.blocks.get(t)
        if yb is not None:
            s += float(np.dot(x.blocks[t].ravel(), yb.ravel()))
    return s


def nrm2(x: QSDArray) -> float:
    return math.sqrt(sum(float(np.dot(b.ravel(), b.ravel())) for _, b in sorted(x.blocks.items())))


def scal(alpha: float, x: QSDArray):
    for t in x.blocks:
        x.blocks[t] = x.blocks[t] * alpha


def axpy(alpha: float, x: QSDArray, y: QSDArray):
    """y += alpha*x; blocks missing in y are created (``STBLAS.h:431-453``)."""
    if y.size() == 0:
        y.q, y.qshape, y.dshape = x.q, [list(v) for v in x.qshape], [list(v) for v in x.dshape]
        y._update_strides()
    for t, b in x.blocks.items():
        if t in y.blocks:
            y.blocks[t] = y.blocks[t] + alpha * b
        else:
            y.blocks[t] = alpha * b


def copy_into(x: QSDArray, y: QSDArray):
    y.q, y.qshape, y.dshape = x.q, [list(v) for v in x.qshape], [list(v) for v in x.dshape]
    y._update_strides()
    y.blocks = {t: b.copy() for t, b in x.blocks.items()}


def normalize(x: QSDArray):
    scal(1.0 / nrm2(x), x)


def orthogonalize(x: QSDArray, y: QSDArray):
    axpy(-dotc(x, y), x, y)


# ----------------------------------------------------------------------------
# Gemm with the reference's block-task enumeration
# ----------------------------------------------------------------------------

def transposed_view_tags(a: QSDArray, K: int):
    """Tag map of ``transposed_view(K)``: view tag -> original tag (``STArray.h:558-577``)."""
    N = a.rank
    if K == N:
        return {t: t for t in a.blocks}, list(a.shape)
    oldstr = a.strides[K - 1]
    newstr = a.nsparse // oldstr
    out = {}
    for t in a.blocks:
        out[t // oldstr + (t % oldstr) * newstr] = t
    vshape = list(a.shape[K:]) + list(a.shape[:K])
    return out, vshape


def gemm_contract_qshape(transa, transb, a: QSDArray, b: QSDArray, NC: int):
    """``btas_contract_qshape.h:60-108`` for real data (Trans == ConjTrans-free)."""
    NA, NB = a.rank, b.rank
    K = (NA + NB - NC) // 2
    if transa == NoTrans:
        qc = a.q
        cq = a.qshape[: NA - K]
        cd = a.dshape[: NA - K]
        kq = a.qshape[NA - K:]
    else:
        qc = a.q
        cq = a.qshape[K:]
        cd = a.dshape[K:]
        kq = a.qshape[:K]
    if transb == NoTrans:
        qc = qadd(b.q, qc)
        cq = cq + b.qshape[K:]
        cd = cd + b.dshape[K:]
        bk = b.qshape[:K]
    else:
        qc = qadd(b.q, qc)
        cq = cq + b.qshape[: NB - K]
        cd = cd + b.dshape[: NB - K]
        bk = b.qshape[NB - K:]
    for i in range(K):
        if list(kq[i]) != [qneg(q) for q in bk[i]]:
            raise RuntimeError("btas::gemm_contract_qshape contraction of quantum numbers failed")
    return qc, [list(x) for x in cq], [list(x) for x in cd], K


def st_gemm_tasks(transa, transb, a: QSDArray, b: QSDArray, c: QSDArray, K: int):
    """Block-task enumeration of ``ST_Gemm_thread`` (``STBLAS.h:297-359``).

    Returns ``[(c_tag, [(a_tag, b_tag), ...]), ...]`` in enumeration order, the
    tags being those of the original (un-viewed) operands.  The views are the
    ones ``QSTBLAS.h:215-225`` passes for each transpose combination.
    """
    L, M = a.rank, b.rank
    if transa == NoTrans:
        av = {t: t for t in a.blocks}
        ashape = list(a.shape)
    else:
        av, ashape = transposed_view_tags(a, K)
    if transb == NoTrans:
        bv, bshape = transposed_view_tags(b, K)
    else:
        bv = {t: t for t in b.blocks}
        bshape = list(b.shape)
    rowsA = int(np.prod(ashape[: L - K], dtype=np.int64))
    colsA = int(np.prod(ashape[L - K:], dtype=np.int64))
    colsB = int(np.prod(bshape[: M - K], dtype=np.int64))
    a_sorted = sorted(av)
    b_sorted = sorted(bv)
    # group views by row (tag // colsA)
    a_rows: Dict[int, List[int]] = {}
    for t in a_sorted:
        a_rows.setdefault(t // colsA, []).append(t)
    b_rows: Dict[int, List[int]] = {}
    for t in b_sorted:
        b_rows.setdefault(t // colsA, []).append(t)
    tasks = []
    for i in range(rowsA):
        arow = a_rows.get(i)
        if not arow:
            continue
        for j in range(colsB):
            ij = i * colsB + j
            if not c.allowed(c.index(ij)):
                continue
            brow = b_rows.get(j)
            if not brow:
                continue
            pairs = []
            for ta in arow:
                for tb in brow:
                    if ta % colsA == tb % colsA:
                        pairs.append((av[ta], bv[tb]))
            if pairs:
                tasks.append((ij, pairs))
    return tasks


def _as_matrix(blk: np.ndarray, nrow_idx: int, trans: bool) -> np.ndarray:
    rows = int(np.prod(blk.shape[:nrow_idx], dtype=np.int64))
    m = blk.reshape(rows, -1)
    return m.T if trans else m


def gemm(transa, transb, alpha: float, a: QSDArray, b: QSDArray, beta: float, c: QSDArray,
         nc: int = None, return_tasks: bool = False):
    """``btas::Gemm`` for QSDArray (``QSTBLAS.h:182-226``)."""
    if nc is None:
        nc = c.rank if c.size() > 0 else None
    if nc is None:
        raise ValueError("rank of the result must be given for an empty result")
    qc, cq, cd, K = gemm_contract_qshape(transa, transb, a, b, nc)
    if c.size() > 0:
        if c.q != qc:
            raise RuntimeError("Gemm(QSPARSE): quantum number of c must equal to a.q() + b.q().")
        if [list(x) for x in c.qshape] != cq:
            raise RuntimeError("Gemm(QSPARSE): c must have the same quantum shape of [ a * b ].")
        scal(beta, c)
    else:
        c.q = qc
        c.qshape = cq
        c.dshape = cd
        c._update_strides()
        c.blocks = {}
    tasks = st_gemm_tasks(transa, transb, a, b, c, K)
    L, M = a.rank, b.rank
    for ctag, pairs in tasks:
        cidx = c.index(ctag)
        cdims = c.block_dims(cidx)
        cblk = c.reserve(ctag)
        nrow_c = L - K
        cm = cblk.reshape(int(np.prod(cdims[:nrow_c], dtype=np.int64)), -1)
        for ta, tb in pairs:
            ablk = a.blocks[ta]
            bblk = b.blocks[tb]
            if ablk.size == 0 or bblk.size == 0:
                continue
            am = _as_matrix(ablk, L - K if transa == NoTrans else K, transa != NoTrans)
            bm = _as_matrix(bblk, K if transb == NoTrans else M - K, transb != NoTrans)
            cm += alpha * (am @ bm)
        c.blocks[ctag] = cm.reshape(cdims)
    if return_tasks:
        return tasks
    return None


# ----------------------------------------------------------------------------
# Generic labelled contraction (used off the hot Gemm path: MPO contractions)
# ----------------------------------------------------------------------------

def contract(a: QSDArray, a_lab: Sequence, b: QSDArray, b_lab: Sequence, c_lab: Sequence,
             alpha: float = 1.0, c: QSDArray = None) -> QSDArray:
    """c[c_lab] += alpha * sum a[a_lab] b[b_lab] over shared labels.

    Same algebra as ``btas::Contract`` (``include/btas/QSPARSE/QSTCONTRACT.h:15-89``):
    contracted indices must carry opposite quantum numbers; the result's total
    quantum number is ``a.q + b.q``.
    """
    a_lab = list(a_lab)
    b_lab = list(b_lab)
    c_lab = list(c_lab)
    shared = [l for l in a_lab if l in b_lab]
    for l in shared:
        qa = a.qshape[a_lab.index(l)]
        qb = b.qshape[b_lab.index(l)]
        if list(qa) != [qneg(q) for q in qb]:
            raise RuntimeError("contract: contracted quantum numbers must be opposite")
    cq, cd = [], []
    for l in c_lab:
        if l in a_lab:
            k = a_lab.index(l)
            cq.append(list(a.qshape[k]))
            cd.append(list(a.dshape[k]))
        else:
            k = b_lab.index(l)
            cq.append(list(b.qshape[k]))
            cd.append(list(b.dshape[k]))
    qc = qadd(a.q, b.q)
    if c is None or c.size() == 0:
        c = QSDArray(qc, cq, cd)
    else:
        assert c.q == qc
    sa = [a_lab.index(l) for l in shared]
    sb = [b_lab.index(l) for l in shared]
    # bucket b blocks by contracted sector index
    bbuck: Dict[Tuple[int, ...], List[Tuple[Tuple[int, ...], np.ndarray]]] = {}
    for tb in sorted(b.blocks):
        ib = b.index(tb)
        bbuck.setdefault(tuple(ib[k] for k in sb), []).append((ib, b.blocks[tb]))
    letters = "abcdefghijklmnopqrstuvwxyz"
    lab2chr = {}
    for l in a_lab + b_lab:
        if l not in lab2chr:
            lab2chr[l] = letters[len(lab2chr)]
    spec = "".join(lab2chr[l] for l in a_lab) + "," + "".join(lab2chr[l] for l in b_lab) + "->" + \
        "".join(lab2chr[l] for l in c_lab)
    for ta in sorted(a.blocks):
        ia = a.index(ta)
        key = tuple(ia[k] for k in sa)
        for ib, bblk in bbuck.get(key, []):
            cidx = []
            for l in c_lab:
                if l in a_lab:
                    cidx.append(ia[a_lab.index(l)])
                else:
                    cidx.append(ib[b_lab.index(l)])
            if not c.allowed(cidx):
                continue
            val = np.einsum(spec, a.blocks[ta], bblk)
            ct = c.tag(cidx)
            if ct in c.blocks:
                c.blocks[ct] = c.blocks[ct] + alpha * val
            else:
                c.blocks[ct] = alpha * val
    return c


# ----------------------------------------------------------------------------
# Merge / expand of index groups (QSTmergeInfo.h:44-90, QSTmerge.h:31-450)
# ----------------------------------------------------------------------------

class MergeInfo:
    """Packed product of index sectors, merged by quantum number.

    Merged sector numbering follows first appearance in packed order; packed
    sub-blocks are stacked in packed order (``QSTmergeInfo.h:44-90``).
    """

    def __init__(self, qshapes: Sequence[Sequence[Q]], dshapes: Sequence[Sequence[int]]):
        self.qshape = [list(map(tuple, q)) for q in qshapes]
        self.dshape = [list(map(int, d)) for d in dshapes]
        qp: List[Q] = [ZERO]
        dp: List[int] = [1]
        for q, d in zip(self.qshape, self.dshape):
            qp = [qadd(x, y) for x in qp for y in q]
            dp = [x * y for x in dp for y in d]
        self.q_packed = qp
        self.d_packed = dp
        order: Dict[Q, int] = {}
        for q in qp:
            if q not in order:
                order[q] = len(order)
        self.q_merged: List[Q] = [None] * len(order)
        for q, i in order.items():
            self.q_merged[i] = q
        self.members: List[List[int]] = [[] for _ in order]
        self.d_merged = [0] * len(order)
        self.offset_packed = [0] * len(qp)
        self.merged_of = [0] * len(qp)
        for i, q in enumerate(qp):
            j = order[q]
            self.offset_packed[i] = self.d_merged[j]
            self.merged_of[i] = j
            self.members[j].append(i)
            self.d_merged[j] += dp[i]

    def packed_to_multi(self, ip: int) -> Tuple[int, ...]:
        out = []
        for q in reversed(self.qshape):
            out.append(ip % len(q))
            ip //= len(q)
        return tuple(reversed(out))


def merge_rows(info: MergeInfo, a: QSDArray) -> QSDArray:
    """Row merge ``A(i,j,k,l) -> B(r,k,l)`` (``QSTmerge.h:31-83``)."""
    MR = len(info.qshape)
    b = QSDArray(a.q, [info.q_merged] + a.qshape[MR:], [info.d_merged] + a.dshape[MR:])
    a_stride = a.strides[MR - 1]
    b_stride = b.strides[0] if b.rank > 1 else 1
    for i in range(b.shape[0]):
        if not info.members[i]:
            continue
        for j in range(b_stride):
            bidx = b.index(i * b_stride + j)
            if not b.allowed(bidx):
                continue
            dims = b.block_dims(bidx)
            blk = np.zeros(dims)
            nz = False
            for ip in info.members[i]:
                src = a.blocks.get(ip * a_stride + j)
                if src is not None:
                    nz = True
                    o = info.offset_packed[ip]
                    d = info.d_packed[ip]
                    blk[o:o + d] = src.reshape((d,) + tuple(dims[1:]))
            if nz:
                b.blocks[b.tag(bidx)] = blk
    return b


def merge_cols(a: QSDArray, info: MergeInfo) -> QSDArray:
    """Column merge ``A(i,j,k,l) -> B(i,j,c)`` (``QSTmerge.h:85-140``)."""
    MC = len(info.qshape)
    MR = a.rank - MC
    b = QSDArray(a.q, a.qshape[:MR] + [info.q_merged], a.dshape[:MR] + [info.d_merged])
    a_stride = a.strides[MR - 1]
    b_stride = b.strides[MR - 1]
    nrows = b.nsparse // b_stride
    for i in range(nrows):
        for j in range(b_stride):
            if not info.members[j]:
                continue
            bidx = b.index(i * b_stride + j)
            if not b.allowed(bidx):
                continue
            dims = b.block_dims(bidx)
            blk = np.zeros(dims)
            nz = False
            for ip in info.members[j]:
                src = a.blocks.get(i * a_stride + ip)
                if src is not None:
                    nz = True
                    o = info.offset_packed[ip]
                    d = info.d_packed[ip]
                    blk[..., o:o + d] = src.reshape(tuple(dims[:-1]) + (d,))
            if nz:
                b.blocks[b.tag(bidx)] = blk
    return b


def expand_rows(info: MergeInfo, b: QSDArray) -> QSDArray:
    """Inverse of ``merge_rows`` (``QSTexpand``, ``QSTmerge.h:300-450``)."""
    MR = len(info.qshape)
    a = QSDArray(b.q, info.qshape + b.qshape[1:], info.dshape + b.dshape[1:])
    b_stride = b.strides[0] if b.rank > 1 else 1
    a_stride = a.strides[MR - 1]
    for tb in sorted(b.blocks):
        i, j = tb // b_stride, tb % b_stride
        blk = b.blocks[tb]
        for ip in info.members[i]:
            d = info.d_packed[ip]
            if d == 0:
                continue
            aidx = a.index(ip * a_stride + j)
            if not a.allowed(aidx):
                continue
            o = info.offset_packed[ip]
            a.blocks[a.tag(aidx)] = blk[o:o + d].reshape(a.block_dims(aidx)).copy()
    return a


def expand_cols(b: QSDArray, info: MergeInfo) -> QSDArray:
    MC = len(info.qshape)
    MR = b.rank - 1
    a = QSDArray(b.q, b.qshape[:MR] + info.qshape, b.dshape[:MR] + info.dshape)
    b_stride = b.strides[MR - 1]
    a_stride = a.strides[MR - 1]
    for tb in sorted(b.blocks):
        i, j = tb // b_stride, tb % b_stride
        blk = b.blocks[tb]
        for ip in info.members[j]:
            d = info.d_packed[ip]
            if d == 0:
                continue
            aidx = a.index(i * a_stride + ip)
            if not a.allowed(aidx):
                continue
            o = info.offset_packed[ip]
            a.blocks[a.tag(aidx)] = blk[..., o:o + d].reshape(a.block_dims(aidx)).copy()
    return a


# ----------------------------------------------------------------------------
# Tie (diagonal extraction) and Dimm (SPARSE/STREINDEX.h:95-147, STBLAS.h:581-624)
# ----------------------------------------------------------------------------

def tie_02(x: QSDArray):
    """``Tie(x, shape(0,2))`` on a 3-index operator: y[A,w] = x[A,w,A].

    Returns a plain block map {(iA, iw): ndarray(dA, dw)} keyed by sparse index
    (the reference result is an un-quantised STArray).
    """
    out = {}
    for t in sorted(x.blocks):
        i, w, j = x.index(t)
        if i != j:
            continue
        blk = x.blocks[t]
        out[(i, w)] = np.einsum("awa->aw", blk)
    return out


def dimm_rows(s_blocks: Dict[int, np.ndarray], b: QSDArray):
    """(diagonal) x (matrix): scale rows of each block by s of its row sector."""
    n = b.nsparse // b.shape[0]
    for t in b.blocks:
        sv = s_blocks.get(t // n)
        if sv is not None:
            b.blocks[t] = b.blocks[t] * sv[:, None]


def dimm_cols(a: QSDArray, s_blocks: Dict[int, np.ndarray]):
    """(matrix) x (diagonal): scale columns of each block by s of its column sector."""
    n = a.shape[-1]
    for t in a.blocks:
        sv = s_blocks.get(t % n)
        if sv is not None:
            a.blocks[t] = a.blocks[t] * sv[None, :]
