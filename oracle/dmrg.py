"""CPU oracle: the reference's merged two-site DMRG path, restated in NumPy.

Test infrastructure only (imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``).  Each function cites the reference
file:line it follows (paths relative to the mpsxx project root).  Single root
(``nroots = 1``): the Davidson functor then applies no projections
(``src/diagonalize.hpp:217-233``).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .qsd import (NoTrans, Trans, ZERO, MergeInfo, QSDArray, axpy, contract, copy_into, dimm_cols,
                  dimm_rows, dotc, expand_cols, expand_rows, gemm, merge_cols, merge_rows, normalize,
                  nrm2, orthogonalize, qadd, qneg, scal, tie_02)

# relative window inside which singular values count as ties of the cutoff
SVD_TIE_RTOL = 1e-10


# ----------------------------------------------------------------------------
# a6: sigma vector (src/compute_sigma_vector.hpp:85-96)
# ----------------------------------------------------------------------------

def compute_sigma_vector(lopr: QSDArray, ropr: QSDArray, wfn0: QSDArray, sgv0: QSDArray,
                         tasks: Optional[list] = None):
    """sgv0 += sum_{w,A',B'} L[A,w,A'] psi[A',B'] R[B,w,B'] (two Gemm's)."""
    scr1 = QSDArray()
    t1 = gemm(NoTrans, NoTrans, 1.0, lopr, wfn0, 1.0, scr1, nc=3, return_tasks=True)
    t2 = gemm(NoTrans, Trans, 1.0, scr1, ropr, 1.0, sgv0, nc=2, return_tasks=True)
    if tasks is not None:
        tasks.append(("LxPsi", t1))
        tasks.append(("ScrxRt", t2))
    return scr1


def compute_sigma_vector_onesite(mpo0: QSDArray, lopr: QSDArray, ropr: QSDArray, wfn0: QSDArray,
                                 sgv0: QSDArray) -> QSDArray:
    """One-site sigma with the site MPO (``src/compute_sigma_vector.hpp:9-22``):
    scr1 = Gemm(lopr, wfn0); scr2 = Contract(scr1 (1,2), mpo0 (0,2));
    sgv0 += Contract(scr2 (3,1), ropr (1,2))."""
    scr1 = QSDArray()
    gemm(NoTrans, NoTrans, 1.0, lopr, wfn0, 1.0, scr1, nc=4)
    scr2 = contract(scr1, "awnr", mpo0, "wmnv", "armv")
    return contract(scr2, "armv", ropr, "svr", "ams", c=sgv0)


def compute_sigma_vector_twosite(lmpo: QSDArray, rmpo: QSDArray, lopr: QSDArray, ropr: QSDArray, wfn0: QSDArray,
                                 sgv0: QSDArray) -> QSDArray:
    """Four-index two-site sigma (``src/compute_sigma_vector.hpp:53-70``): four
    Contracts, lopr (2)-wfn0 (0), lmpo (0,2), rmpo (0,2), ropr (1,2)."""
    scr1 = contract(lopr, "awk", wfn0, "knpr", "awnpr")
    scr2 = contract(scr1, "awnpr", lmpo, "wmnv", "aprmv")
    scr3 = contract(scr2, "aprmv", rmpo, "vqpx", "armqx")
    return contract(scr3, "armqx", ropr, "sxr", "amqs", c=sgv0)


def compute_sigma_vector_overlap(lopr: QSDArray, ropr: QSDArray, wfn0: QSDArray, sgv0: QSDArray) -> QSDArray:
    """sgv0 += lopr wfn0 ropr^T with two-index (S) operators, wfn0 of 2 to 4 indices
    (``src/compute_sigma_vector.hpp:24-35, 72-83, 98-109``): two Gemms."""
    scr1 = QSDArray()
    gemm(NoTrans, NoTrans, 1.0, lopr, wfn0, 1.0, scr1, nc=wfn0.rank)
    gemm(NoTrans, Trans, 1.0, scr1, ropr, 1.0, sgv0, nc=wfn0.rank)
    return sgv0


# ----------------------------------------------------------------------------
# a9: renormalize merged operator / overlap (src/renormalize.hpp:57-95)
# ----------------------------------------------------------------------------

def renormalize_mpo(forward: bool, mpo0: QSDArray, opr0: QSDArray, bra0: QSDArray, ket0: QSDArray) -> QSDArray:
    """renormalize with the site MPO (``src/renormalize.hpp:10-32``): three Contracts
    (also used to build the initial environments)."""
    b = bra0.conjugate()
    if forward:
        scr1 = contract(opr0, "lwk", b, "lna", "wkna")
        scr2 = contract(scr1, "wkna", mpo0, "wnmv", "kamv")
        return contract(scr2, "kamv", ket0, "kmb", "avb")
    scr1 = contract(b, "anr", opr0, "rvs", "anvs")
    scr2 = contract(scr1, "anvs", mpo0, "wnmv", "aswm")
    return contract(scr2, "aswm", ket0, "bms", "awb")


def compute_guesswave(forward: bool, mps0: QSDArray, wfn0: QSDArray, mps1: QSDArray, wfn1: QSDArray) -> QSDArray:
    """compute_guesswave (``src/compute_guesswave.hpp:11-38``): two Gemms into wfn1.  The
    reference's ConjTrans operand is the Trans of its conjugate for real data (the
    q-shape rule of ``include/btas/QSPARSE/btas_contract_qshape.h:76-79, 94-100`` negates
    the quantum numbers; the dense layer treats ConjTrans of doubles as Trans)."""
    gmat = QSDArray()
    if forward:  # C(i+1) = L(i)^+ C(i) R(i+1)
        gemm(Trans, NoTrans, 1.0, mps0.conjugate(), wfn0, 1.0, gmat, nc=2)
        gemm(NoTrans, NoTrans, 1.0, gmat, mps1, 1.0, wfn1, nc=3)
    else:  # C(i) = L(i) C(i+1) R(i+1)^+
        gemm(NoTrans, Trans, 1.0, wfn0, mps0.conjugate(), 1.0, gmat, nc=2)
        gemm(NoTrans, NoTrans, 1.0, mps1, gmat, 1.0, wfn1, nc=3)
    return wfn1


def renormalize_overlap(forward: bool, sov0: QSDArray, bra0: QSDArray, ket0: QSDArray) -> QSDArray:
    """renormalize an overlap matrix (``src/renormalize.hpp:35-54``): two Gemms."""
    scr1, sov1 = QSDArray(), QSDArray()
    if forward:
        gemm(Trans, NoTrans, 1.0, sov0, bra0.conjugate(), 1.0, scr1, nc=3)
        gemm(Trans, NoTrans, 1.0, scr1, ket0, 1.0, sov1, nc=2)
    else:
        gemm(NoTrans, NoTrans, 1.0, bra0.conjugate(), sov0, 1.0, scr1, nc=3)
        gemm(NoTrans, Trans, 1.0, scr1, ket0, 1.0, sov1, nc=2)
    return sov1


def renormalize_merged(forward: bool, opr0: QSDArray, bra0: QSDArray, ket0: QSDArray,
                       tasks: Optional[list] = None) -> QSDArray:
    opr1 = QSDArray()
    scr1 = QSDArray()
    if forward:
        t1 = gemm(Trans, NoTrans, 1.0, bra0.conjugate(), opr0, 1.0, scr1, nc=3, return_tasks=True)
        t2 = gemm(NoTrans, NoTrans, 1.0, scr1, ket0, 1.0, opr1, nc=3, return_tasks=True)
    else:
        t1 = gemm(NoTrans, NoTrans, 1.0, bra0.conjugate(), opr0, 1.0, scr1, nc=3, return_tasks=True)
        t2 = gemm(NoTrans, Trans, 1.0, scr1, ket0, 1.0, opr1, nc=3, return_tasks=True)
    if tasks is not None:
        tasks.append(("BraxOp", t1))
        tasks.append(("ScrxKet", t2))
    return opr1


# ----------------------------------------------------------------------------
# a5: diagonal of H_eff (src/compute_diagonal_elements.hpp:65-80)
# ----------------------------------------------------------------------------

def compute_diagonal_elements(lopr: QSDArray, ropr: QSDArray, diag: QSDArray):
    """diag[A,B] += sum_w L[A,w,A] R[B,w,B] on the blocks diag's quantum numbers allow."""
    ld = tie_02(lopr)
    rd = tie_02(ropr)
    # Gemm(NoTrans, Trans) over the un-quantised tied arrays: c(i,j) = sum_w a(i,w) b(j,w)
    scr: Dict[tuple, np.ndarray] = {}
    rbyw: Dict[int, list] = {}
    for (j, w), blk in sorted(rd.items()):
        rbyw.setdefault(w, []).append((j, blk))
    for (i, w), ablk in sorted(ld.items()):
        for j, bblk in rbyw.get(w, []):
            v = ablk @ bblk.T
            if (i, j) in scr:
                scr[(i, j)] = scr[(i, j)] + v
            else:
                scr[(i, j)] = v
    # Copy(scr, diag, 1): keep blocks allowed by diag's quantum numbers
    for (i, j), blk in scr.items():
        if diag.allowed((i, j)):
            t = diag.tag((i, j))
            if t in diag.blocks:
                diag.blocks[t] = diag.blocks[t] + blk
            else:
                diag.blocks[t] = blk.copy()


def _tie_mpo(mpo: QSDArray) -> Dict[tuple, np.ndarray]:
    """``Tie(mpo, shape(1,2))``: y[w,n,w'] = mpo[w,n,n,w'] as an un-quantised block map."""
    out = {}
    for t in sorted(mpo.blocks):
        w, n, m, v = mpo.index(t)
        if n == m:
            out[(w, n, v)] = np.einsum("wnnv->wnv", mpo.blocks[t])
    return out


def _copy_allowed(scr: Dict[tuple, np.ndarray], diag: QSDArray):
    """``Copy(scr, diag, 1)`` (``src/compute_diagonal_elements.hpp:31,58``;
    ``include/btas/SPARSE/STBLAS.h:374-388``): diag is resized to scr's shape, which
    drops every block it held, then takes the blocks of scr its quantum numbers allow."""
    diag.blocks = {}
    for idx, blk in scr.items():
        if diag.allowed(idx):
            diag.blocks[diag.tag(idx)] = blk.copy()


def compute_diagonal_elements_onesite(mpo0: QSDArray, lopr: QSDArray, ropr: QSDArray, diag: QSDArray):
    """One-site diagonal (``src/compute_diagonal_elements.hpp:10-32``): Tie the MPO over
    (1,2) and the operators over (0,2), then diag[l,n,r] = sum Ld[l,w] Wd[w,n,w'] Rd[r,w']."""
    ld, rd, wd = tie_02(lopr), tie_02(ropr), _tie_mpo(mpo0)
    scr: Dict[tuple, np.ndarray] = {}
    for (l, w), a in sorted(ld.items()):
        for (w2, n, v), b in sorted(wd.items()):
            if w2 != w:
                continue
            for (r, v2), c in sorted(rd.items()):
                if v2 != v:
                    continue
                val = np.einsum("lw,wnv,rv->lnr", a, b, c)
                k = (l, n, r)
                scr[k] = scr[k] + val if k in scr else val
    _copy_allowed(scr, diag)


def compute_diagonal_elements_twosite(lmpo: QSDArray, rmpo: QSDArray, lopr: QSDArray, ropr: QSDArray,
                                      diag: QSDArray):
    """Four-index two-site diagonal (``src/compute_diagonal_elements.hpp:35-62``):
    diag[l,n,m,r] = sum Ld[l,w] Wl[w,n,v] Wr[v,m,x] Rd[r,x]."""
    ld, rd, wl, wr = tie_02(lopr), tie_02(ropr), _tie_mpo(lmpo), _tie_mpo(rmpo)
    scr: Dict[tuple, np.ndarray] = {}
    for (l, w), a in sorted(ld.items()):
        for (w2, n, v), b in sorted(wl.items()):
            if w2 != w:
                continue
            for (v2, m, x), c in sorted(wr.items()):
                if v2 != v:
                    continue
                for (r, x2), d in sorted(rd.items()):
                    if x2 != x:
                        continue
                    val = np.einsum("lw,wnv,vmx,rx->lnmr", a, b, c, d)
                    k = (l, n, m, r)
                    scr[k] = scr[k] + val if k in scr else val
    _copy_allowed(scr, diag)


# ----------------------------------------------------------------------------
# a7: Davidson (src/diagonalize.hpp:283-449), single root
# ----------------------------------------------------------------------------

@dataclass
class DavidsonStats:
    n_sigma: int = 0
    macro: int = 0
    micro: int = 0
    rnorm: float = 0.0
    converged: bool = False


def precondition(eval_: float, diag: QSDArray, errv: QSDArray):
    """(E - diag)^-1 with |.| floored at 1e-8; 1/E where diag has no block (``:283-304``)."""
    for t in errv.blocks:
        d = diag.blocks.get(t)
        if d is not None:
            denm = eval_ - d
            denm = np.where(np.abs(denm) < 1.0e-8, 1.0e-8, denm)
            errv.blocks[t] = errv.blocks[t] / denm
        else:
            errv.blocks[t] = errv.blocks[t] * (1.0 / eval_)


def davidson(multH, diag: QSDArray, wfnc: QSDArray, tolerance: float = 1.0e-8,
             stats: Optional[DavidsonStats] = None) -> float:
    """``Davidson::diagonalize`` (``src/diagonalize.hpp:310-449``)."""
    max_ritz = 10
    eval_ = 0.0
    trial = [QSDArray() for _ in range(max_ritz)]
    sigma = [QSDArray() for _ in range(max_ritz)]
    copy_into(wfnc, trial[0])
    niter = 0
    iconv = 0
    st = stats if stats is not None else DavidsonStats()
    while iconv < 1 and niter < 4:
        normalize(trial[0])
        sigma[0] = QSDArray()
        multH(trial[0], sigma[0])
        st.n_sigma += 1
        for m in range(1, max_ritz + 1):
            heff = np.zeros((m, m))
            for i in range(m):
                heff[i, i] = dotc(trial[i], sigma[i])
                for j in range(i):
                    hij = dotc(trial[i], sigma[j])
                    heff[i, j] = hij
                    heff[j, i] = hij
            rval, rvec = np.linalg.eigh(heff)
            eval_ = float(rval[0])
            st.micro += 1
            trial_save = [t.copy() for t in trial[:m]]
            sigma_save = [s.copy() for s in sigma[:m]]
            for i in range(m):
                scal(rvec[i, i], trial[i])
                scal(rvec[i, i], sigma[i])
            for i in range(m):
                for j in range(m):
                    if i != j:
                        axpy(rvec[i, j], trial_save[i], trial[j])
                        axpy(rvec[i, j], sigma_save[i], sigma[j])
            errv = sigma[0].copy()
            axpy(-eval_, trial[0], errv)
            rnorm = dotc(errv, errv)
            st.rnorm = rnorm
            if rnorm < tolerance:
                iconv += 1
                break
            if m < max_ritz:
                precondition(eval_, diag, errv)
                for i in range(m):
                    normalize(errv)
                    orthogonalize(trial[i], errv)
                normalize(errv)
                trial[m] = errv.copy()
                sigma[m] = QSDArray()
                multH(trial[m], sigma[m])
                st.n_sigma += 1
        niter += 1
    st.macro = niter
    st.converged = iconv > 0
    copy_into(trial[0], wfnc)
    normalize(wfnc)  # Functor<2>::orthonormalize with no lower roots
    return eval_


# ----------------------------------------------------------------------------
# a8: truncated SVD + canonicalize (include/btas/QSPARSE/QSTLAPACK.h:121-288,
#     src/canonicalize.hpp:48-106)
# ----------------------------------------------------------------------------

def select_kept(svals: Dict[int, np.ndarray], M: int, tie_rtol: float = SVD_TIE_RTOL):
    """Global top-M selection (``QSTLAPACK.h:204-232``).

    cutoff = s_sorted[M-1] when 0 < M < #s, else 1e-16; a sector keeps its
    leading values >= cutoff.  Values within ``tie_rtol`` (relative) below the
    cutoff count as ties and are kept: degenerate spin-flip sectors otherwise
    split on last-bit rounding.
    """
    allv = np.concatenate([v for _, v in sorted(svals.items())]) if svals else np.zeros(0)
    s_sorted = np.sort(allv)[::-1]
    cutoff = 1.0e-16
    if 0 < M < s_sorted.size:
        cutoff = float(s_sorted[M - 1]) * (1.0 - tie_rtol)
    kept = {}
    dnorm = 0.0
    for sec, v in sorted(svals.items()):
        n = int(np.sum(v >= cutoff))
        # values come sorted descending; keep the prefix
        kept[sec] = n
        dnorm += float(np.sum(v[n:] ** 2))
    return kept, dnorm


def gesvd_merged(a: QSDArray, M: int, left_arrow: bool, tie_rtol: float = SVD_TIE_RTOL):
    """Truncated SVD of a 2-index merged array (``QSTLAPACK.h:121-288``).

    Returns (s_blocks by new-bond sector, U [rows, s], Vt [s, cols], kept map).
    LeftArrow: U carries zero quantum number, s sectors = row sectors.
    RightArrow: Vt carries zero quantum number, s sectors = column sectors.
    """
    q_rows = a.qshape[0]
    q_cols = a.qshape[1]
    ncols = a.shape[1]
    svals: Dict[int, np.ndarray] = {}
    uvs: Dict[int, tuple] = {}
    for t in sorted(a.blocks):
        blk = a.blocks[t]
        if blk.size == 0:
            continue
        i, j = t // ncols, t % ncols
        u, s, vt = np.linalg.svd(blk, full_matrices=False)
        sec = i if left_arrow else j
        svals[sec] = s
        uvs[sec] = (i, j, u, vt)
    kept, dnorm = select_kept(svals, M, tie_rtol)
    q_sval = q_rows if left_arrow else [qneg(q) for q in q_cols]
    secs = [sec for sec in sorted(svals) if kept[sec] > 0]
    q_nz = [q_sval[sec] for sec in secs]
    d_nz = [kept[sec] for sec in secs]
    newidx = {sec: n for n, sec in enumerate(secs)}
    if left_arrow:
        U = QSDArray(ZERO, [q_rows, [qneg(q) for q in q_nz]], [a.dshape[0], d_nz])
        V = QSDArray(a.q, [q_nz, q_cols], [d_nz, a.dshape[1]])
    else:
        U = QSDArray(a.q, [q_rows, [qneg(q) for q in q_nz]], [a.dshape[0], d_nz])
        V = QSDArray(ZERO, [q_nz, q_cols], [d_nz, a.dshape[1]])
    s_out = {}
    for sec in secs:
        i, j, u, vt = uvs[sec]
        k = kept[sec]
        n = newidx[sec]
        s_out[n] = svals[sec][:k].copy()
        U.blocks[U.tag((i, n))] = u[:, :k].copy()
        V.blocks[V.tag((n, j))] = vt[:k, :].copy()
    return s_out, U, V, kept, dnorm


# ----------------------------------------------------------------------------
# a8: make_noise (src/canonicalize.hpp:11-24)
# ----------------------------------------------------------------------------

MT_N, MT_M = 624, 397
MT_MATRIX_A = 0x9908B0DF
MT_UPPER, MT_LOWER = 0x80000000, 0x7FFFFFFF
MT_DEFAULT_SEED = 5489  # seed of a default-constructed std::mt19937


def _mt_twist(mt: np.ndarray) -> None:
    """One regeneration of the 624-word state, in place, in the three stretches
    whose far word (i + 397 mod 624) is already regenerated or not."""
    def step(cur, nxt, far):
        y = (cur & MT_UPPER) | (nxt & MT_LOWER)
        return far ^ (y >> np.uint64(1)) ^ np.where((y & np.uint64(1)) != 0, np.uint64(MT_MATRIX_A), np.uint64(0))

    a = MT_N - MT_M  # 227
    mt[0:a] = step(mt[0:a], mt[1:a + 1], mt[MT_M:MT_N])
    mt[a:2 * a] = step(mt[a:2 * a], mt[a + 1:2 * a + 1], mt[0:a])
    mt[2 * a:MT_N - 1] = step(mt[2 * a:MT_N - 1], mt[2 * a + 1:MT_N], mt[a:MT_N - 1 - a])
    mt[MT_N - 1:] = step(mt[MT_N - 1:], mt[0:1], mt[MT_M - 1:MT_M])


def mt19937_words(count: int, seed: int = MT_DEFAULT_SEED) -> np.ndarray:
    """The first ``count`` 32-bit outputs of MT19937 (Matsumoto and Nishimura, ACM
    TOMACS 8(1), 1998: initialisation by x[i] = 1812433253 (x[i-1] ^ (x[i-1] >> 30)) + i,
    the twist and the tempering of that paper; the C++ standard defines std::mt19937
    with the same parameters).  The reference draws from a default-constructed engine
    (``src/canonicalize.hpp:16``)."""
    mask = 0xFFFFFFFF
    mt = np.zeros(MT_N, dtype=np.uint64)
    mt[0] = seed & mask
    for i in range(1, MT_N):
        p = int(mt[i - 1])
        mt[i] = (1812433253 * (p ^ (p >> 30)) + i) & mask
    out = np.empty(count, dtype=np.uint64)
    pos = 0
    while pos < count:
        _mt_twist(mt)
        y = mt.copy()
        y ^= y >> np.uint64(11)
        y ^= (y << np.uint64(7)) & np.uint64(0x9D2C5680)
        y ^= (y << np.uint64(15)) & np.uint64(0xEFC60000)
        y ^= y >> np.uint64(18)
        take = min(MT_N, count - pos)
        out[pos:pos + take] = y[:take] & np.uint64(mask)
        pos += take
    return out


def noise_sequence(n: int) -> np.ndarray:
    """The first n values of ``uniform_real_distribution<double>(-1, 1)`` over a
    default-seeded mt19937 (``src/canonicalize.hpp:16-17``): generate_canonical<double,
    53> takes two 32-bit words per value, r = (w0 + w1 2^32) / 2^64 with the sum rounded
    to double (C++ standard [rand.util.canonical]; libstdc++ returns the largest double
    below 1 when r rounds to 1), and the distribution returns r (b - a) + a."""
    w = mt19937_words(2 * int(n)).astype(np.float64)
    s = w[0::2] + w[1::2] * 4294967296.0
    r = s / 18446744073709551616.0
    r = np.where(r >= 1.0, np.nextafter(1.0, 0.0), r)
    return r * 2.0 + (-1.0)


def make_noise(wfnc: QSDArray, noise: float) -> None:
    """``make_noise`` (``src/canonicalize.hpp:11-24``), in place: wfnc += noise * wfpt.
    wfpt holds every allowed block of non-zero size under the net dense shape of wfnc
    (``check_net_dshape``, ``include/btas/SPARSE/STArray.h:386-401``; ``allocate``,
    ``:219-237``).  STArray::generate passes the generator to each block by value
    (``STArray.h:259-262``), so every block is filled, row-major, with the leading values
    of the same sequence; Axpy adds the blocks wfnc lacks (``SPARSE/STBLAS.h:133-145``)."""
    if noise < 1.0e-8:
        return
    net = [[0] * len(x) for x in wfnc.qshape]
    for t, b in wfnc.blocks.items():
        for k, i in enumerate(wfnc.index(t)):
            net[k][i] = b.shape[k]
    wfpt = QSDArray(wfnc.q, wfnc.qshape, net)
    tags = []
    for t in range(wfpt.nsparse):
        idx = wfpt.index(t)
        dims = wfpt.block_dims(idx)
        if wfpt.allowed(idx) and int(np.prod(dims)) > 0:
            tags.append((t, dims))
    nmax = max((int(np.prod(d)) for _, d in tags), default=0)
    seq = noise_sequence(nmax)
    for t, dims in tags:
        wfpt.blocks[t] = seq[:int(np.prod(dims))].reshape(dims).copy()
    axpy(noise, wfpt, wfnc)


def canonicalize_merged(forward: bool, wfnc: QSDArray, M: int, noise: float = 0.0):
    """``canonicalize`` for merged MPS (``src/canonicalize.hpp:88-106``); wfnc is
    noised in place first, as in the reference."""
    make_noise(wfnc, noise)
    if forward:
        s, U, V, kept, dn = gesvd_merged(wfnc, M, True)
        dimm_rows(s, V)
    else:
        s, U, V, kept, dn = gesvd_merged(wfnc, M, False)
        dimm_cols(U, s)
    return U, V, kept


def canonicalize_twosite(forward: bool, wfnc: QSDArray, M: int, noise: float = 0.0):
    """``canonicalize`` of a two-site wavefunction wfnc[l,n,n',r]
    (``src/canonicalize.hpp:27-45``): make_noise, then Gesvd<4,3> over the row
    merge (l,n) and the column merge (n',r); forward returns (U, s V), backward (U s, V),
    both as three-index site tensors."""
    make_noise(wfnc, noise)
    rinfo = MergeInfo(wfnc.qshape[:2], wfnc.dshape[:2])
    cinfo = MergeInfo(wfnc.qshape[2:], wfnc.dshape[2:])
    a2 = merge_rows(rinfo, merge_cols(wfnc, cinfo))
    s, U, V, kept, dn = gesvd_merged(a2, M, forward)
    if forward:
        dimm_rows(s, V)
    else:
        dimm_cols(U, s)
    return expand_rows(rinfo, U), expand_cols(V, cinfo)


def canonicalize_onesite_noise(forward: bool, wfnc: QSDArray, nb: QSDArray, M: int, noise: float):
    """One-site ``canonicalize`` with noise >= 1e-8 (``src/canonicalize.hpp:56-66``):
    wfnc is joined with the neighbouring site nb (forward wfnc*nb, backward nb*wfnc) and
    the two-site tensor is canonicalised with noise; returns (lmps, rmps)."""
    t = QSDArray()
    if forward:
        gemm(NoTrans, NoTrans, 1.0, wfnc, nb, 1.0, t, nc=4)
    else:
        gemm(NoTrans, NoTrans, 1.0, nb, wfnc, 1.0, t, nc=4)
    return canonicalize_twosite(forward, t, M, noise)


def canonicalize_onesite_backward(wfnc: QSDArray, lmps: QSDArray, M: int):
    """One-site backward canonicalize (``src/canonicalize.hpp:77-85``):
    Gesvd<3,2,RightArrow>(wfnc -> g, rmps), g *= s, lmps <- lmps * g."""
    rinfo = MergeInfo(wfnc.qshape[1:], wfnc.dshape[1:])
    lq = MergeInfo(wfnc.qshape[:1], wfnc.dshape[:1])
    a2 = merge_rows(lq, merge_cols(wfnc, rinfo))
    s, U, V, kept, dn = gesvd_merged(a2, M, False)
    g = expand_rows(lq, U)
    rmps = expand_cols(V, rinfo)
    dimm_cols(g, s)
    out = QSDArray()
    gemm(NoTrans, NoTrans, 1.0, lmps, g, 1.0, out, nc=3)
    return out, rmps


# ----------------------------------------------------------------------------
# a3: merged super-block operators (src/optimize.hpp:273-368)
# ----------------------------------------------------------------------------

def compute_merged_operator(forward: bool, mpo: QSDArray, hopr: QSDArray):
    if forward:
        m_bra = MergeInfo([hopr.qshape[0], mpo.qshape[1]], [hopr.dshape[0], mpo.dshape[1]])
        m_ket = MergeInfo([hopr.qshape[2], mpo.qshape[2]], [hopr.dshape[2], mpo.dshape[2]])
        # Contract(xHopr(0,1,2), xmpo(1,3,4,5)) -> (0,3,5,2,4) = [a, s, w', a', s']
        t5 = contract(hopr, "awx", mpo, "wstv", "asvxt")
        t4 = merge_rows(m_bra, t5)
        return merge_cols(t4, m_ket)
    m_bra = MergeInfo([mpo.qshape[1], hopr.qshape[0]], [mpo.dshape[1], hopr.dshape[0]])
    m_ket = MergeInfo([mpo.qshape[2], hopr.qshape[2]], [mpo.dshape[1], hopr.dshape[0]])
    # Contract(xmpo(0,1,2,3), xHopr(4,3,5)) -> (1,4,0,2,5) = [s, b, w, s', b']
    t5 = contract(mpo, "wstv", hopr, "bvy", "sbwty")
    t4 = merge_rows(m_bra, t5)
    return merge_cols(t4, m_ket)


def wave_merge_infos(lmpo: QSDArray, rmpo: QSDArray, lopr: QSDArray, ropr: QSDArray):
    """Ket merge infos of ``optimize_twosite_merged`` (``src/optimize.hpp:542-551``)."""
    q_l = [qneg(q) for q in lopr.qshape[2]]
    q_m = [qneg(q) for q in lmpo.qshape[2]]
    ql_info = MergeInfo([q_l, q_m], [lopr.dshape[0], lmpo.dshape[1]])
    q_n = [qneg(q) for q in rmpo.qshape[2]]
    q_r = [qneg(q) for q in ropr.qshape[2]]
    qr_info = MergeInfo([q_n, q_r], [rmpo.dshape[1], ropr.dshape[0]])
    return ql_info, qr_info


# ----------------------------------------------------------------------------
# a10: one bond (src/optimize.hpp:495-651), single root, one operator group
# ----------------------------------------------------------------------------

@dataclass
class BondResult:
    energy: float
    n_sigma: int
    kept: Dict[int, int]
    davidson: DavidsonStats
    times: Dict[str, float] = field(default_factory=dict)


def optimize_twosite_merged(forward: bool, lmpo: QSDArray, rmpo: QSDArray, lopr: QSDArray,
                            ropr: QSDArray, lwfn: QSDArray, rwfn: QSDArray, tole: float, M: int,
                            noise: float = 0.0):
    """Returns (BondResult, new_env, new_lwfn, new_rwfn); new_env is the renormalised
    left (forward) or right (backward) operator."""
    times = {}
    t0 = time.perf_counter()
    mL = compute_merged_operator(True, lmpo, lopr)
    mR = compute_merged_operator(False, rmpo, ropr)
    ql_info, qr_info = wave_merge_infos(lmpo, rmpo, lopr, ropr)
    twf = QSDArray()
    gemm(NoTrans, NoTrans, 1.0, lwfn, rwfn, 1.0, twf, nc=4)
    psi = merge_cols(merge_rows(ql_info, twf), qr_info)
    t1 = time.perf_counter()
    times["merge"] = t1 - t0
    diag = QSDArray(psi.q, psi.qshape, psi.dshape)
    compute_diagonal_elements(mL, mR, diag)
    t2 = time.perf_counter()
    times["diag"] = t2 - t1

    def multH(c, v):
        compute_sigma_vector(mL, mR, c, v)

    st = DavidsonStats()
    energy = davidson(multH, diag, psi, tole, st)
    t3 = time.perf_counter()
    times["davidson"] = t3 - t2
    U, V, kept = canonicalize_merged(forward, psi, M, noise)
    t4 = time.perf_counter()
    times["svd"] = t4 - t3
    if forward:
        new_env = renormalize_merged(True, mL, U, U)
    else:
        new_env = renormalize_merged(False, mR, V, V)
    t5 = time.perf_counter()
    times["renorm"] = t5 - t4
    new_l = expand_rows(ql_info, U)
    new_r = expand_cols(V, qr_info)
    return BondResult(energy, st.n_sigma, kept, st, times), new_env, new_l, new_r


# ----------------------------------------------------------------------------
# initial MPS (src/make_random_mpss.cpp:15-271) and sweeps (src/make_sweep.cpp,
# src/dmrg.cpp:21-132)
# ----------------------------------------------------------------------------

SITE_QUANTA = [(0, 0), (1, 1), (1, -1), (2, 0)]


def _unique_sorted_product(qa, qb):
    return sorted({qadd(x, y) for x in qa for y in qb})


def generate_quantum_states(nsite: int, qt, max_blocks: int):
    """``generate_quantum_states`` (``src/make_random_mpss.cpp:15-94``)."""
    sites = [list(SITE_QUANTA) for _ in range(nsite)]
    qb = [None] * nsite
    qb[0] = list(sites[0])
    for i in range(1, nsite - 1):
        bare = _unique_sorted_product(qb[i - 1], sites[i])
        qb[i] = [q for q in bare if q[0] <= qt[0]]
    qb[nsite - 1] = [tuple(qt)]
    for i in range(nsite - 1, 0, -1):
        qn = sites[i]
        qr = qb[i]
        qb[i - 1] = [ql for ql in qb[i - 1] if any(r == qadd(n, ql) for n in qn for r in qr)]
        assert qb[i - 1]
    for i in range(nsite - 1):
        qn = sites[i]
        if max_blocks > 0 and len(qb[i]) > max_blocks:
            offs = (len(qb[i]) - max_blocks) // 2
            qb[i] = qb[i][offs:offs + max_blocks]
            qb[i + 1] = [r for r in qb[i + 1] if any(r == qadd(l, n) for l in qb[i] for n in qn)]
            assert qb[i + 1]
    return qb


def site_tensor(ql, qr, q_total, fill=1.0) -> QSDArray:
    qn = list(SITE_QUANTA)
    a = QSDArray(q_total, [ql, qn, [qneg(q) for q in qr]], [[1] * len(ql), [1] * 4, [1] * len(qr)])
    a.allocate(fill)
    normalize(a)
    return a


def boundary_operator() -> QSDArray:
    op = QSDArray(ZERO, [[ZERO]] * 3, [[1]] * 3)
    op.allocate(1.0)
    return op


@dataclass
class MPSState:
    """In-memory sweep state: MPO sites, MPS site tensors, environments."""
    mpo: List[QSDArray]
    wave: List[Optional[QSDArray]]
    lenv: List[Optional[QSDArray]]
    renv: List[Optional[QSDArray]]
    M: int


def make_initial_state(mpo: List[QSDArray], n_elec: int, two_sz: int, M: int) -> MPSState:
    """Constant-filled, normalised site tensors then backward canonicalisation and
    right environments (``src/make_random_mpss.cpp:97-271``).  The reference fills
    each site with one uniform draw; after normalisation only its sign survives,
    which changes no energy, so +1 is used."""
    N = len(mpo)
    qt = (n_elec, two_sz)
    qb = generate_quantum_states(N, qt, M)
    wave: List[Optional[QSDArray]] = [None] * N
    ql = [ZERO]
    for i in range(N - 1):
        wave[i] = site_tensor(ql, qb[i], ZERO)
        ql = qb[i]
    wave[N - 1] = site_tensor(ql, [ZERO], qt)
    renv: List[Optional[QSDArray]] = [None] * N
    lenv: List[Optional[QSDArray]] = [None] * N
    renv[N - 1] = boundary_operator()
    wfnc = wave[N - 1]
    rmps = [None] * N
    for i in range(N - 1, 0, -1):
        lm, rm = canonicalize_onesite_backward(wfnc, wave[i - 1], M)
        wfnc = lm
        normalize(wfnc)
        wave[i - 1] = wfnc
        rmps[i] = rm
        renv[i - 1] = renormalize_mpo(False, mpo[i], renv[i], rm, rm)
    for i in range(1, N):
        wave[i] = rmps[i]
    lenv[0] = boundary_operator()
    return MPSState(mpo, wave, lenv, renv, M)


@dataclass
class SweepLog:
    energy: float
    bond_energies: List[float]
    n_sigma: int
    seconds: float
    times: Dict[str, float]


def make_sweep(state: MPSState, tole: float, bond_hook=None) -> SweepLog:
    """Forward then backward two-site sweep (``src/make_sweep.cpp:12-253``).

    Davidson tolerance is 0.1*tole (``src/make_sweep.cpp:112,215``); the sweep
    energy is the minimum over bonds."""
    N = len(state.mpo)
    t0 = time.perf_counter()
    emin = 1.0e8
    es = []
    nsig = 0
    times: Dict[str, float] = {}
    wave = state.wave
    # forward: bond (i, i+1)
    for i in range(N - 1):
        res, env, nl, nr = optimize_twosite_merged(True, state.mpo[i], state.mpo[i + 1], state.lenv[i],
                                                   state.renv[i + 1], wave[i], wave[i + 1], 0.1 * tole,
                                                   state.M)
        if bond_hook:
            bond_hook(True, i, res)
        state.lenv[i + 1] = env
        wave[i] = nl
        wave[i + 1] = nr
        emin = min(emin, res.energy)
        es.append(res.energy)
        nsig += res.n_sigma
        for k, v in res.times.items():
            times[k] = times.get(k, 0.0) + v
    # backward: bond (i-1, i)
    for i in range(N - 1, 0, -1):
        res, env, nl, nr = optimize_twosite_merged(False, state.mpo[i - 1], state.mpo[i], state.lenv[i - 1],
                                                   state.renv[i], wave[i - 1], wave[i], 0.1 * tole, state.M)
        if bond_hook:
            bond_hook(False, i - 1, res)
        state.renv[i - 1] = env
        wave[i - 1] = nl
        wave[i] = nr
        emin = min(emin, res.energy)
        es.append(res.energy)
        nsig += res.n_sigma
        for k, v in res.times.items():
            times[k] = times.get(k, 0.0) + v
    return SweepLog(emin, es, nsig, time.perf_counter() - t0, times)


def dmrg(mpo: List[QSDArray], n_elec: int, two_sz: int, M: int, tole: float, max_sweeps: int,
         min_sweeps: int = 0, state: Optional[MPSState] = None, verbose: bool = False):
    """Sweeps until |dE| < tole after at least one iteration (``src/dmrg.cpp:37-79``)."""
    if state is None:
        state = make_initial_state(mpo, n_elec, two_sz, M)
    e_prev = 0.0
    logs = []
    for it in range(max_sweeps):
        log = make_sweep(state, tole)
        logs.append(log)
        de = log.energy - e_prev
        e_prev = log.energy
        if verbose:
            print(f"sweep {it}: E = {log.energy:.16f} dE = {de:.2e} ({log.seconds:.2f}s)", flush=True)
        if it > 0 and abs(de) < tole and it + 1 >= min_sweeps:
            break
    return state, logs
