"""In-memory two-site DMRG sweeps on the device (the caller of the hot path).

Replaces the reference's disk-backed sweep driver (src/make_sweep.cpp:12-253,
src/dmrg.cpp:21-132) and initial-state builder (src/make_random_mpss.cpp:15-271):
MPO, site tensors and block operators stay in HBM; each bond is one call of
``optimize_twosite_merged`` through the C ABI.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from . import core
from .core import Context, Tensor

SITE_QUANTA = [(0, 0), (1, 1), (1, -1), (2, 0)]


def _qadd(a, b):
    return (a[0] + b[0], a[1] + b[1])


def generate_quantum_states(nsite: int, qt, max_blocks: int):
    """Bond quantum numbers of the initial MPS (src/make_random_mpss.cpp:15-94):
    unique products filtered by particle number, pruned from the right, then
    capped to ``max_blocks`` central sectors."""
    qb = [None] * nsite
    qb[0] = list(SITE_QUANTA)
    for i in range(1, nsite - 1):
        bare = sorted({_qadd(x, y) for x in qb[i - 1] for y in SITE_QUANTA})
        qb[i] = [q for q in bare if q[0] <= qt[0]]
    qb[nsite - 1] = [tuple(qt)]
    for i in range(nsite - 1, 0, -1):
        qr = qb[i]
        qb[i - 1] = [ql for ql in qb[i - 1] if any(r == _qadd(n, ql) for n in SITE_QUANTA for r in qr)]
        if not qb[i - 1]:
            raise ValueError("no quantum states reach the target quantum number")
    for i in range(nsite - 1):
        if max_blocks > 0 and len(qb[i]) > max_blocks:
            offs = (len(qb[i]) - max_blocks) // 2
            qb[i] = qb[i][offs:offs + max_blocks]
            qb[i + 1] = [r for r in qb[i + 1] if any(r == _qadd(l, n) for l in qb[i] for n in SITE_QUANTA)]
    return qb


def _site_tensor(ctx: Context, ql, qr, q_total) -> Tensor:
    qshape = [list(ql), list(SITE_QUANTA), [(-q[0], -q[1]) for q in qr]]
    dshape = [[1] * len(ql), [1] * 4, [1] * len(qr)]
    t = Tensor.create(ctx, q_total, qshape, dshape)  # every allowed block
    t.upload(np.ones(t.nnz))
    core.normalize(ctx, t)
    return t


def _boundary(ctx: Context) -> Tensor:
    t = Tensor.create(ctx, (0, 0), [[(0, 0)]] * 3, [[1]] * 3)
    t.upload(np.ones(1))
    return t


@dataclass
class DeviceState:
    mpo: List[Tensor]
    wave: List[Tensor]
    lenv: List[Optional[Tensor]]
    renv: List[Optional[Tensor]]
    M: int


def make_initial_state(ctx: Context, mpo: List[Tensor], n_elec: int, two_sz: int, M: int) -> DeviceState:
    """Constant-filled normalised site tensors, backward canonicalisation with
    truncation M, and the right block operators (src/make_random_mpss.cpp:97-271).
    The reference fills each site with one uniform draw; after normalisation only
    its sign survives, which changes no energy, so +1 is used."""
    N = len(mpo)
    qt = (n_elec, two_sz)
    qb = generate_quantum_states(N, qt, M)
    wave: List[Optional[Tensor]] = [None] * N
    ql = [(0, 0)]
    for i in range(N - 1):
        wave[i] = _site_tensor(ctx, ql, qb[i], (0, 0))
        ql = qb[i]
    wave[N - 1] = _site_tensor(ctx, ql, [(0, 0)], qt)
    renv: List[Optional[Tensor]] = [None] * N
    lenv: List[Optional[Tensor]] = [None] * N
    renv[N - 1] = _boundary(ctx)
    wfnc = wave[N - 1]
    for i in range(N - 1, 0, -1):
        # one-site backward canonicalize (src/canonicalize.hpp:77-85)
        m2 = core.merge_cols(ctx, wfnc)
        g, v = core.canonicalize(ctx, False, m2, M)
        rmps = core.expand_cols(ctx, v, wfnc)
        lm = core.gemm(ctx, 0, 0, 1.0, wave[i - 1], g, 3)
        core.normalize(ctx, lm)
        wfnc = lm
        wave[i - 1] = lm
        wave[i] = rmps
        # right block operator through the merged-operator path
        mR = core.compute_merged_operator(ctx, False, mpo[i], renv[i])
        vm = core.merge_cols(ctx, rmps)
        renv[i - 1] = core.renormalize(ctx, False, mR, vm, vm)
    lenv[0] = _boundary(ctx)
    return DeviceState(mpo, wave, lenv, renv, M)


def _sector_dim(nsites: int, q) -> int:
    from math import comb

    p, s = q
    if (p + s) % 2:
        return 0
    nu, nd = (p + s) // 2, (p - s) // 2
    if nu < 0 or nd < 0 or nu > nsites or nd > nsites:
        return 0
    return comb(nsites, nu) * comb(nsites, nd)


def make_random_state(ctx: Context, mpo: List[Tensor], n_elec: int, two_sz: int, M: int, seed: int = 0,
                      oversample: float = 2.0) -> DeviceState:
    """Random MPS of bond dimension M: bond sectors as the initial state, sector dims
    proportional to the block Hilbert-space dimension (total about oversample*M per
    bond, each at most its Hilbert dimension), normal random entries, then the same
    backward canonicalisation with truncation M as ``make_initial_state``."""
    N = len(mpo)
    qt = (n_elec, two_sz)
    qb = generate_quantum_states(N, qt, 0)
    rng = np.random.default_rng(seed)
    dims = []
    for i in range(N - 1):
        left = i + 1
        right = N - 1 - i
        hd = []
        for q in qb[i]:
            qr = (qt[0] - q[0], qt[1] - q[1])
            hd.append(min(_sector_dim(left, q), _sector_dim(right, qr)))
        tot = float(sum(hd)) or 1.0
        target = oversample * M
        dims.append([max(1, min(h, int(np.ceil(target * h / tot)))) if h > 0 else 0 for h in hd])
    wave: List[Optional[Tensor]] = [None] * N
    ql, dl = [(0, 0)], [1]
    for i in range(N):
        if i < N - 1:
            qr, dr, q_tot = qb[i], dims[i], (0, 0)
        else:
            qr, dr, q_tot = [(0, 0)], [1], qt
        qshape = [list(ql), list(SITE_QUANTA), [(-q[0], -q[1]) for q in qr]]
        dshape = [list(dl), [1] * 4, list(dr)]
        t = Tensor.create(ctx, q_tot, qshape, dshape)
        t.upload(rng.standard_normal(t.nnz))
        core.normalize(ctx, t)
        wave[i] = t
        ql, dl = qr, dr
    renv: List[Optional[Tensor]] = [None] * N
    lenv: List[Optional[Tensor]] = [None] * N
    renv[N - 1] = _boundary(ctx)
    wfnc = wave[N - 1]
    for i in range(N - 1, 0, -1):
        m2 = core.merge_cols(ctx, wfnc)
        g, v = core.canonicalize(ctx, False, m2, M)
        rmps = core.expand_cols(ctx, v, wfnc)
        lm = core.gemm(ctx, 0, 0, 1.0, wave[i - 1], g, 3)
        core.normalize(ctx, lm)
        wfnc = lm
        wave[i - 1] = lm
        wave[i] = rmps
        mR = core.compute_merged_operator(ctx, False, mpo[i], renv[i])
        vm = core.merge_cols(ctx, rmps)
        renv[i - 1] = core.renormalize(ctx, False, mR, vm, vm)
    lenv[0] = _boundary(ctx)
    return DeviceState(mpo, wave, lenv, renv, M)


def bond_operands(ctx: Context, st: DeviceState, i: int):
    """Merged operators and merged wavefunction of bond (i, i+1) in the state's current gauge."""
    mL = core.compute_merged_operator(ctx, True, st.mpo[i], st.lenv[i])
    mR = core.compute_merged_operator(ctx, False, st.mpo[i + 1], st.renv[i + 1])
    psi = core.merge_wavefunction(ctx, st.mpo[i], st.mpo[i + 1], st.lenv[i], st.renv[i + 1], st.wave[i],
                                  st.wave[i + 1])
    return mL, mR, psi


def advance_left(ctx: Context, st: DeviceState, stop: int):
    """Move the orthogonality centre from site 0 to site ``stop`` by forward
    canonicalisation without optimisation: at each bond U becomes the left site
    tensor, s V^T joins the next site and the left block operator is renormalised."""
    for i in range(stop):
        mL = core.compute_merged_operator(ctx, True, st.mpo[i], st.lenv[i])
        psi = core.merge_wavefunction(ctx, st.mpo[i], st.mpo[i + 1], st.lenv[i], st.renv[i + 1], st.wave[i],
                                      st.wave[i + 1])
        U, sV = core.canonicalize(ctx, True, psi, st.M)
        st.lenv[i + 1] = core.renormalize(ctx, True, mL, U, U)
        st.wave[i], st.wave[i + 1] = core.expand_wavefunction(ctx, st.mpo[i], st.mpo[i + 1], st.lenv[i],
                                                              st.renv[i + 1], U, sV)


@dataclass
class SweepLog:
    energy: float
    bond_energies: List[float]
    n_sigma: int
    sigma_flops: float
    seconds: float
    times: Dict[str, float] = field(default_factory=dict)
    kind: str = "twosite"


def _left_env_step(ctx: Context, st: DeviceState, L: Tensor, k: int) -> Tensor:
    """L_{k+1} from L_k and the left-canonical site tensor k (the product a forward
    bond step forms from the same operands)."""
    mL = core.compute_merged_operator(ctx, True, st.mpo[k], L)
    um = core.merge_rows(ctx, st.wave[k])
    return core.renormalize(ctx, True, mL, um, um)


def make_sweep(ctx: Context, st: DeviceState, tole: float, bond_hook=None, noise: float = 0.0,
               env_checkpoint: int = 0) -> SweepLog:
    """Forward then backward sweep; Davidson tolerance 0.1*tole; sweep energy =
    minimum over bonds (src/make_sweep.cpp:12-253); ``noise`` is added to every bond's
    wavefunction before its truncation (make_noise, src/canonicalize.hpp:11-24).

    Block operators that a pass has made stale are dropped as it goes (the right
    ones behind the forward pass, the left ones behind the backward pass), so about
    one operator per site is resident instead of two; the sweep ends with the
    orthogonality centre at site 0, the right operators current and the left ones
    (but the boundary) dropped.  The reference keeps each in a file per site and
    reads back the ones a bond needs.

    ``env_checkpoint`` = k > 0 keeps, of the operators a pass leaves behind for the
    other pass, only those at every k-th site (and the boundaries); a bond whose
    operator was dropped rebuilds it, with the ones between, from the nearest kept
    one by the same merged-operator and renormalisation products that made it (so
    the sweep's results do not change), and drops each once used.  Resident
    operators fall from ~N to ~2N/k + 2k at the cost of ~(k-1)/k extra
    renormalisations per bond."""
    N = len(st.mpo)
    k = int(env_checkpoint)
    t0 = time.perf_counter()
    es: List[float] = []
    nsig = 0
    flops = 0.0
    times: Dict[str, float] = {}

    def acc(stats):
        nonlocal nsig, flops
        nsig += int(stats["n_sigma"])
        flops += stats["sigma_flops"]
        for key in ("t_merge", "t_diag", "t_davidson", "t_svd", "t_renorm", "n_sigma_fp64"):
            times[key] = times.get(key, 0.0) + stats[key]
        times["n_unconverged"] = times.get("n_unconverged", 0.0) + (0.0 if stats["converged"] else 1.0)

    def kept(j: int) -> bool:
        return k <= 0 or j % k == 0 or j == 0 or j == N - 1

    def rebuild(side: str, j: int):
        """st.lenv[j] (or st.renv[j]) and the dropped ones between it and the nearest kept one."""
        t = time.perf_counter()
        if side == "l":
            c = max(m for m in range(j) if st.lenv[m] is not None)
            for m in range(c, j):
                st.lenv[m + 1] = _left_env_step(ctx, st, st.lenv[m], m)
            n = j - c
        else:
            c = min(m for m in range(j + 1, N) if st.renv[m] is not None)
            for m in range(c, j, -1):
                st.renv[m - 1] = _right_env_step(ctx, st, st.renv[m], m)
            n = c - j
        times["env_rebuilt"] = times.get("env_rebuilt", 0.0) + n
        times["t_env_rebuild"] = times.get("t_env_rebuild", 0.0) + time.perf_counter() - t

    for i in range(N - 1):
        if st.renv[i + 1] is None:
            rebuild("r", i + 1)
        e, env, nl, nr, stats = core.optimize_twosite_merged(ctx, True, st.mpo[i], st.mpo[i + 1], st.lenv[i],
                                                             st.renv[i + 1], st.wave[i], st.wave[i + 1],
                                                             0.1 * tole, st.M, noise)
        # L_{N-1} is used by no two-site bond
        st.lenv[i + 1] = env if i + 1 < N - 1 else None
        st.wave[i], st.wave[i + 1] = nl, nr
        if i + 1 < N - 1:
            st.renv[i + 1] = None  # stale once the bond moves on; rebuilt by the backward pass
        if not kept(i) and i < N - 2:
            st.lenv[i] = None  # rebuilt from the nearest kept one when the backward pass needs it
        es.append(e)
        acc(stats)
        if bond_hook:
            bond_hook(True, i, e, stats)
    for i in range(N - 1, 0, -1):
        if st.lenv[i - 1] is None:
            rebuild("l", i - 1)
        e, env, nl, nr, stats = core.optimize_twosite_merged(ctx, False, st.mpo[i - 1], st.mpo[i], st.lenv[i - 1],
                                                             st.renv[i], st.wave[i - 1], st.wave[i], 0.1 * tole,
                                                             st.M, noise)
        st.renv[i - 1] = env
        st.wave[i - 1], st.wave[i] = nl, nr
        if i - 1 > 0:
            st.lenv[i - 1] = None  # stale; rebuilt by the next forward pass
        if not kept(i) and i > 1:
            st.renv[i] = None  # rebuilt from the nearest kept one when the next forward pass needs it
        es.append(e)
        acc(stats)
        if bond_hook:
            bond_hook(False, i - 1, e, stats)
    return SweepLog(min(es), es, nsig, flops, time.perf_counter() - t0, times)


def split_onesite_noise(ctx: Context, forward: bool, wf: Tensor, nb: Tensor, M: int, noise: float):
    """One-site canonicalize with noise (src/canonicalize.hpp:48-66): the optimised site
    tensor wf is joined with its neighbour nb (forward: wf[l,n,a] nb[a,n',r]; backward:
    nb[l,n',a] wf[a,n,r]) into a two-site tensor, which is noised (make_noise) and split
    again with truncation M (Gesvd<4,3>, src/canonicalize.hpp:27-45).  Returns (left,
    right, merged factor): forward (U[l,n,a], sV[a,n',r], U merged over (l,n)); backward
    (Us[l,n',a], V[a,n,r], V merged over (n,r))."""
    if forward:
        t4 = core.gemm(ctx, 0, 0, 1.0, wf, nb, 4)
    else:
        t4 = core.gemm(ctx, 0, 0, 1.0, nb, wf, 4)
    core.make_noise(ctx, t4, noise)
    m = core.merge_cols(ctx, core.merge_rows(ctx, t4))
    a, b = core.canonicalize(ctx, forward, m, M)
    lk, rk = (wf, nb) if forward else (nb, wf)
    left = core.expand_rows(ctx, a, lk)
    right = core.expand_cols(ctx, b, rk)
    return left, right, (a if forward else b)


def optimize_onesite(ctx: Context, forward: bool, st: DeviceState, i: int, tole: float, noise: float = 0.0):
    """One-site step at site i (src/optimize.hpp:37-145) through the merged hot path:
    forward, psi[(l,n), r] with mL = merge(L_i, W_i) and the unmerged R_i; backward,
    psi[l, (n,r)] with the unmerged L_i and mR = merge(R_i, W_i).  Davidson, truncated
    SVD (M kept), s V^T (or U s) moved into the neighbouring site, and the block
    operator renormalised past site i.  Returns (energy, diagonalize stats)."""
    wf = st.wave[i]
    if forward:
        op = core.compute_merged_operator(ctx, True, st.mpo[i], st.lenv[i])
        L, R = op, st.renv[i]
        psi = core.merge_rows(ctx, wf)
    else:
        op = core.compute_merged_operator(ctx, False, st.mpo[i], st.renv[i])
        L, R = st.lenv[i], op
        psi = core.merge_cols(ctx, wf)
    diag = psi.like()
    core.compute_diagonal_elements(ctx, L, R, diag)
    e, stats = core.diagonalize(ctx, L, R, diag, psi, tole)
    if noise >= 1.0e-8:
        wf_opt = core.expand_rows(ctx, psi, wf) if forward else core.expand_cols(ctx, psi, wf)
        j = i + 1 if forward else i - 1
        left, right, f = split_onesite_noise(ctx, forward, wf_opt, st.wave[j], st.M, noise)
        if forward:
            st.wave[i], st.wave[i + 1] = left, right
            st.lenv[i + 1] = core.renormalize(ctx, True, op, f, f)
        else:
            st.wave[i - 1], st.wave[i] = left, right
            st.renv[i - 1] = core.renormalize(ctx, False, op, f, f)
        return e, stats
    if forward:
        U, sV = core.canonicalize(ctx, True, psi, st.M)
        st.wave[i] = core.expand_rows(ctx, U, wf)
        nxt = core.gemm(ctx, 0, 0, 1.0, sV, st.wave[i + 1], 3)
        st.wave[i + 1] = nxt
        st.lenv[i + 1] = core.renormalize(ctx, True, op, U, U)
    else:
        Us, V = core.canonicalize(ctx, False, psi, st.M)
        st.wave[i] = core.expand_cols(ctx, V, wf)
        prv = core.gemm(ctx, 0, 0, 1.0, st.wave[i - 1], Us, 3)
        st.wave[i - 1] = prv
        st.renv[i - 1] = core.renormalize(ctx, False, op, V, V)
    return e, stats


def make_sweep_onesite(ctx: Context, st: DeviceState, tole: float, noise: float = 0.0) -> SweepLog:
    """One-site forward then backward sweep (sites 0..N-2, then N-1..1); Davidson
    tolerance 0.1*tole; sweep energy = minimum over sites."""
    N = len(st.mpo)
    t0 = time.perf_counter()
    es: List[float] = []
    nsig = 0
    for i in range(N - 1):
        e, s = optimize_onesite(ctx, True, st, i, 0.1 * tole, noise)
        es.append(e)
        nsig += s["n_sigma"]
    for i in range(N - 1, 0, -1):
        e, s = optimize_onesite(ctx, False, st, i, 0.1 * tole, noise)
        es.append(e)
        nsig += s["n_sigma"]
    return SweepLog(min(es), es, nsig, 0.0, time.perf_counter() - t0, kind="onesite")


def fill_right_envs(ctx: Context, st: DeviceState):
    """Rebuild every dropped right block operator of a state whose orthogonality centre
    is at site 0 (as a two-site sweep with checkpointed operators leaves it)."""
    for j in range(len(st.mpo) - 2, -1, -1):
        if st.renv[j] is None:
            st.renv[j] = _right_env_step(ctx, st, st.renv[j + 1], j + 1)


def dmrg(ctx: Context, mpo_dicts: List[dict], n_elec: int, two_sz: int, M: int, tole: float, max_sweeps: int,
         min_sweeps: int = 0, verbose: bool = False, onesite: bool = False, noise: float = 0.0,
         env_checkpoint: int = 0):
    """Sweeps until |dE| < tole after at least one iteration (src/dmrg.cpp:37-79); with
    ``onesite``, the reference's second stage follows: one-site sweeps from the
    converged two-site state until |dE| < tole again (src/dmrg.cpp:80-115).  ``noise``
    is the dmrg.conf keyword of that name, passed to every truncation;
    ``env_checkpoint`` is make_sweep's (two-site stage)."""
    mpo = [Tensor.from_dict(ctx, d) for d in mpo_dicts]
    st = make_initial_state(ctx, mpo, n_elec, two_sz, M)
    e_prev = 0.0
    logs = []
    stages = [make_sweep] + ([make_sweep_onesite] if onesite else [])
    for stage in stages:
        if stage is make_sweep_onesite:
            fill_right_envs(ctx, st)  # the one-site stage reads every right operator
        extra = {"env_checkpoint": env_checkpoint} if stage is make_sweep else {}
        for it in range(max_sweeps):
            log = stage(ctx, st, tole, noise=noise, **extra)
            logs.append(log)
            de = log.energy - e_prev
            e_prev = log.energy
            if verbose:
                print(f"{stage.__name__} {it}: E = {log.energy:.16f} dE = {de:.2e} ({log.seconds:.2f}s)", flush=True)
            if it > 0 and abs(de) < tole and it + 1 >= min_sweeps:
                break
    return st, logs


# ---------------------------------------------------------------------------
# energy gradient with respect to the MPO and the Hamiltonian parameters
# ---------------------------------------------------------------------------
def _right_env_step(ctx: Context, st: DeviceState, R: Tensor, k: int) -> Tensor:
    """R_{k-1} from R_k and the right-canonical site tensor k."""
    mR = core.compute_merged_operator(ctx, False, st.mpo[k], R)
    vm = core.merge_cols(ctx, st.wave[k])
    return core.renormalize(ctx, False, mR, vm, vm)


@dataclass
class GradientLog:
    energy: float                 # <psi|H|psi> of the (unchanged) state
    bond_energies: List[float]    # the same value measured at every bond
    site_grads: List[np.ndarray]  # dE/dW per site, in the MPO's block order
    env_recomputed: int           # right environments rebuilt from checkpoints
    env_peak: int                 # right environments held at once
    seconds: float


def gradient_sweep(ctx: Context, st: DeviceState, checkpoint: int = 4) -> GradientLog:
    """dE/dW for every site MPO of a state whose orthogonality centre is at site 0
    (as a backward sweep leaves it).

    One forward pass: at bond (i, i+1) the merged two-site wavefunction gives
    dE/dW_i (and dE/dW_{i+1} at the last bond) through the adjoint of the merged
    operator; the centre then moves on by an SVD that keeps every non-zero singular
    value, so the state and its energy do not change.  Right block operators are
    kept only at every ``checkpoint``-th site; the others are recomputed from the
    nearest checkpoint to the right when the pass reaches them and dropped once used.
    The state's own list of right environments is not modified."""
    t0 = time.perf_counter()
    N = len(st.mpo)
    ckpt = {j: st.renv[j] for j in range(N) if j % checkpoint == 0 or j == N - 1}
    pending: Dict[int, Tensor] = {}
    recomputed = 0
    peak = len(ckpt)
    wave = list(st.wave)
    work = DeviceState(st.mpo, wave, [None] * N, [None] * N, st.M)

    def right_env(j: int) -> Tensor:
        nonlocal recomputed, peak
        if j in ckpt:
            return ckpt[j]
        if j in pending:
            return pending.pop(j)
        c = min(k for k in ckpt if k > j)
        R = ckpt[c]
        for k in range(c, j, -1):
            R = _right_env_step(ctx, work, R, k)
            recomputed += 1
            if k - 1 > j:
                pending[k - 1] = R
        peak = max(peak, len(ckpt) + len(pending) + 1)
        return R

    L = st.lenv[0]
    grads: List[Optional[np.ndarray]] = [None] * N
    energies = []
    for i in range(N - 1):
        R = right_env(i + 1)
        psi = core.merge_wavefunction(ctx, st.mpo[i], st.mpo[i + 1], L, R, wave[i], wave[i + 1])
        core.normalize(ctx, psi)
        gl, gr = core.mpo_gradient(ctx, st.mpo[i], st.mpo[i + 1], L, R, psi)
        grads[i] = gl
        if i == N - 2:
            grads[i + 1] = gr
        # E is linear in W_i: E = sum_b W_i[b] dE/dW_i[b]
        energies.append(float(np.dot(st.mpo[i].download(), gl)))
        if i < N - 2:
            # move the centre: psi has rank <= M, so keeping M singular values is exact
            mL = core.compute_merged_operator(ctx, True, st.mpo[i], L)
            U, sV = core.canonicalize(ctx, True, psi, st.M)
            wave[i], wave[i + 1] = core.expand_wavefunction(ctx, st.mpo[i], st.mpo[i + 1], L, R, U, sV)
            L = core.renormalize(ctx, True, mL, U, U)
    return GradientLog(float(np.mean(energies)), energies, grads, recomputed, peak, time.perf_counter() - t0)


def parameter_gradient(site_grads: List[np.ndarray], mpo_tags: List[np.ndarray],
                       jacobians: List[Dict[int, Dict[object, float]]]) -> Dict[object, float]:
    """Chain rule through the MPO generator: dE/dtheta = sum over sites and blocks of
    dE/dW[b] * dW[b]/dtheta, with the generator's per-site {tag: {theta: dW/dtheta}}."""
    out: Dict[object, float] = {}
    for g, tags, jac in zip(site_grads, mpo_tags, jacobians):
        for b, tag in enumerate(tags):
            d = jac.get(int(tag))
            if not d:
                continue
            for par, f in d.items():
                out[par] = out.get(par, 0.0) + float(g[b]) * f
    return out


def restart_state(ctx: Context, mpo: List[Tensor], st: DeviceState) -> DeviceState:
    """The MPS of ``st`` (orthogonality centre at site 0) with a new Hamiltonian of
    the same MPO block structure: right block operators rebuilt for ``mpo``."""
    N = len(mpo)
    wave = list(st.wave)
    renv: List[Optional[Tensor]] = [None] * N
    lenv: List[Optional[Tensor]] = [None] * N
    renv[N - 1] = _boundary(ctx)
    new = DeviceState(mpo, wave, lenv, renv, st.M)
    for k in range(N - 1, 0, -1):
        renv[k - 1] = _right_env_step(ctx, new, renv[k], k)
    lenv[0] = _boundary(ctx)
    return new


# ---------------------------------------------------------------------------
# multiple roots: state-specific targeting with the lower roots projected out
# ---------------------------------------------------------------------------
def identity_mpo(ctx: Context, N: int) -> List[Tensor]:
    """MPO of the identity (bond dimension 1): the overlap block operators of two
    states are block operators of this MPO."""
    from .mpogen import SiteMPO, _op_matrix

    out = []
    for _ in range(N):
        W = SiteMPO([(0, 0)], [(0, 0)])
        W.add(0, _op_matrix("I"), 0)
        out.append(Tensor.from_dict(ctx, W.to_dict()))
    return out


@dataclass
class LowerRoot:
    """A converged lower root and its block operators against the state being
    optimised (bra = current state, ket = this root): Hamiltonian (Lx, Rx) and
    overlap (Lo, Ro).  Its own orthogonality centre follows the current bond."""
    st: DeviceState
    energy: float
    Lx: List[Optional[Tensor]]
    Rx: List[Optional[Tensor]]
    Lo: List[Optional[Tensor]]
    Ro: List[Optional[Tensor]]


def _cross_sigma(ctx: Context, mL: Tensor, mR: Tensor, psi_k: Tensor, like: Tensor) -> Tensor:
    """mL psi_k mR^T: a lower root's wavefunction carried into this bond's basis,
    stored in `like`'s layout."""
    scr = core.gemm(ctx, 0, 0, 1.0, mL, psi_k, 3)
    out = core.gemm(ctx, 0, 1, 1.0, scr, mR, 2)
    t = like.like()
    core.accumulate(ctx, 1.0, out, t)
    return t


def _two_site(ctx: Context, a: Tensor, b: Tensor) -> Tensor:
    return core.gemm(ctx, 0, 0, 1.0, core.merge_rows(ctx, a), core.merge_cols(ctx, b), 2)


def make_lower_root(ctx: Context, st: DeviceState, root: DeviceState, energy: float,
                    idm: List[Tensor]) -> LowerRoot:
    """Cross block operators of a lower root against state `st`, both centred at site 0."""
    N = len(st.mpo)
    Lx, Rx, Lo, Ro = [None] * N, [None] * N, [None] * N, [None] * N
    Lx[0], Lo[0], Rx[N - 1], Ro[N - 1] = _boundary(ctx), _boundary(ctx), _boundary(ctx), _boundary(ctx)
    for i in range(N - 1, 0, -1):
        vc = core.merge_cols(ctx, st.wave[i])
        vk = core.merge_cols(ctx, root.wave[i])
        Rx[i - 1] = core.renormalize(ctx, False, core.compute_merged_operator(ctx, False, st.mpo[i], Rx[i]), vc, vk)
        Ro[i - 1] = core.renormalize(ctx, False, core.compute_merged_operator(ctx, False, idm[i], Ro[i]), vc, vk)
    return LowerRoot(DeviceState(root.mpo, list(root.wave), [None] * N, [None] * N, root.M), energy, Lx, Rx, Lo, Ro)


def optimize_twosite_projected(ctx: Context, forward: bool, st: DeviceState, i: int, tole: float,
                               lowers: List[LowerRoot], idm: List[Tensor]) -> float:
    """One two-site step at bond (i, i+1) (forward) or (i-1, i) (backward) with the lower
    roots projected out (src/optimize.hpp:495-651 with the Functor<2> of
    src/diagonalize.hpp:200-277); the lower roots' centres and cross operators move on."""
    j = i if forward else i - 1  # left site of the bond
    mL = core.compute_merged_operator(ctx, True, st.mpo[j], st.lenv[j])
    mR = core.compute_merged_operator(ctx, False, st.mpo[j + 1], st.renv[j + 1])
    psi = core.merge_wavefunction(ctx, st.mpo[j], st.mpo[j + 1], st.lenv[j], st.renv[j + 1], st.wave[j],
                                  st.wave[j + 1])
    diag = psi.like()
    core.compute_diagonal_elements(ctx, mL, mR, diag)
    S, H, E, cross = [], [], [], []
    for lr in lowers:
        psi_k = _two_site(ctx, lr.st.wave[j], lr.st.wave[j + 1])
        mLx = core.compute_merged_operator(ctx, True, st.mpo[j], lr.Lx[j])
        mRx = core.compute_merged_operator(ctx, False, st.mpo[j + 1], lr.Rx[j + 1])
        mLo = core.compute_merged_operator(ctx, True, idm[j], lr.Lo[j])
        mRo = core.compute_merged_operator(ctx, False, idm[j + 1], lr.Ro[j + 1])
        S.append(_cross_sigma(ctx, mLo, mRo, psi_k, psi))
        H.append(_cross_sigma(ctx, mLx, mRx, psi_k, psi))
        E.append(lr.energy)
        cross.append((psi_k, mLx, mRx, mLo, mRo))
    e, _ = core.diagonalize_projected(ctx, mL, mR, diag, psi, tole, S, H, E)
    if forward:
        U, sV = core.canonicalize(ctx, True, psi, st.M)
        st.wave[j], st.wave[j + 1] = core.expand_wavefunction(ctx, st.mpo[j], st.mpo[j + 1], st.lenv[j],
                                                              st.renv[j + 1], U, sV)
        st.lenv[j + 1] = core.renormalize(ctx, True, mL, U, U)
        for lr, (psi_k, mLx, _, mLo, _) in zip(lowers, cross):
            Uk, sVk = core.canonicalize(ctx, True, psi_k, lr.st.M)
            lr.st.wave[j] = core.expand_rows(ctx, Uk, lr.st.wave[j])
            lr.st.wave[j + 1] = core.expand_cols(ctx, sVk, lr.st.wave[j + 1])
            lr.Lx[j + 1] = core.renormalize(ctx, True, mLx, U, Uk)
            lr.Lo[j + 1] = core.renormalize(ctx, True, mLo, U, Uk)
    else:
        Us, V = core.canonicalize(ctx, False, psi, st.M)
        st.wave[j], st.wave[j + 1] = core.expand_wavefunction(ctx, st.mpo[j], st.mpo[j + 1], st.lenv[j],
                                                              st.renv[j + 1], Us, V)
        st.renv[j] = core.renormalize(ctx, False, mR, V, V)
        for lr, (psi_k, _, mRx, _, mRo) in zip(lowers, cross):
            Usk, Vk = core.canonicalize(ctx, False, psi_k, lr.st.M)
            lr.st.wave[j + 1] = core.expand_cols(ctx, Vk, lr.st.wave[j + 1])
            lr.st.wave[j] = core.expand_rows(ctx, Usk, lr.st.wave[j])
            lr.Rx[j] = core.renormalize(ctx, False, mRx, V, Vk)
            lr.Ro[j] = core.renormalize(ctx, False, mRo, V, Vk)
    return e


def dmrg_roots(ctx: Context, mpo_dicts: List[dict], n_elec: int, two_sz: int, M: int, tole: float, max_sweeps: int,
               nroots: int, seed: int = 0, verbose: bool = False):
    """State-specific DMRG for the lowest nroots states (src/dmrg.cpp:37-79 over iroot):
    each root is swept to |dE| < tole with every lower root projected out of H_eff.
    Returns the roots' energies and states."""
    mpo = [Tensor.from_dict(ctx, d) for d in mpo_dicts]
    N = len(mpo)
    idm = identity_mpo(ctx, N)
    energies: List[float] = []
    states: List[DeviceState] = []
    for r in range(nroots):
        if r == 0:
            st = make_initial_state(ctx, mpo, n_elec, two_sz, M)
        else:
            st = make_random_state(ctx, mpo, n_elec, two_sz, M, seed=seed + r)
        lowers = [make_lower_root(ctx, st, states[k], energies[k], idm) for k in range(r)]
        e_prev = 0.0
        e_sweep = 0.0
        for it in range(max_sweeps):
            es = [optimize_twosite_projected(ctx, True, st, i, 0.1 * tole, lowers, idm) for i in range(N - 1)]
            es += [optimize_twosite_projected(ctx, False, st, i, 0.1 * tole, lowers, idm) for i in range(N - 1, 0, -1)]
            e_sweep = min(es)
            if verbose:
                print(f"root {r} sweep {it}: E = {e_sweep:.14f}", flush=True)
            if it > 0 and abs(e_sweep - e_prev) < tole:
                break
            e_prev = e_sweep
        energies.append(e_sweep)
        states.append(st)
    return energies, states
