"""Batched parameter scan: many independent DMRG chains swept in lockstep.

Every chain runs the two-site sweep of ``dmrg.make_sweep`` (src/make_sweep.cpp:12-253)
with its own Hamiltonian and length.  Bond step k of the sweep is taken for all
chains that have one at the same time, through ``optimize_twosite_merged_batch``:
their Davidson iterations share one grouped tensor-core launch per H_eff*psi stage.
Chains of different lengths simply drop out of the later steps of a sweep.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import List, Sequence

import numpy as np

from . import core, dmrg
from .core import Context


@dataclass
class Chain:
    L: int
    U: float
    t: float
    st: dmrg.DeviceState
    energies: List[float] = field(default_factory=list)


def make_chains(ctx: Context, specs: Sequence[tuple], M0: int) -> List[Chain]:
    """specs: (L, U, t) per chain; half filling (N = L) with the smallest |Sz| (0 for
    even L, 1/2 for odd L); the reference's initial state."""
    from .mpogen import hubbard_mpo

    chains = []
    for L, U, t in specs:
        mpo = [core.Tensor.from_dict(ctx, d) for d in hubbard_mpo(L, t, U)]
        chains.append(Chain(L, U, t, dmrg.make_initial_state(ctx, mpo, L, L % 2, M0)))
    # room for a whole sweep's plans of every chain (two merged operators per bond step),
    # so that converged sweeps reuse them
    steps = sum(2 * (L - 1) for L, _, _ in specs)
    ctx.set_plan_cache(max(512, 4 * steps))
    return chains


def _bond(st: dmrg.DeviceState, k: int):
    """Bond step k of a sweep: forward bonds 0..N-2, then backward N-1..1."""
    N = len(st.mpo)
    if k < N - 1:
        return True, k
    return False, N - 1 - (k - (N - 1))


def sweep_batched(ctx: Context, chains: List[Chain], M: int, tole: float) -> dict:
    """One sweep of every chain with bond dimension M, bond steps batched across chains."""
    t0 = time.perf_counter()
    nsteps = max(2 * (c.L - 1) for c in chains)
    bond_e = [[] for _ in chains]
    nsig = 0
    for c in chains:
        c.st.M = M
    for k in range(nsteps):
        act = [i for i, c in enumerate(chains) if k < 2 * (c.L - 1)]
        fw, lm, rm, lo, ro, lw, rw = [], [], [], [], [], [], []
        for i in act:
            st = chains[i].st
            f, b = _bond(st, k)
            j = b if f else b - 1  # left site of the bond
            fw.append(f)
            lm.append(st.mpo[j])
            rm.append(st.mpo[j + 1])
            lo.append(st.lenv[j])
            ro.append(st.renv[j + 1])
            lw.append(st.wave[j])
            rw.append(st.wave[j + 1])
        e, env, nl, nr, stats = core.optimize_twosite_merged_batch(ctx, fw, lm, rm, lo, ro, lw, rw, 0.1 * tole, M)
        for a, i in enumerate(act):
            st = chains[i].st
            f, b = _bond(st, k)
            j = b if f else b - 1
            if f:
                st.lenv[j + 1] = env[a]
            else:
                st.renv[j] = env[a]
            st.wave[j], st.wave[j + 1] = nl[a], nr[a]
            bond_e[i].append(float(e[a]))
            nsig += int(stats[a]["n_sigma"])
    for i, c in enumerate(chains):
        c.energies.append(min(bond_e[i]))
    return {"seconds": time.perf_counter() - t0, "n_sigma": nsig, "bond_steps": nsteps}


def sweep_sequential(ctx: Context, chains: List[Chain], M: int, tole: float) -> dict:
    """The same sweep chain after chain (one bond at a time, no batching)."""
    t0 = time.perf_counter()
    nsig = 0
    for c in chains:
        c.st.M = M
        log = dmrg.make_sweep(ctx, c.st, tole)
        c.energies.append(log.energy)
        nsig += log.n_sigma
    return {"seconds": time.perf_counter() - t0, "n_sigma": nsig}


def m_schedule(m0: int, m1: int, sweeps: int, step: int = 16) -> List[int]:
    """Bond dimensions ramped linearly from m0 to m1 over the sweeps (multiples of step)."""
    return [int(round(m / step)) * step for m in np.linspace(m0, m1, sweeps)]


def random_specs(n: int, seed: int, lmin: int = 16, lmax: int = 32, umax: float = 8.0):
    rng = np.random.default_rng(seed)
    return [(int(rng.integers(lmin, lmax + 1)), float(rng.uniform(0.0, umax)), -1.0) for _ in range(n)]
