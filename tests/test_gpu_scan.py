"""Batched scan (needs a GPU): chains of different lengths and couplings swept in
lockstep through optimize_twosite_merged_batch (grouped tensor-core H_eff*psi across
chains) agree with the same chains swept one by one, and with exact diagonalisation
where the bond dimension is exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SPECS = [(6, 4.0, -1.0), (8, 2.5, -1.0), (7, 6.0, -1.0), (10, 1.0, -1.0)]


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    c = core.Context(0)
    yield c
    core.set_precision(c, core.FP64)


@pytest.mark.parametrize("precision", ["split", "fp64"])
def test_batched_sweeps_match_sequential(ctx, precision):
    from oracle import ed
    from mpsxx_gb300 import core, scan

    core.set_precision(ctx, core.SPLIT_TF32 if precision == "split" else core.FP64)
    try:
        batched = scan.make_chains(ctx, SPECS, 16)
        single = scan.make_chains(ctx, SPECS, 16)
        sched = [16, 32, 64, 64]
        for M in sched:
            scan.sweep_batched(ctx, batched, M, 1e-10)
            scan.sweep_sequential(ctx, single, M, 1e-10)
    finally:
        core.set_precision(ctx, core.FP64)
    for b, s in zip(batched, single):
        print(precision, b.L, b.U, "batched", b.energies[-1], "single", s.energies[-1])
        assert abs(b.energies[-1] - s.energies[-1]) < 1e-8
    # L=6 with M=64 is exact
    exact = ed.hubbard_ground_energy(6, -1.0, 4.0, 3, 3)[0]
    assert abs(batched[0].energies[-1] - exact) < 1e-9


def test_batched_bond_steps_on_full_tiles_match_single_steps(ctx):
    """Two QC bonds (n=12, M=256, different integrals; states converged by four sweeps)
    advanced in one batched step — grouped split H_eff*psi over full 128x128
    tensor-core tiles and tails — give the energies of the same bond steps taken one at
    a time from identical inputs to 1e-9 Eh (split precision with the FP64 anchor)."""
    from mpsxx_gb300 import core, dmrg, mpogen

    bonds = []
    core.set_precision(ctx, core.SPLIT_TF32)
    try:
        for seed in (5, 6):
            h, eri = mpogen.synthetic_qc_integrals(12, 24, seed)
            mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
            st = dmrg.make_initial_state(ctx, mpo, 12, 0, 256)
            for _ in range(4):
                dmrg.make_sweep(ctx, st, 1e-9)
            dmrg.advance_left(ctx, st, 5)
            bonds.append(st)
    finally:
        core.set_precision(ctx, core.FP64)
    tole = 1e-9
    core.set_precision(ctx, core.SPLIT_TF32)
    try:
        args = [(st.mpo[5], st.mpo[6], st.lenv[5], st.renv[6], st.wave[5], st.wave[6]) for st in bonds]
        single = [core.optimize_twosite_merged(ctx, True, *a, 0.1 * tole, 256) for a in args]
        e, env, nl, nr, stats = core.optimize_twosite_merged_batch(ctx, [True, True], *[list(x) for x in zip(*args)],
                                                                   0.1 * tole, 256)
    finally:
        core.set_precision(ctx, core.FP64)
    for b, (es, _, _, _, ss) in enumerate(single):
        print("bond", b, "batched", e[b], stats[b]["converged"], "single", es, ss["converged"])
        assert stats[b]["converged"] and ss["converged"]
        assert abs(e[b] - es) < 1e-9
