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
