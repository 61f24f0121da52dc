"""Split-precision (3xTF32 tensor-core) path against the FP64 path (needs a GPU).

Tolerances written here: H_eff*psi in split precision within 2e-6 of the FP64
result relative to its largest magnitude (TF32 hi+lo keeps ~22 bits, FP32
accumulation spans one block pair); energies within 1e-8 Eh of the FP64 path
after the FP64 refinement step.
"""
import json
import os

import numpy as np
import pytest

from tests.bondcase import hubbard_bond, to_dict

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    c = core.Context(0)
    yield c
    core.set_precision(c, core.FP64)


def dev(ctx, a):
    from mpsxx_gb300 import core

    return core.Tensor.from_dict(ctx, to_dict(a))


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def sigma_both(ctx, L, R, P):
    from mpsxx_gb300 import core

    out = []
    for prec in (core.FP64, core.SPLIT_TF32):
        core.set_precision(ctx, prec)
        S = P.like()
        core.compute_sigma_vector(ctx, L, R, P, S)
        out.append(S.download())
    core.set_precision(ctx, core.FP64)
    return out


def test_split_sigma_matches_fp64_hubbard_bond(ctx):
    case = hubbard_bond()
    s64, s32 = sigma_both(ctx, dev(ctx, case["mL"]), dev(ctx, case["mR"]), dev(ctx, case["full"]))
    err = rel_err(s32, s64)
    print("hubbard bond split-vs-fp64 sigma rel err", err)
    assert err < 2e-6


def test_split_sigma_matches_fp64_qc_bond(ctx):
    """QC n=8 random-MPS bond: blocks larger than one 128x64 tile and split-K partials."""
    from mpsxx_gb300 import core, dmrg, mpogen

    h, eri = mpogen.synthetic_qc_integrals(8, 16, 5)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
    st = dmrg.make_random_state(ctx, mpo, 8, 0, 128, seed=4)
    dmrg.advance_left(ctx, st, 3)
    mL, mR, psi = dmrg.bond_operands(ctx, st, 3)
    s64, s32 = sigma_both(ctx, mL, mR, psi)
    err = rel_err(s32, s64)
    print("qc bond split-vs-fp64 sigma rel err", err, "nnz psi", psi.nnz)
    assert err < 2e-6


def test_split_sigma_tail_tiles_are_exercised(ctx):
    """A QC n=12, M=256 bond: its plan has full 128x128 tiles and 64-row and 64-column
    tail tiles (M=64 / N=64 MMAs, compact packing), and its split H_eff*psi matches
    FP64 within 2e-6 (the plan statistics count the tiles; no device data is read for
    that).  The smaller test bonds have tail tiles only."""
    from mpsxx_gb300 import core, dmrg, mpogen

    h, eri = mpogen.synthetic_qc_integrals(12, 24, 5)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
    st = dmrg.make_random_state(ctx, mpo, 12, 0, 256, seed=4)
    dmrg.advance_left(ctx, st, 5)
    mL, mR, psi = dmrg.bond_operands(ctx, st, 5)
    stats = core.sigma_plan_stats(ctx, mL, mR, psi)
    print({k: stats[k] for k in ("tiles_stage1", "tiles_stage2", "tiles_64row_tail", "tiles_64col_tail")})
    assert stats["tiles_64row_tail"] > 0 and stats["tiles_64col_tail"] > 0
    # and full 128-row / 128-column tiles as well
    assert stats["tiles_64row_tail"] < stats["tiles_stage1"] + stats["tiles_stage2"]
    assert stats["tiles_64col_tail"] < stats["tiles_stage1"] + stats["tiles_stage2"]
    s64, s32 = sigma_both(ctx, mL, mR, psi)
    assert rel_err(s32, s64) < 2e-6
    # every schedule on these tiles: FP32 intermediate in one pass, w groups in both
    # formats; the merged operators as pre-split hi|lo tiles (the default) and as FP32
    # tiles split on chip
    for fp32_ops in (True, False):
        ctx.set_sigma_operator_format(fp32_ops)
        for schedule in ((0, 152 * 8, True), (0, 152 * 8, False), (1 << 20, 0, True), (1 << 20, 0, False)):
            ctx.set_sigma_schedule(*schedule)
            try:
                _, s = sigma_both(ctx, mL, mR, psi)
            finally:
                ctx.set_sigma_schedule(-1)
            print("fp32 operators", fp32_ops, "schedule", schedule, rel_err(s, s64))
            assert rel_err(s, s64) < 2e-6
    ctx.set_sigma_operator_format(False)


def test_split_davidson_refined_energy_matches_fp64(ctx):
    from mpsxx_gb300 import core

    case = hubbard_bond()
    L, R = dev(ctx, case["mL"]), dev(ctx, case["mR"])
    energies = []
    for prec in (core.FP64, core.SPLIT_TF32):
        core.set_precision(ctx, prec)
        P = dev(ctx, case["full"])
        D = P.like()
        core.compute_diagonal_elements(ctx, L, R, D)
        e, st = core.diagonalize(ctx, L, R, D, P, 1e-11)
        energies.append(e)
    core.set_precision(ctx, core.FP64)
    assert abs(energies[1] - energies[0]) < 1e-9, energies


def test_split_dmrg_hubbard12_matches_fp64(ctx):
    """Hubbard L=12, U=4, M=64: split-precision sweeps reach the FP64 energies within 1e-8 Eh."""
    from mpsxx_gb300 import core, dmrg
    from mpsxx_gb300.mpogen import hubbard_mpo

    gold = json.load(open(os.path.join(HERE, "golden", "hubbard12_u4_m64.json")))
    core.set_precision(ctx, core.SPLIT_TF32)
    try:
        mpo = [core.Tensor.from_dict(ctx, d) for d in hubbard_mpo(12, -1.0, 4.0)]
        st = dmrg.make_initial_state(ctx, mpo, 12, 0, 64)
        es = [dmrg.make_sweep(ctx, st, gold["tole"]).energy for _ in gold["sweeps"]]
    finally:
        core.set_precision(ctx, core.FP64)
    print("split sweep energies - fp64 oracle:", [e - g["energy"] for e, g in zip(es, gold["sweeps"])])
    assert abs(es[-1] - gold["sweeps"][-1]["energy"]) < 1e-8


def _qc8_bond(ctx, i=3):
    """The operands of bond (i, i+1) of a converged QC n=8 M=64 state (FP64 sweeps)."""
    from mpsxx_gb300 import core, dmrg, mpogen

    h, eri = mpogen.synthetic_qc_integrals(8, 16, 3)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
    core.set_precision(ctx, core.FP64)
    st = dmrg.make_initial_state(ctx, mpo, 8, 0, 64)
    for _ in range(3):
        dmrg.make_sweep(ctx, st, 1e-9)
    dmrg.advance_left(ctx, st, i)  # orthogonality centre from site 0 to the bond
    return (st.mpo[i], st.mpo[i + 1], st.lenv[i], st.renv[i + 1], st.wave[i], st.wave[i + 1])


def _bond_step(ctx, prec, args, tole):
    from mpsxx_gb300 import core

    core.set_precision(ctx, prec)
    try:
        e, _, nl, nr, s = core.optimize_twosite_merged(ctx, True, *args, tole, 64)
    finally:
        core.set_precision(ctx, core.FP64)
    return e, s, nl, nr


def test_split_bond_step_refines_with_few_fp64_products(ctx):
    """One bond of a converged QC n=8 sweep from identical inputs: the split step's
    refined energy matches the FP64 step within 1e-9 Eh with at most two FP64
    H_eff*psi (the anchor, and a second one only if the continuation fills up)."""
    from mpsxx_gb300 import core

    args = _qc8_bond(ctx)
    e64, s64, _, _ = _bond_step(ctx, core.FP64, args, 1e-11)
    e32, s32, _, _ = _bond_step(ctx, core.SPLIT_TF32, args, 1e-11)
    print("bond step fp64", e64, s64["n_sigma"], "split", e32, s32["n_sigma"], s32["n_sigma_fp64"], s32["rnorm"])
    assert abs(e32 - e64) < 1e-9
    assert 1 <= s32["n_sigma_fp64"] <= 2
    assert s32["converged"] == 1


def test_split_bond_step_when_refinement_rounds_run_out(ctx):
    """The refinement's limits.  Without refinement rounds the step returns the split
    Davidson's energy (no FP64 product; within the operator's 1e-5 relative
    resolution of the FP64 step).  With a tolerance below FP64 rounding of |r|^2
    (1e-40) every round ends unconverged: the step still returns, reports
    converged = 0 with one FP64 anchor per round, and its energy — the FP64-anchored
    Rayleigh quotient of the last round — matches the converged FP64 step within
    1e-9 Eh; the new site tensors are finite."""
    from mpsxx_gb300 import core

    args = _qc8_bond(ctx)
    e64, _, _, _ = _bond_step(ctx, core.FP64, args, 1e-11)
    try:
        ctx.set_split_refinement(rounds=0)
        e0, s0, _, _ = _bond_step(ctx, core.SPLIT_TF32, args, 1e-11)
        ctx.set_split_refinement(rounds=2)
        e2, s2, nl, nr = _bond_step(ctx, core.SPLIT_TF32, args, 1e-40)
    finally:
        ctx.set_split_refinement()
    print("no rounds", e0 - e64, s0["n_sigma_fp64"], "rounds exhausted", e2 - e64, s2["n_sigma_fp64"], s2["rnorm"])
    assert s0["n_sigma_fp64"] == 0
    assert abs(e0 - e64) < 1e-5 * abs(e64)
    assert s2["converged"] == 0
    assert s2["n_sigma_fp64"] == 2
    assert abs(e2 - e64) < 1e-9
    assert np.all(np.isfinite(nl.download())) and np.all(np.isfinite(nr.download()))


def test_split_renormalize_matches_fp64_qc_bond(ctx):
    """Renormalisation contractions (U^T mL U forward, V mR V^T backward) in split
    precision within 2e-6 of FP64, relative to the largest magnitude."""
    from mpsxx_gb300 import core, dmrg, mpogen

    h, eri = mpogen.synthetic_qc_integrals(8, 16, 5)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
    st = dmrg.make_random_state(ctx, mpo, 8, 0, 128, seed=4)
    dmrg.advance_left(ctx, st, 3)
    mL, mR, psi = dmrg.bond_operands(ctx, st, 3)
    for forward in (True, False):
        U, V = core.canonicalize(ctx, forward, psi, 128)
        op, bra = (mL, U) if forward else (mR, V)
        out = {}
        try:
            for prec in (core.FP64, core.SPLIT_TF32_ALL):
                core.set_precision(ctx, prec)
                out[prec] = core.renormalize(ctx, forward, op, bra, bra).download()
        finally:
            core.set_precision(ctx, core.FP64)
        err = rel_err(out[core.SPLIT_TF32_ALL], out[core.FP64])
        print("renormalize forward" if forward else "renormalize backward", "split rel err", err)
        assert err < 2e-6


@pytest.mark.parametrize("fp32_ops", [True, False])
@pytest.mark.parametrize("schedule", [(0, 152 * 4, False), (256 * 1024, 0, False), (4 * 1024 * 1024, 152 * 2, False),
                                      (0, 152 * 8, True), (256 * 1024, 0, True)])
def test_split_sigma_schedules_agree(ctx, schedule, fp32_ops):
    """Every schedule of the split H_eff*psi (one pass over w with different split-K
    targets, and w processed in groups out of an L2-sized scratch, through the CUDA
    graph; the L*psi intermediate as hi|lo tiles or as FP32 tiles split on chip; the
    merged operators as FP32 tiles split on chip or as hi|lo tiles) gives the same
    result as FP64 within 2e-6."""
    from mpsxx_gb300 import core, dmrg, mpogen

    h, eri = mpogen.synthetic_qc_integrals(8, 16, 5)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h, eri)]
    st = dmrg.make_random_state(ctx, mpo, 8, 0, 128, seed=4)
    dmrg.advance_left(ctx, st, 3)
    mL, mR, psi = dmrg.bond_operands(ctx, st, 3)
    ctx.set_sigma_operator_format(fp32_ops)
    ctx.set_sigma_schedule(*schedule)
    try:
        s64, s32 = sigma_both(ctx, mL, mR, psi)
        # a second application reuses the plan (and its graph)
        core.set_precision(ctx, core.SPLIT_TF32)
        again = psi.like()
        core.compute_sigma_vector(ctx, mL, mR, psi, again)
        core.set_precision(ctx, core.FP64)
    finally:
        ctx.set_sigma_schedule(-1)
        ctx.set_sigma_operator_format(False)
    err = rel_err(s32, s64)
    print("schedule", schedule, "split-vs-fp64 rel err", err)
    assert err < 2e-6
    assert np.array_equal(again.download(), s32)


def test_split_sigma_wait_limit_reports_timeout_and_context_stays_usable(ctx):
    """Failure detection without a GPU fault: with a 1 ns wait limit the tensor-core
    kernel's first wait gives up (the limit is checked on entry), it drains its own
    copies and MMAs, frees its tensor memory and returns; the call reports
    DEVICE_TIMEOUT, and with the default limit back the same context computes the split
    H_eff*psi within 2e-6 of FP64."""
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import MpsxxError

    case = hubbard_bond()
    L, R, P = dev(ctx, case["mL"]), dev(ctx, case["mR"]), dev(ctx, case["full"])
    core.set_precision(ctx, core.SPLIT_TF32)
    ctx.set_device_timeout(1)
    try:
        S = P.like()
        with pytest.raises(MpsxxError) as err:
            core.compute_sigma_vector(ctx, L, R, P, S)
        assert "DEVICE_TIMEOUT" in str(err.value) or getattr(err.value, "code", None) == 4
    finally:
        ctx.set_device_timeout(0)
        core.set_precision(ctx, core.FP64)
    s64, s32 = sigma_both(ctx, L, R, P)
    assert rel_err(s32, s64) < 2e-6
