"""Block operators held during a two-site sweep (needs a GPU).

A sweep drops the operators it has made stale, and with ``env_checkpoint`` = k keeps
only every k-th of those the other pass needs, rebuilding the rest from the nearest
kept one.  The rebuilt operators come from the same products on the same operands, so
the sweep energies must not change: compared here at 1e-12 Eh (identical in practice).
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    return core.Context(0)


def _sweeps(ctx, mpo_d, n_elec, M, k, nsweeps):
    from mpsxx_gb300 import core, dmrg

    mpo = [core.Tensor.from_dict(ctx, d) for d in mpo_d]
    st = dmrg.make_initial_state(ctx, mpo, n_elec, 0, M)
    logs = [dmrg.make_sweep(ctx, st, 1e-9, env_checkpoint=k) for _ in range(nsweeps)]
    return logs, st


@pytest.mark.parametrize("k", [2, 3])
def test_checkpointed_environments_leave_the_sweep_unchanged(ctx, k):
    from mpsxx_gb300 import core, mpogen

    core.set_precision(ctx, core.FP64)
    h, eri = mpogen.synthetic_qc_integrals(10, 20, 2)
    mpo_d = mpogen.qc_mpo(h, eri)
    full, st_full = _sweeps(ctx, mpo_d, 10, 64, 0, 3)
    ckpt, st_ckpt = _sweeps(ctx, mpo_d, 10, 64, k, 3)
    for a, b in zip(full, ckpt):
        print("sweep", a.energy, b.energy - a.energy, b.times.get("env_rebuilt"))
        assert abs(a.energy - b.energy) < 1e-12
        assert max(abs(x - y) for x, y in zip(a.bond_energies, b.bond_energies)) < 1e-12
    assert all(log.times.get("env_rebuilt", 0) > 0 for log in ckpt)
    assert "env_rebuilt" not in full[-1].times
    N = len(mpo_d)
    # after a sweep: the right operators of every site (full), of the kept sites (checkpointed)
    held_full = sum(x is not None for x in st_full.lenv + st_full.renv)
    held_ckpt = sum(x is not None for x in st_ckpt.lenv + st_ckpt.renv)
    assert held_full == N + 1  # R_0 .. R_{N-1} and the left boundary
    assert held_ckpt < held_full
    # the checkpointed state continues as the full one does
    from mpsxx_gb300 import dmrg

    e_full = dmrg.make_sweep(ctx, st_full, 1e-9).energy
    e_ckpt = dmrg.make_sweep(ctx, st_ckpt, 1e-9, env_checkpoint=k).energy
    assert abs(e_full - e_ckpt) < 1e-12


def test_dmrg_driver_with_checkpointed_operators_and_a_onesite_stage(ctx):
    """dmrg() with checkpointed operators in the two-site stage, then the one-site stage
    (which first rebuilds the dropped right operators): every sweep energy as without."""
    from mpsxx_gb300 import core, dmrg
    from mpsxx_gb300.mpogen import hubbard_mpo

    core.set_precision(ctx, core.FP64)
    mpo = hubbard_mpo(8, -1.0, 4.0)
    _, full = dmrg.dmrg(ctx, mpo, 8, 0, 32, 1e-10, 6, onesite=True)
    _, ckpt = dmrg.dmrg(ctx, mpo, 8, 0, 32, 1e-10, 6, onesite=True, env_checkpoint=3)
    assert [log.kind for log in full] == [log.kind for log in ckpt]
    assert max(abs(a.energy - b.energy) for a, b in zip(full, ckpt)) < 1e-12
