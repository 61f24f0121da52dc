"""Which block operators a two-site sweep holds, and that every bond gets current ones
(host logic of ``dmrg.make_sweep``, no GPU).

The library calls are replaced by stand-ins that track provenance: a site tensor is a
(site, version) pair, the left block operator of site j is the tuple of the versions of
sites 0..j-1 it was built from, the right one of site j those of sites j+1..N-1.  A bond
step checks that it received the operators of the current site tensors and returns new
versions; the rebuild path (merged operator + renormalisation) composes the same
tuples.  So a stale or wrongly rebuilt operator fails the run, and the count of
operators held after each sweep shows what checkpointing saves.
"""
import itertools

import pytest

from mpsxx_gb300 import dmrg


class FakeCore:
    def __init__(self):
        self.version = itertools.count(1)
        self.st = None
        self.bonds = 0

    def left(self, j):
        return ("L",) + tuple(self.st.wave[m][1] for m in range(j))

    def right(self, j):
        return ("R",) + tuple(self.st.wave[m][1] for m in range(j + 1, len(self.st.wave)))

    def optimize_twosite_merged(self, ctx, forward, lmpo, rmpo, lopr, ropr, lwfn, rwfn, tole, M, noise=0.0):
        i = lmpo
        assert rmpo == i + 1
        assert lwfn == self.st.wave[i] and rwfn == self.st.wave[i + 1]
        assert lopr == self.left(i), f"bond ({i},{i + 1}): stale left operator"
        assert ropr == self.right(i + 1), f"bond ({i},{i + 1}): stale right operator"
        nl, nr = (i, next(self.version)), (i + 1, next(self.version))
        env = lopr + (nl[1],) if forward else ("R", nr[1]) + ropr[1:]
        self.bonds += 1
        stats = {"n_sigma": 1, "sigma_flops": 0.0, "t_merge": 0.0, "t_diag": 0.0, "t_davidson": 0.0, "t_svd": 0.0,
                 "t_renorm": 0.0, "n_sigma_fp64": 0.0, "converged": 1.0}
        return -float(self.bonds), env, nl, nr, stats

    def compute_merged_operator(self, ctx, left, mpo, opr):
        return ("merged", left, mpo, opr)

    def merge_rows(self, ctx, wave):
        return ("rows", wave)

    def merge_cols(self, ctx, wave):
        return ("cols", wave)

    def renormalize(self, ctx, forward, merged, bra, ket):
        _, left, site, opr = merged
        assert left == forward and bra == ket and bra[1] == self.st.wave[site]
        assert bra[1][0] == site
        if forward:
            return opr + (bra[1][1],)
        return ("R", bra[1][1]) + opr[1:]


def _state(fake, N):
    wave = [(j, next(fake.version)) for j in range(N)]
    st = dmrg.DeviceState(mpo=list(range(N)), wave=wave, lenv=[None] * N, renv=[None] * N, M=8)
    fake.st = st
    st.lenv[0] = fake.left(0)
    for j in range(N):
        st.renv[j] = fake.right(j)
    return st


@pytest.fixture
def fake(monkeypatch):
    f = FakeCore()
    for name in ("optimize_twosite_merged", "compute_merged_operator", "merge_rows", "merge_cols", "renormalize"):
        monkeypatch.setattr(dmrg.core, name, getattr(f, name))
    return f


@pytest.mark.parametrize("N", [2, 3, 7, 12])
@pytest.mark.parametrize("k", [0, 1, 2, 3, 5])
def test_every_bond_gets_current_operators(fake, N, k):
    st = _state(fake, N)
    for sweep in range(3):
        log = dmrg.make_sweep(None, st, 1e-9, env_checkpoint=k)
        assert len(log.bond_energies) == 2 * (N - 1)
        # after a sweep: centre at site 0, the right operators current where held
        for j in range(N):
            if st.renv[j] is not None:
                assert st.renv[j] == fake.right(j)
        assert st.lenv[0] == fake.left(0)
        assert all(x is None for x in st.lenv[1:])
        assert st.renv[N - 1] is not None and (N < 3 or st.renv[1] is not None)


def test_checkpointing_holds_fewer_operators_and_rebuilds_each_once_per_pass(fake):
    N = 24
    held, rebuilt = {}, {}
    for k in (0, 4):
        st = _state(fake, N)
        peak = 0

        def hook(forward, i, e, stats):
            nonlocal peak
            peak = max(peak, sum(x is not None for x in st.lenv + st.renv))

        dmrg.make_sweep(None, st, 1e-9, env_checkpoint=k)  # the start holds every right operator
        log = dmrg.make_sweep(None, st, 1e-9, bond_hook=hook, env_checkpoint=k)
        held[k] = peak
        rebuilt[k] = log.times.get("env_rebuilt", 0.0)
    print("peak operators held", held, "rebuilt per sweep", rebuilt)
    assert rebuilt[0] == 0.0
    # each dropped operator is rebuilt once per pass: (N - 2) - kept ones, both passes
    assert 0 < rebuilt[4] <= 2 * (N - 2)
    assert held[0] <= N + 2
    assert held[4] <= 2 * (N // 4) + 2 * 4 + 4
    assert held[4] < held[0]


def test_fill_right_envs_restores_every_operator_after_a_checkpointed_sweep(fake):
    N = 11
    st = _state(fake, N)
    for _ in range(2):
        dmrg.make_sweep(None, st, 1e-9, env_checkpoint=3)
    assert any(x is None for x in st.renv)
    dmrg.fill_right_envs(None, st)
    assert all(st.renv[j] == fake.right(j) for j in range(N))
