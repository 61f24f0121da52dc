"""compute_guesswave (src/compute_guesswave.hpp:11-38) on the device against the oracle,
through the C ABI (needs a GPU).  FP64: block data compared at 1e-12 relative to the
largest magnitude (the device sums in another order than the oracle's BLAS)."""
import numpy as np
import pytest

from tests.bondcase import to_dict

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core

    return core.Context(0)


def dev(ctx, a):
    from mpsxx_gb300 import core

    return core.Tensor.from_dict(ctx, to_dict(a))


def max_block_diff(ref_blocks, got_blocks):
    scale = max([float(np.max(np.abs(b))) for b in ref_blocks.values() if b.size] + [1e-300])
    err = 0.0
    for k in set(ref_blocks) | set(got_blocks):
        r, g = ref_blocks.get(k), got_blocks.get(k)
        r = np.zeros_like(g) if r is None else r
        g = np.zeros_like(r) if g is None else g
        err = max(err, float(np.max(np.abs(r - g))) if r.size else 0.0)
    return err / scale


@pytest.mark.parametrize("forward", [True, False])
def test_guesswave_matches_oracle(ctx, forward):
    """compute_guesswave (src/compute_guesswave.hpp:11-38) on random tensors with the
    layouts of a Hubbard bond's sites, allocated and accumulated."""
    from oracle import dmrg as od
    from oracle import qsd as oq
    from tests.bondcase import guesswave_case
    from mpsxx_gb300 import core

    L, C, R, rand_like = guesswave_case()
    mps0, wfn0 = (rand_like(L), rand_like(L)) if forward else (rand_like(R), rand_like(R))
    mps1 = rand_like(C)
    ref = od.compute_guesswave(forward, mps0, wfn0, mps1, oq.QSDArray())
    ops = [dev(ctx, x) for x in (mps0, wfn0, mps1)]
    got = core.compute_guesswave(ctx, forward, *ops)
    assert max_block_diff(ref.blocks, got.to_blocks()) < 1e-12
    acc = dev(ctx, C)
    core.compute_guesswave(ctx, forward, *ops, acc)
    expect = C.copy()
    oq.axpy(1.0, ref, expect)
    assert max_block_diff(expect.blocks, acc.to_blocks()) < 1e-12
