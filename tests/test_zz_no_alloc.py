"""The allocation-free multi-dot entry point against the regular path (needs a GPU).

mpsxx_multidot_noalloc serves callers that cannot call cudaMalloc while they run
(a host application that owns the device memory through its own pool, a loop that
cannot afford an allocation's device-wide synchronisation): its reduction scratch
is a fixed array inside the library.
This file is collected last so that a failure here cannot hide any other test.
Tolerance: 1e-12 relative, the FP64 reduction order differs from NumPy's.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def vec_tensor(ctx, data):
    from mpsxx_gb300 import core

    t = core.Tensor.create(ctx, (0, 0), [[(0, 0)]], [[int(data.size)]])
    t.upload(data)
    return t


def test_multidot_noalloc_matches_regular_entry_point_twice():
    import torch

    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import check, lib

    ctx = core.Context(0)
    rng = np.random.default_rng(11)
    n = 300_001
    for call, (nx, ny) in enumerate([(3, 4), (10, 1)]):
        X = rng.standard_normal((nx, n))
        Y = rng.standard_normal((ny, n))
        tx, ty = vec_tensor(ctx, X.ravel()), vec_tensor(ctx, Y.ravel())
        out = vec_tensor(ctx, np.full(nx * ny, np.nan))
        check(lib().mpsxx_multidot_noalloc(C.c_void_p(tx.device_ptr()), nx, C.c_void_p(ty.device_ptr()), ny, n, n,
                                           C.c_void_p(out.device_ptr()), None))
        torch.cuda.synchronize()
        got = out.download().reshape(nx, ny)
        ref = X @ Y.T
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(X)) * np.max(np.abs(Y)) * n
        # against the regular entry point: mpsxx_normalize returns ||x|| through the
        # same reduction with context-owned scratch
        self_dot = vec_tensor(ctx, np.full(1, np.nan))
        check(lib().mpsxx_multidot_noalloc(C.c_void_p(tx.device_ptr()), 1, C.c_void_p(tx.device_ptr()), 1, n, n,
                                           C.c_void_p(self_dot.device_ptr()), None))
        torch.cuda.synchronize()
        x0 = vec_tensor(ctx, X[0].copy())
        norm = core.normalize(ctx, x0)
        assert abs(np.sqrt(self_dot.download()[0]) - norm) <= 1e-12 * norm, call


def test_multidot_noalloc_rejects_oversized_requests():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import MpsxxError, check, lib

    ctx = core.Context(0)
    t = vec_tensor(ctx, np.ones(16))
    out = vec_tensor(ctx, np.zeros(121))
    with pytest.raises(MpsxxError) as ei:
        check(lib().mpsxx_multidot_noalloc(C.c_void_p(t.device_ptr()), 11, C.c_void_p(t.device_ptr()), 1, 1, 1,
                                           C.c_void_p(out.device_ptr()), None))
    assert ei.value.code == 5 and "10 x 10" in str(ei.value)
