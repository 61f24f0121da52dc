"""Python mirror of the reference's hot-path call surface over the C ABI.

``Tensor`` is a device-resident block-sparse QSDArray (see include/mpsxx_gb300.h
for the layout); the free functions keep the reference's names and argument
meaning (src/compute_sigma_vector.hpp, src/renormalize.hpp,
src/compute_diagonal_elements.hpp, src/diagonalize.hpp, src/canonicalize.hpp,
src/optimize.hpp).  Errors raise ``MpsxxError`` carrying the C status code.
"""
from __future__ import annotations

import ctypes as C
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from ._lib import check, lib

Q = Tuple[int, int]


def _i32(a) -> C.Array:
    arr = (C.c_int * max(1, len(a)))(*[int(x) for x in a])
    return arr


class Context:
    """One device and one CUDA stream (``stream`` is a raw cudaStream_t or None)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        h = C.c_void_p()
        check(lib().mpsxx_context_create(int(device), C.c_void_p(stream) if stream else None, C.byref(h)))
        self.h = h

    def sync(self):
        check(lib().mpsxx_context_sync(self.h))

    def counters(self):
        la = C.c_int64()
        fl = C.c_double()
        ca = C.c_int64()
        check(lib().mpsxx_context_counters(self.h, C.byref(la), C.byref(fl), C.byref(ca)))
        return {"launches": la.value, "sigma_flops": fl.value, "sigma_calls": ca.value}

    def set_truncation(self, tie_rtol: float = -1.0):
        """Relative tie window at the truncation cutoff (< 0: the precision's default)."""
        check(lib().mpsxx_context_set_truncation(self.h, float(tie_rtol)))

    def set_split_refinement(self, residual_floor: float = -1.0, rounds: int = -1):
        """Split-precision diagonalize: tensor-core Davidson down to |r|^2 < (floor*E)^2,
        then up to ``rounds`` FP64-anchored continuations (negative: defaults 1e-5, 2)."""
        check(lib().mpsxx_context_set_split_refinement(self.h, float(residual_floor), int(rounds)))

    def set_sigma_schedule(self, w_budget_bytes: int = -1, target_tiles: int = 0, fp32_intermediate: bool = False):
        """Fix the split H_eff*psi schedule (w scratch budget, tile target, FP32 L*psi
        intermediate split on chip); budget < 0: autotune."""
        check(lib().mpsxx_context_set_sigma_schedule(self.h, int(w_budget_bytes), int(target_tiles),
                                                     int(bool(fp32_intermediate))))

    def set_sigma_operator_format(self, fp32_operators: bool = False):
        """Merged operators of the split H_eff*psi packed as hi|lo TF32 tiles (default)
        or as FP32 tiles split on chip (half the bytes, slower); applies to plans made
        afterwards."""
        check(lib().mpsxx_context_set_sigma_operator_format(self.h, int(bool(fp32_operators))))

    def set_device_timeout(self, timeout_ns: int = 0):
        """Wait limit of the tensor-core kernels in ns (<= 0: the default 20 s)."""
        check(lib().mpsxx_context_set_device_timeout(self.h, int(timeout_ns)))

    def set_plan_cache(self, max_plans: int = 512):
        """Plans kept per kind before a cache is emptied."""
        check(lib().mpsxx_context_set_plan_cache(self.h, int(max_plans)))

    def set_svd_routes(self, jacobi_max_cols: int = -1, gram_max_dim: int = -1):
        """Routing of canonicalize's block SVDs (batched Jacobi / batched eigensolver /
        solver lanes); negative: defaults, 0: route off."""
        check(lib().mpsxx_context_set_svd_routes(self.h, int(jacobi_max_cols), int(gram_max_dim)))

    def tuning(self):
        """Last sigma autotuning: [(w scratch budget bytes, target tiles, FP32 intermediate,
        milliseconds), ...]."""
        buf = (C.c_double * 64)()
        cnt = C.c_int()
        check(lib().mpsxx_context_tuning(self.h, buf, 64, C.byref(cnt)))
        v = list(buf)[: min(cnt.value, 64)]
        return [(int(v[i]), int(v[i + 1]), bool(v[i + 2]), v[i + 3]) for i in range(0, len(v) - 3, 4)]

    def profile(self, enable=-1, reset=False):
        """Phase timers in seconds (PHASE_NAMES); enable=1/0 switches timing on/off."""
        t = (C.c_double * len(PHASE_NAMES))()
        cnt = C.c_int()
        check(lib().mpsxx_context_profile(self.h, int(enable), int(bool(reset)), t, len(PHASE_NAMES), C.byref(cnt)))
        assert cnt.value == len(PHASE_NAMES)
        return dict(zip(PHASE_NAMES, list(t)))

    def close(self):
        if getattr(self, "h", None):
            lib().mpsxx_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tensor:
    """Block-sparse quantum-number tensor held by the library (device or host-only)."""

    def __init__(self, handle: C.c_void_p, ctx: Optional[Context]):
        self.h = handle
        self.ctx = ctx  # keeps the context alive

    # -- construction ---------------------------------------------------------
    @classmethod
    def create(cls, ctx: Optional[Context], q: Q, qshape: Sequence[Sequence[Q]], dshape: Sequence[Sequence[int]],
               tags: Optional[Sequence[int]] = None) -> "Tensor":
        rank = len(qshape)
        nsec = [len(x) for x in qshape]
        qn = [v for x in qshape for qq in x for v in qq]
        dims = [d for x in dshape for d in x]
        h = C.c_void_p()
        if tags is None:
            nb, tg = -1, None
        else:
            tl = [int(t) for t in tags]
            nb = len(tl)
            tg = (C.c_int64 * max(1, nb))(*tl)
        check(lib().mpsxx_tensor_create(ctx.h if ctx else None, rank, _i32(q), _i32(nsec), _i32(qn), _i32(dims),
                                        nb, tg, C.byref(h)))
        return cls(h, ctx)

    @classmethod
    def from_dict(cls, ctx: Optional[Context], d: dict) -> "Tensor":
        """From the neutral exchange dict {"q","qshape","dshape","blocks": {tag: ndarray}}."""
        tags = sorted(int(t) for t in d["blocks"])
        t = cls.create(ctx, tuple(d["q"]), d["qshape"], d["dshape"], tags)
        t.upload_blocks(d["blocks"])
        return t

    def like(self) -> "Tensor":
        h = C.c_void_p()
        check(lib().mpsxx_tensor_create_like(self.ctx.h, self.h, C.byref(h)))
        return Tensor(h, self.ctx)

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().mpsxx_tensor_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # -- inspection -------------------------------------------------------------
    def info(self):
        r = C.c_int()
        q = (C.c_int * 2)()
        nb = C.c_int64()
        nnz = C.c_int64()
        check(lib().mpsxx_tensor_info(self.h, C.byref(r), q, C.byref(nb), C.byref(nnz)))
        return r.value, (q[0], q[1]), nb.value, nnz.value

    @property
    def rank(self) -> int:
        return self.info()[0]

    @property
    def q(self) -> Q:
        return self.info()[1]

    @property
    def nnz(self) -> int:
        return self.info()[3]

    def shape(self):
        rank, _, _, _ = self.info()
        nsec = (C.c_int * rank)()
        check(lib().mpsxx_tensor_shape(self.h, nsec, None, None))
        tot = sum(nsec)
        qn = (C.c_int * max(1, 2 * tot))()
        dims = (C.c_int * max(1, tot))()
        check(lib().mpsxx_tensor_shape(self.h, nsec, qn, dims))
        qshape, dshape, pos = [], [], 0
        for i in range(rank):
            qshape.append([(qn[2 * (pos + j)], qn[2 * (pos + j) + 1]) for j in range(nsec[i])])
            dshape.append([dims[pos + j] for j in range(nsec[i])])
            pos += nsec[i]
        return qshape, dshape

    def blocks(self):
        _, _, nb, _ = self.info()
        tags = np.zeros(max(1, nb), dtype=np.int64)
        offs = np.zeros(max(1, nb), dtype=np.int64)
        check(lib().mpsxx_tensor_blocks(self.h, tags.ctypes.data_as(C.POINTER(C.c_int64)),
                                        offs.ctypes.data_as(C.POINTER(C.c_int64))))
        return tags[:nb], offs[:nb]

    def device_ptr(self) -> int:
        p = C.POINTER(C.c_double)()
        check(lib().mpsxx_tensor_device_ptr(self.h, C.byref(p)))
        return C.cast(p, C.c_void_p).value or 0

    # -- data -------------------------------------------------------------------
    def upload(self, flat: np.ndarray):
        a = np.ascontiguousarray(flat, dtype=np.float64)
        if a.size != self.nnz:
            raise ValueError("upload: size does not match the tensor's nnz")
        check(lib().mpsxx_tensor_upload(self.h, a.ctypes.data_as(C.POINTER(C.c_double))))

    def download(self) -> np.ndarray:
        out = np.zeros(max(1, self.nnz), dtype=np.float64)
        check(lib().mpsxx_tensor_download(self.h, out.ctypes.data_as(C.POINTER(C.c_double))))
        return out[: self.nnz]

    def _strides(self, qshape):
        n = [len(x) for x in qshape]
        st = [1] * len(n)
        for i in range(len(n) - 2, -1, -1):
            st[i] = st[i + 1] * n[i + 1]
        return st

    def block_dims(self, tag: int, qshape=None, dshape=None):
        if qshape is None:
            qshape, dshape = self.shape()
        st = self._strides(qshape)
        idx = []
        for s in st:
            idx.append(tag // s)
            tag %= s
        return tuple(dshape[i][k] for i, k in enumerate(idx))

    def upload_blocks(self, blocks: Dict[int, np.ndarray]):
        qshape, dshape = self.shape()
        tags, offs = self.blocks()
        flat = np.zeros(self.nnz)
        for t, o in zip(tags, offs):
            b = blocks.get(int(t))
            if b is None:
                continue
            dims = self.block_dims(int(t), qshape, dshape)
            n = int(np.prod(dims))
            flat[o:o + n] = np.asarray(b, dtype=np.float64).reshape(-1)
        self.upload(flat)

    def to_blocks(self) -> Dict[int, np.ndarray]:
        qshape, dshape = self.shape()
        tags, offs = self.blocks()
        flat = self.download()
        out = {}
        for t, o in zip(tags, offs):
            dims = self.block_dims(int(t), qshape, dshape)
            n = int(np.prod(dims))
            out[int(t)] = flat[o:o + n].reshape(dims).copy()
        return out

    def to_dict(self) -> dict:
        qshape, dshape = self.shape()
        return {"q": self.q, "qshape": qshape, "dshape": dshape, "blocks": self.to_blocks()}


def _out():
    return C.c_void_p()


# ---------------------------------------------------------------------------
# planner
# ---------------------------------------------------------------------------

def gemm_tasks(transa: int, transb: int, a: Tensor, b: Tensor, c_rank: int):
    """Reference block-task list [(c_tag, [(a_tag, b_tag), ...]), ...] (host only)."""
    nt = C.c_int64()
    npr = C.c_int64()
    check(lib().mpsxx_gemm_tasks(transa, transb, a.h, b.h, c_rank, C.byref(nt), C.byref(npr), None, None, None, None))
    ct = np.zeros(max(1, nt.value), dtype=np.int64)
    pp = np.zeros(nt.value + 1, dtype=np.int64)
    at = np.zeros(max(1, npr.value), dtype=np.int64)
    bt = np.zeros(max(1, npr.value), dtype=np.int64)
    P = C.POINTER(C.c_int64)
    check(lib().mpsxx_gemm_tasks(transa, transb, a.h, b.h, c_rank, C.byref(nt), C.byref(npr), ct.ctypes.data_as(P),
                                 pp.ctypes.data_as(P), at.ctypes.data_as(P), bt.ctypes.data_as(P)))
    tasks = []
    for i in range(nt.value):
        tasks.append((int(ct[i]), [(int(at[p]), int(bt[p])) for p in range(pp[i], pp[i + 1])]))
    return tasks


# ---------------------------------------------------------------------------
# hot path (reference names)
# ---------------------------------------------------------------------------

def compute_sigma_vector(ctx: Context, lopr: Tensor, ropr: Tensor, wfn: Tensor, sgv: Tensor):
    check(lib().mpsxx_compute_sigma_vector(ctx.h, lopr.h, ropr.h, wfn.h, sgv.h))


def _in_out(ctx: Context, sgv: Optional[Tensor], call) -> Tensor:
    h = C.c_void_p(sgv.h.value if isinstance(sgv.h, C.c_void_p) else sgv.h) if sgv is not None else C.c_void_p()
    check(call(C.byref(h)))
    return sgv if sgv is not None else Tensor(h, ctx)


def compute_sigma_vector_onesite(ctx: Context, mpo: Tensor, lopr: Tensor, ropr: Tensor, wfn: Tensor,
                                 sgv: Optional[Tensor] = None) -> Tensor:
    """One-site H wfn with the site MPO (src/compute_sigma_vector.hpp:9-22); allocated
    when sgv is None, otherwise added to sgv (which grows by any missing blocks)."""
    return _in_out(ctx, sgv, lambda o: lib().mpsxx_compute_sigma_vector_onesite(ctx.h, mpo.h, lopr.h, ropr.h,
                                                                                  wfn.h, o))


def compute_sigma_vector_twosite(ctx: Context, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor, wfn: Tensor,
                                 sgv: Optional[Tensor] = None) -> Tensor:
    """Four-index two-site H wfn (src/compute_sigma_vector.hpp:53-70)."""
    return _in_out(ctx, sgv, lambda o: lib().mpsxx_compute_sigma_vector_twosite(ctx.h, lmpo.h, rmpo.h, lopr.h,
                                                                                  ropr.h, wfn.h, o))


def renormalize_mpo(ctx: Context, forward: bool, mpo: Tensor, opr0: Tensor, bra: Tensor, ket: Tensor,
                    opr1: Optional[Tensor] = None) -> Tensor:
    """renormalize with the site MPO (src/renormalize.hpp:10-32)."""
    return _in_out(ctx, opr1, lambda o: lib().mpsxx_renormalize_mpo(ctx.h, int(bool(forward)), mpo.h, opr0.h, bra.h,
                                                                     ket.h, o))


def renormalize_overlap(ctx: Context, forward: bool, sov0: Tensor, bra: Tensor, ket: Tensor,
                        sov1: Optional[Tensor] = None) -> Tensor:
    """renormalize an overlap matrix (src/renormalize.hpp:35-54)."""
    return _in_out(ctx, sov1, lambda o: lib().mpsxx_renormalize_overlap(ctx.h, int(bool(forward)), sov0.h, bra.h,
                                                                         ket.h, o))


def compute_guesswave(ctx: Context, forward: bool, mps0: Tensor, wfn0: Tensor, mps1: Tensor,
                      wfn1: Optional[Tensor] = None) -> Tensor:
    """compute_guesswave (src/compute_guesswave.hpp:11-38): the one-site centre moved to
    the next site (forward: (L^+ C) R; backward: L (C R^+)), allocate-or-accumulate."""
    return _in_out(ctx, wfn1, lambda o: lib().mpsxx_compute_guesswave(ctx.h, int(bool(forward)), mps0.h, wfn0.h,
                                                                       mps1.h, o))


def compute_diagonal_elements_onesite(ctx: Context, mpo: Tensor, lopr: Tensor, ropr: Tensor, diag: Tensor):
    """diag = one-site diagonal (src/compute_diagonal_elements.hpp:10-32): as the
    reference's Copy(scr, diag, 1), diag's previous blocks are dropped and it holds the
    computed blocks its quantum numbers allow (sum operator groups with
    Tensor.accumulate on separate results)."""
    check(lib().mpsxx_compute_diagonal_elements_onesite(ctx.h, mpo.h, lopr.h, ropr.h, diag.h))


def compute_diagonal_elements_twosite(ctx: Context, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor,
                                      diag: Tensor):
    """diag = four-index two-site diagonal (src/compute_diagonal_elements.hpp:35-62),
    overwritten as by the reference's Copy(scr, diag, 1)."""
    check(lib().mpsxx_compute_diagonal_elements_twosite(ctx.h, lmpo.h, rmpo.h, lopr.h, ropr.h, diag.h))


def compute_sigma_vector_overlap(ctx: Context, lopr: Tensor, ropr: Tensor, wfn: Tensor,
                                 sgv: Optional[Tensor] = None) -> Tensor:
    """lopr wfn ropr^T for two-index overlap operators (src/compute_sigma_vector.hpp:24-35,
    72-83, 98-109)."""
    return _in_out(ctx, sgv, lambda o: lib().mpsxx_compute_sigma_vector_overlap(ctx.h, lopr.h, ropr.h, wfn.h, o))


SIGMA_PLAN_KEYS = ("flops_stage1", "flops_stage2", "tile_flops_stage1", "tile_flops_stage2", "slices_stage1",
                   "slices_stage2", "tiles_stage1", "tiles_stage2", "packed_bytes_L", "packed_bytes_R",
                   "packed_bytes_intermediate", "packed_bytes_psi", "intermediate_elements",
                   "flops_rows_padded_stage1", "flops_cols_padded_stage1", "flops_k_padded_stage1",
                   "flops_rows_padded_stage2", "flops_cols_padded_stage2", "flops_k_padded_stage2",
                   "tile_flops_64row_tail_stage1", "tile_flops_64row_tail_stage2", "tiles_64row_tail",
                   "tiles_64col_tail")


def sigma_plan_stats(ctx: Context, lopr: Tensor, ropr: Tensor, wfn: Tensor) -> dict:
    """Useful vs tensor-core tile work and packed bytes of the split H_eff*psi plan."""
    out = (C.c_double * len(SIGMA_PLAN_KEYS))()
    cnt = C.c_int()
    check(lib().mpsxx_sigma_plan_stats(ctx.h, lopr.h, ropr.h, wfn.h, out, len(SIGMA_PLAN_KEYS), C.byref(cnt)))
    return dict(zip(SIGMA_PLAN_KEYS, list(out)))


def compute_diagonal_elements(ctx: Context, lopr: Tensor, ropr: Tensor, diag: Tensor):
    check(lib().mpsxx_compute_diagonal_elements(ctx.h, lopr.h, ropr.h, diag.h))


def renormalize(ctx: Context, forward: bool, opr0: Tensor, bra: Tensor, ket: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_renormalize(ctx.h, int(bool(forward)), opr0.h, bra.h, ket.h, C.byref(o)))
    return Tensor(o, ctx)


def compute_merged_operator(ctx: Context, forward: bool, mpo: Tensor, opr: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_compute_merged_operator(ctx.h, int(bool(forward)), mpo.h, opr.h, C.byref(o)))
    return Tensor(o, ctx)


def diagonalize(ctx: Context, lopr: Tensor, ropr: Tensor, diag: Tensor, wfnc: Tensor, tol: float = 1e-8):
    e = C.c_double()
    st = (C.c_int * 4)()
    check(lib().mpsxx_diagonalize(ctx.h, lopr.h, ropr.h, diag.h, wfnc.h, float(tol), C.byref(e), st))
    return e.value, {"n_sigma": st[0], "macro": st[1], "micro": st[2], "converged": st[3]}


def diagonalize_projected(ctx: Context, lopr: Tensor, ropr: Tensor, diag: Tensor, wfnc: Tensor, tol: float,
                          S: Sequence[Tensor], H: Sequence[Tensor], E: Sequence[float]):
    """diagonalize with the lower roots (S_j, H_j, E_j) projected out."""
    n = len(S)
    e = C.c_double()
    st = (C.c_int * 4)()
    hs = lambda ts: (C.c_void_p * max(n, 1))(*[t.h.value if isinstance(t.h, C.c_void_p) else t.h for t in ts])  # noqa: E731
    ev = (C.c_double * max(n, 1))(*E)
    check(lib().mpsxx_diagonalize_projected(ctx.h, lopr.h, ropr.h, diag.h, wfnc.h, float(tol), n, hs(S), hs(H), ev,
                                            C.byref(e), st))
    return e.value, {"n_sigma": st[0], "macro": st[1], "micro": st[2], "converged": st[3]}


def accumulate(ctx: Context, alpha: float, x: Tensor, y: Tensor):
    """y += alpha x (x's blocks must be stored in y)."""
    check(lib().mpsxx_tensor_accumulate(ctx.h, float(alpha), x.h, y.h))


def canonicalize(ctx: Context, forward: bool, wfnc: Tensor, M: int = 0, noise: float = 0.0):
    """Truncated SVD (src/canonicalize.hpp:88-106); with noise >= 1e-8 of
    make_noise(wfnc, noise), wfnc itself unchanged."""
    lo, ro = _out(), _out()
    check(lib().mpsxx_canonicalize(ctx.h, int(bool(forward)), wfnc.h, int(M), float(noise), C.byref(lo), C.byref(ro)))
    return Tensor(lo, ctx), Tensor(ro, ctx)


def make_noise(ctx: Context, wfnc: Tensor, noise: float):
    """wfnc += noise * noise array, in place (src/canonicalize.hpp:11-24); nothing
    when noise < 1e-8.  Blocks the noise array has and wfnc lacks are added."""
    check(lib().mpsxx_make_noise(ctx.h, wfnc.h, float(noise)))


def noise_sequence(n: int) -> np.ndarray:
    """The first n values make_noise draws (host only)."""
    out = np.zeros(max(int(n), 0))
    check(lib().mpsxx_noise_sequence(int(n), out.ctypes.data_as(C.POINTER(C.c_double))))
    return out


def gemm(ctx: Context, transa: int, transb: int, alpha: float, a: Tensor, b: Tensor, c_rank: int) -> Tensor:
    o = _out()
    check(lib().mpsxx_gemm(ctx.h, transa, transb, float(alpha), a.h, b.h, int(c_rank), C.byref(o)))
    return Tensor(o, ctx)


BATCH_STAT_KEYS = ("n_sigma", "n_sigma_fp64", "micro", "converged", "rnorm", "energy_split")


def optimize_twosite_merged_batch(ctx: Context, forward, lmpo, rmpo, lopr, ropr, lwfn, rwfn, tole: float, M,
                                  noise=0.0):
    """optimize_twosite_merged for n independent bonds at once (lists of n entries;
    forward, M and noise may be scalars).  Returns (energies, envs, new_lwfns, new_rwfns, stats)."""
    n = len(lmpo)
    fw = [int(bool(forward))] * n if isinstance(forward, (bool, int)) else [int(bool(f)) for f in forward]
    Ms = [int(M)] * n if isinstance(M, int) else [int(m) for m in M]
    nz = np.full(max(n, 1), float(noise)) if np.isscalar(noise) else np.asarray(noise, dtype=np.float64)

    def handles(ts):
        return (C.c_void_p * n)(*[t.h.value if isinstance(t.h, C.c_void_p) else t.h for t in ts])

    e = np.zeros(n)
    st = np.zeros(6 * max(n, 1))
    env, nl, nr = (C.c_void_p * n)(), (C.c_void_p * n)(), (C.c_void_p * n)()
    dp = C.POINTER(C.c_double)
    check(lib().mpsxx_optimize_twosite_merged_batch(
        ctx.h, n, (C.c_int * n)(*fw), handles(lmpo), handles(rmpo), handles(lopr), handles(ropr), handles(lwfn),
        handles(rwfn), float(tole), (C.c_int * n)(*Ms), nz.ctypes.data_as(dp), e.ctypes.data_as(dp), env, nl, nr,
        st.ctypes.data_as(dp)))
    wrap = lambda arr: [Tensor(C.c_void_p(arr[i]), ctx) for i in range(n)]  # noqa: E731
    stats = [dict(zip(BATCH_STAT_KEYS, st[6 * i:6 * i + 6])) for i in range(n)]
    return e, wrap(env), wrap(nl), wrap(nr), stats


def mpo_gradient(ctx: Context, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor, psi: Tensor):
    """dE/dW for both site MPOs of a bond, E = <psi|H_eff|psi> (psi normalised,
    merged two-site form); arrays in the MPOs' block order."""
    gl = np.zeros(lmpo.nnz)
    gr = np.zeros(rmpo.nnz)
    dp = C.POINTER(C.c_double)
    check(lib().mpsxx_mpo_gradient(ctx.h, lmpo.h, rmpo.h, lopr.h, ropr.h, psi.h, gl.ctypes.data_as(dp),
                                   gr.ctypes.data_as(dp)))
    return gl, gr


def merge_rows(ctx: Context, a: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_merge_rows(ctx.h, a.h, C.byref(o)))
    return Tensor(o, ctx)


def expand_rows(ctx: Context, b: Tensor, like: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_expand_rows(ctx.h, b.h, like.h, C.byref(o)))
    return Tensor(o, ctx)


def merge_cols(ctx: Context, a: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_merge_cols(ctx.h, a.h, C.byref(o)))
    return Tensor(o, ctx)


def expand_cols(ctx: Context, b: Tensor, like: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_expand_cols(ctx.h, b.h, like.h, C.byref(o)))
    return Tensor(o, ctx)


def normalize(ctx: Context, x: Tensor) -> float:
    n = C.c_double()
    check(lib().mpsxx_normalize(ctx.h, x.h, C.byref(n)))
    return n.value


def merge_wavefunction(ctx: Context, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor, lwfn: Tensor,
                       rwfn: Tensor) -> Tensor:
    o = _out()
    check(lib().mpsxx_merge_wavefunction(ctx.h, lmpo.h, rmpo.h, lopr.h, ropr.h, lwfn.h, rwfn.h, C.byref(o)))
    return Tensor(o, ctx)


def expand_wavefunction(ctx: Context, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor, lmat: Tensor,
                        rmat: Tensor):
    lo, ro = _out(), _out()
    check(lib().mpsxx_expand_wavefunction(ctx.h, lmpo.h, rmpo.h, lopr.h, ropr.h, lmat.h, rmat.h, C.byref(lo),
                                          C.byref(ro)))
    return Tensor(lo, ctx), Tensor(ro, ctx)


PHASE_NAMES = ("merge_plan", "merge_alloc", "merge_run", "wave_merge", "sigma_plan", "sigma", "davidson_rest",
               "svd_solve", "svd_select", "svd_post", "renorm_plan", "renorm_run", "sigma_fp64", "batch_group",
               "batch_plan", "svd_jacobi", "svd_gram")

BOND_STAT_KEYS = ("n_sigma", "sigma_flops", "t_merge", "t_diag", "t_davidson", "t_svd", "t_renorm", "converged",
                  "rnorm", "energy_split", "rnorm_fp64", "n_sigma_fp64")

FP64 = 0
SPLIT_TF32 = 1
SPLIT_TF32_ALL = 2  # H_eff*psi and the renormalisation contractions


def set_precision(ctx: Context, precision: int):
    """Bulk-contraction precision of the context: FP64 or SPLIT_TF32 (tensor cores)."""
    check(lib().mpsxx_context_set_precision(ctx.h, int(precision)))


def get_precision(ctx: Context) -> int:
    v = C.c_int()
    check(lib().mpsxx_context_get_precision(ctx.h, C.byref(v)))
    return v.value


def optimize_twosite_merged(ctx: Context, forward: bool, lmpo: Tensor, rmpo: Tensor, lopr: Tensor, ropr: Tensor,
                            lwfn: Tensor, rwfn: Tensor, tole: float, M: int, noise: float = 0.0):
    e = C.c_double()
    env, nl, nr = _out(), _out(), _out()
    st = (C.c_double * 12)()
    check(lib().mpsxx_optimize_twosite_merged(ctx.h, int(bool(forward)), lmpo.h, rmpo.h, lopr.h, ropr.h, lwfn.h,
                                              rwfn.h, float(tole), int(M), float(noise), C.byref(e), C.byref(env),
                                              C.byref(nl), C.byref(nr), st))
    stats = dict(zip(BOND_STAT_KEYS, list(st)))
    return e.value, Tensor(env, ctx), Tensor(nl, ctx), Tensor(nr, ctx), stats
