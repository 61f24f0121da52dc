"""C++ restatement of the reference's CPU H_eff*psi (oracle/cpu/cpu_sigma.cpp) behind
ctypes: the BTAS task enumeration, FLOP-sorted OpenMP task loop and one dgemm per
block pair, on OpenBLAS opened at run time.  Test infrastructure: tests/ and
bench.py's reference arm time and check with it; the product never loads it."""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess
from typing import Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(os.path.dirname(HERE), "_build")
LIB = os.path.join(BUILD, "libcpu_sigma.so")
_lib: Optional[C.CDLL] = None


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "cpu_sigma.cpp")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        subprocess.run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", src, "-o", LIB, "-ldl"],
                       check=True)
    return LIB


def blas_path() -> str:
    """scipy's bundled OpenBLAS (LP64, "scipy_" symbol prefix)."""
    import scipy

    libs = os.path.join(os.path.dirname(os.path.dirname(scipy.__file__)), "scipy.libs")
    cand = sorted(glob.glob(os.path.join(libs, "libscipy_openblas*.so*")))
    if not cand:
        raise RuntimeError("no OpenBLAS found beside scipy")
    return cand[0]


def load(threads: int = 0) -> C.CDLL:
    global _lib
    if _lib is None:
        lib = C.CDLL(build())
        lib.cpu_sigma_error.restype = C.c_char_p
        if lib.cpu_sigma_init(blas_path().encode(), int(threads)) != 0:
            raise RuntimeError(lib.cpu_sigma_error().decode())
        _lib = lib
    return _lib


def _flatten(t: dict):
    rank = len(t["qshape"])
    desc = [rank] + [len(x) for x in t["qshape"]] + [d for x in t["dshape"] for d in x]
    desc += [v for x in t["qshape"] for q in x for v in q] + [int(t["q"][0]), int(t["q"][1])]
    tags = np.array(sorted(int(k) for k in t["blocks"]), dtype=np.int64)
    desc.append(len(tags))
    sizes = np.array([t["blocks"][int(k)].size for k in tags], dtype=np.int64)
    offs = np.zeros(len(tags), dtype=np.int64)
    if len(tags):
        offs[1:] = np.cumsum(sizes)[:-1]
    data = (np.concatenate([np.ravel(t["blocks"][int(k)]) for k in tags]).astype(np.float64)
            if len(tags) else np.zeros(1))
    return np.array(desc, dtype=np.int32), tags, offs, data


def allowed_layout(t: dict) -> dict:
    """Every block of t's quantum shape allowed by its total quantum number and of
    non-zero size, zero-filled (the layout of a result the reference sizes itself)."""
    import itertools

    rank = len(t["qshape"])
    blocks = {}
    strides = [1] * rank
    for i in range(rank - 2, -1, -1):
        strides[i] = strides[i + 1] * len(t["qshape"][i + 1])
    for idx in itertools.product(*[range(len(x)) for x in t["qshape"]]):
        qp = sum(t["qshape"][i][k][0] for i, k in enumerate(idx))
        qs = sum(t["qshape"][i][k][1] for i, k in enumerate(idx))
        shape = tuple(t["dshape"][i][k] for i, k in enumerate(idx))
        if (qp, qs) == tuple(t["q"]) and min(shape) > 0:
            blocks[sum(k * s for k, s in zip(idx, strides))] = np.zeros(shape)
    return {"q": tuple(t["q"]), "qshape": t["qshape"], "dshape": t["dshape"], "blocks": blocks}


class Operands:
    """mL, mR, psi flattened once, so that repeated H_eff*psi calls time the product alone;
    sigma gets every allowed block of psi's quantum shape."""

    def __init__(self, mL: dict, mR: dict, psi: dict):
        self.L, self.R, self.P = _flatten(mL), _flatten(mR), _flatten(psi)
        self.sig = allowed_layout(psi)
        self.S = _flatten(self.sig)
        self.nnz = int(sum(b.size for b in self.sig["blocks"].values()))


def sigma(ops: Operands, threads: int = 0) -> Tuple[dict, float, float]:
    """sigma = H_eff psi as the reference computes it.  Returns (blocks in psi's layout,
    FLOPs of both Gemm's, seconds)."""
    lib = load(threads)
    out = np.zeros(max(1, ops.nnz))
    fl, sec = C.c_double(), C.c_double()
    i32, i64, f64 = C.POINTER(C.c_int), C.POINTER(C.c_int64), C.POINTER(C.c_double)

    def args(x):
        d, tg, of, da = x
        return (d.ctypes.data_as(i32), tg.ctypes.data_as(i64), of.ctypes.data_as(i64), da.ctypes.data_as(f64))

    d, tg, of, _ = ops.S
    rc = lib.cpu_sigma_run(*args(ops.L), *args(ops.R), *args(ops.P), d.ctypes.data_as(i32), tg.ctypes.data_as(i64),
                           of.ctypes.data_as(i64), out.ctypes.data_as(f64), C.byref(fl), C.byref(sec))
    if rc != 0:
        raise RuntimeError(lib.cpu_sigma_error().decode())
    blocks, off = {}, 0
    for k in sorted(int(t) for t in ops.sig["blocks"]):
        shp = ops.sig["blocks"][k].shape
        n = int(np.prod(shp, dtype=np.int64))
        blocks[k] = out[off:off + n].reshape(shp).copy()
        off += n
    return blocks, fl.value, sec.value


def threads() -> int:
    return int(load().cpu_sigma_threads())


def set_threads(n: int) -> None:
    """OpenMP threads of the following sigma runs (n <= 0: the process's default)."""
    load().cpu_sigma_set_threads(int(n))
