"""Host-side checks of the C ABI library (no GPU): symbol exports, block-task
enumeration bit-exact against the oracle's restatement of ST_Gemm_thread, and
the reference's error behaviour."""
import itertools
import os
import re

import numpy as np
import pytest

from tests.bondcase import hubbard_bond

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300._lib import lib as _lib

    return _lib()


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:int|const char\*)\s+(mpsxx_\w+)\s*\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from mpsxx_gb300._lib import SIGNATURES

    assert declared_symbols() <= set(SIGNATURES)


def host(a):
    from mpsxx_gb300 import core

    return core.Tensor.create(None, a.q, a.qshape, a.dshape, sorted(a.blocks))


def oracle_tasks(ta, tb, a, b, nc):
    from oracle import qsd as oq

    qc, cq, cd, K = oq.gemm_contract_qshape(ta, tb, a, b, nc)
    return oq.st_gemm_tasks(ta, tb, a, b, oq.QSDArray(qc, cq, cd), K)


def test_sigma_and_renormalize_enumeration_bit_exact(lib):
    from oracle import dmrg as od
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    mL, mR, full, psi, M = case["mL"], case["mR"], case["full"], case["psi"], case["M"]
    # sigma, stage 1: L(3) x psi(2)
    assert core.gemm_tasks(0, 0, host(mL), host(full), 3) == oracle_tasks("N", "N", mL, full, 3)
    # sigma, stage 2: scr1(3) x R(3)^T over (w, B')
    scr = oq.QSDArray()
    oq.gemm("N", "N", 1.0, mL, full, 1.0, scr, nc=3)
    t2 = oracle_tasks("N", "T", scr, mR, 2)
    assert sum(len(p) for _, p in t2) > len(t2)  # many pairs per output block
    assert core.gemm_tasks(0, 1, host(scr), host(mR), 2) == t2
    # renormalize forward (T,N then N,N) and backward (N,N then N,T)
    U, V, _ = od.canonicalize_merged(True, psi, M)
    Uc = U.conjugate()
    assert core.gemm_tasks(1, 0, host(Uc), host(mL), 3) == oracle_tasks("T", "N", Uc, mL, 3)
    s3 = oq.QSDArray()
    oq.gemm("T", "N", 1.0, Uc, mL, 1.0, s3, nc=3)
    assert core.gemm_tasks(0, 0, host(s3), host(U), 3) == oracle_tasks("N", "N", s3, U, 3)
    Vc = V.conjugate()
    assert core.gemm_tasks(0, 0, host(Vc), host(mR), 3) == oracle_tasks("N", "N", Vc, mR, 3)
    s5 = oq.QSDArray()
    oq.gemm("N", "N", 1.0, Vc, mR, 1.0, s5, nc=3)
    assert core.gemm_tasks(0, 1, host(s5), host(V), 3) == oracle_tasks("N", "T", s5, V, 3)


def random_pair(rng, ta, tb):
    """Random contractible (a, b) with random sector sets and random stored blocks."""
    from oracle import qsd as oq

    qs = [(-1, 0), (0, 0), (0, 0), (1, 0), (1, 2)]

    def pick(n):
        idx = rng.choice(len(qs), size=n, replace=True)
        return [qs[i] for i in idx]

    L, Mr = int(rng.integers(2, 4)), int(rng.integers(2, 4))
    K = int(rng.integers(1, min(L, Mr)))
    kq = [pick(int(rng.integers(1, 4))) for _ in range(K)]
    a_free = [pick(int(rng.integers(1, 4))) for _ in range(L - K)]
    b_free = [pick(int(rng.integers(1, 4))) for _ in range(Mr - K)]
    neg = lambda v: [(-x[0], -x[1]) for x in v]  # noqa: E731
    aq = (a_free + kq) if ta == "N" else (kq + a_free)
    bq = ([neg(v) for v in kq] + b_free) if tb == "N" else (b_free + [neg(v) for v in kq])
    def total(qshape):  # the charge of one random sector combination, so blocks exist
        return oq.qsum(v[int(rng.integers(len(v)))] for v in qshape)

    A = oq.QSDArray(total(aq), aq, [[int(rng.integers(1, 4)) for _ in v] for v in aq])
    B = oq.QSDArray(total(bq), bq, [[int(rng.integers(1, 4)) for _ in v] for v in bq])
    for T in (A, B):
        T.allocate(0.0)
        keep = [t for t in T.blocks if rng.random() < 0.7]
        T.blocks = {t: T.blocks[t] for t in keep}
    return A, B, L + Mr - 2 * K


@pytest.mark.parametrize("ta,tb", list(itertools.product("NT", "NT")))
def test_random_block_sets_enumeration_bit_exact(lib, ta, tb):
    from mpsxx_gb300 import core

    rng = np.random.default_rng(hash((ta, tb)) % 2**32)
    n_nonempty = 0
    for _ in range(40):
        A, B, nc = random_pair(rng, ta, tb)
        ref = oracle_tasks(ta, tb, A, B, nc)
        got = core.gemm_tasks(int(ta == "T"), int(tb == "T"), host(A), host(B), nc)
        assert got == ref
        n_nonempty += bool(ref)
    assert n_nonempty > 5


def test_empty_operand_gives_no_tasks(lib):
    from oracle import qsd as oq
    from mpsxx_gb300 import core

    case = hubbard_bond()
    empty = case["full"].empty_like()
    assert core.gemm_tasks(0, 0, host(case["mL"]), host(empty), 3) == []


def test_qshape_mismatch_raises_reference_message(lib):
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import MpsxxError

    a = core.Tensor.create(None, (0, 0), [[(1, 1)], [(0, 0)]], [[2], [3]])
    b = core.Tensor.create(None, (0, 0), [[(0, 0)], [(1, 1)]], [[3], [2]])  # index 0 must be -(0,0)... ok
    c = core.Tensor.create(None, (0, 0), [[(1, 0)], [(1, 1)]], [[3], [2]])
    core.gemm_tasks(0, 0, a, b, 2)
    with pytest.raises(MpsxxError) as ei:
        core.gemm_tasks(0, 0, a, c, 2)
    assert ei.value.code == 1
    assert "gemm_contract_qshape contraction of quantum numbers failed" in str(ei.value)


CPP_PROGRAM = r"""
#include <cstdio>
#include "mpsxx_gb300.hpp"
using namespace mpsxx::gb300;
int main() {
  // L[A,w,A'] (3 sectors, w: 2 operators) x psi[A',B] with host-only descriptors
  std::vector<std::vector<Sector>> ls = {{{0,0,2},{1,1,3},{2,0,1}}, {{0,0,1},{1,1,1}}, {{0,0,2},{-1,-1,3},{-2,0,1}}};
  std::vector<std::vector<Sector>> ps = {{{0,0,2},{1,1,3},{2,0,1}}, {{2,0,4},{1,-1,2},{0,0,3}}};
  QSDArray L(nullptr, 0, 0, ls), P(nullptr, 2, 0, ps);
  auto tasks = gemm_tasks(MPSXX_NOTRANS, MPSXX_NOTRANS, L, P, 3);
  size_t np = 0;
  for (auto& t : tasks) np += t.second.size();
  std::printf("%zu %zu %lld %lld\n", tasks.size(), np, (long long)L.nblocks(), (long long)P.nblocks());
  try {
    QSDArray bad(nullptr, 0, 0, ls, nullptr);
    gemm_tasks(MPSXX_NOTRANS, MPSXX_NOTRANS, bad, bad, 5);
  } catch (const std::runtime_error& e) {
    std::printf("error: %s\n", e.what());
  }
  return 0;
}
"""


def test_cpp_dropin_header_compiles_and_plans(lib, tmp_path):
    """The C++ drop-in header (reference names over gb300::QSDArray) builds against the
    library and reproduces the Python binding's enumeration; errors become exceptions."""
    import subprocess

    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import LIB_PATH

    src = tmp_path / "dropin.cpp"
    src.write_text(CPP_PROGRAM)
    exe = tmp_path / "dropin"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe),
                    "-L", str(LIB_PATH.parent), "-lmpsxx_gb300", f"-Wl,-rpath,{LIB_PATH.parent}"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    ntask, npair, nbl, nbp = (int(x) for x in out[0].split())
    L = core.Tensor.create(None, (0, 0), [[(0, 0), (1, 1), (2, 0)], [(0, 0), (1, 1)], [(0, 0), (-1, -1), (-2, 0)]],
                           [[2, 3, 1], [1, 1], [2, 3, 1]])
    P = core.Tensor.create(None, (2, 0), [[(0, 0), (1, 1), (2, 0)], [(2, 0), (1, -1), (0, 0)]], [[2, 3, 1], [4, 2, 3]])
    ref = core.gemm_tasks(0, 0, L, P, 3)
    assert (ntask, npair) == (len(ref), sum(len(p) for _, p in ref)) and ntask > 0
    assert nbl == L.info()[2] and nbp == P.info()[2]
    assert out[1].startswith("error: ") and "rank" in out[1]


def test_invalid_tensor_arguments_are_rejected(lib):
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import MpsxxError

    with pytest.raises(MpsxxError) as ei:  # tags must be ascending
        core.Tensor.create(None, (0, 0), [[(0, 0), (1, 1)], [(0, 0), (-1, -1)]], [[1, 1], [1, 1]], [3, 0])
    assert ei.value.code == 5
    with pytest.raises(MpsxxError) as ei:  # block not allowed by quantum numbers
        core.Tensor.create(None, (0, 0), [[(0, 0), (1, 1)], [(0, 0), (-1, -1)]], [[1, 1], [1, 1]], [1])
    assert ei.value.code == 1
