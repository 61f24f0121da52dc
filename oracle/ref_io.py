"""Block-sparse tensor files exchanged with the compiled reference harness
(``oracle/ref/qsd_io.hpp``) and the reference's task-list dumps.

Test infrastructure for the oracle: only ``tests/`` (and the fixture generator
beside them) use it.  Tensors are the neutral exchange dict
``{"q": (p, s), "qshape": [[(p, s), ...], ...], "dshape": [[d, ...], ...],
"blocks": {tag: ndarray}}`` the oracle and the product share.

File layout (little-endian): ``"MQSD"``, int32 rank, int32 q.p, q.s; per index
int32 nsec and nsec x (int32 p, s, dim); int64 nblocks; per block int64 tag,
int64 size and size float64 values, row-major.
"""
from __future__ import annotations

import struct
from typing import Dict, List, Tuple

import numpy as np


def read_qsd(path: str) -> dict:
    with open(path, "rb") as f:
        buf = f.read()
    if buf[:4] != b"MQSD":
        raise ValueError(f"{path}: not a qsd file")
    off = 4
    rank, qp, qs = struct.unpack_from("<3i", buf, off)
    off += 12
    qshape, dshape = [], []
    for _ in range(rank):
        (ns,) = struct.unpack_from("<i", buf, off)
        off += 4
        v = np.frombuffer(buf, dtype="<i4", count=3 * ns, offset=off).reshape(ns, 3)
        off += 12 * ns
        qshape.append([(int(a), int(b)) for a, b, _ in v])
        dshape.append([int(d) for _, _, d in v])
    (nb,) = struct.unpack_from("<q", buf, off)
    off += 8
    strides = [1] * rank
    for i in range(rank - 2, -1, -1):
        strides[i] = strides[i + 1] * len(qshape[i + 1])
    blocks = {}
    for _ in range(nb):
        tag, size = struct.unpack_from("<2q", buf, off)
        off += 16
        idx = [(tag // strides[i]) % len(qshape[i]) for i in range(rank)]
        shape = tuple(dshape[i][idx[i]] for i in range(rank))
        blocks[int(tag)] = np.frombuffer(buf, dtype="<f8", count=size, offset=off).reshape(shape).copy()
        off += 8 * size
    return {"q": (qp, qs), "qshape": qshape, "dshape": dshape, "blocks": blocks}


def write_qsd(path: str, t: dict) -> None:
    rank = len(t["qshape"])
    out = [b"MQSD", struct.pack("<3i", rank, int(t["q"][0]), int(t["q"][1]))]
    for qs, ds in zip(t["qshape"], t["dshape"]):
        out.append(struct.pack("<i", len(qs)))
        out.append(np.array([(q[0], q[1], d) for q, d in zip(qs, ds)], dtype="<i4").tobytes())
    tags = sorted(int(k) for k in t["blocks"])
    out.append(struct.pack("<q", len(tags)))
    for tag in tags:
        b = np.ascontiguousarray(t["blocks"][tag], dtype="<f8")
        out.append(struct.pack("<2q", tag, b.size))
        out.append(b.tobytes())
    with open(path, "wb") as f:
        f.write(b"".join(out))


def read_tasks(path: str) -> Dict[str, List[Tuple[int, List[Tuple[int, int]]]]]:
    """Task lists written by the harness: {gemm name: [(c_tag, [(a_tag, b_tag), ...]), ...]}
    in the reference's enumeration order."""
    lists: Dict[str, list] = {}
    cur = None
    with open(path) as f:
        for line in f:
            w = line.split()
            if not w:
                continue
            if w[0] == "gemm":
                cur = lists.setdefault(w[1], [])
                continue
            c, npair = int(w[0]), int(w[1])
            v = [int(x) for x in w[2:]]
            assert len(v) == 2 * npair
            cur.append((c, [(v[2 * i], v[2 * i + 1]) for i in range(npair)]))
    return lists


def pack_tensor(name: str, t: dict, with_data: bool = True) -> Dict[str, np.ndarray]:
    """Arrays for an .npz archive: layout (and optionally the block values) of one tensor."""
    nsec = np.array([len(x) for x in t["qshape"]], dtype=np.int32)
    qs = np.array([q for x in t["qshape"] for q in x], dtype=np.int32).reshape(-1, 2)
    ds = np.array([d for x in t["dshape"] for d in x], dtype=np.int32)
    tags = np.array(sorted(int(k) for k in t["blocks"]), dtype=np.int64)
    out = {f"{name}.q": np.array(t["q"], dtype=np.int32), f"{name}.nsec": nsec, f"{name}.qshape": qs,
           f"{name}.dshape": ds, f"{name}.tags": tags}
    if with_data:
        out[f"{name}.data"] = (np.concatenate([np.ravel(t["blocks"][int(k)]) for k in tags])
                               if len(tags) else np.zeros(0))
    return out


def unpack_tensor(z, name: str) -> dict:
    """Inverse of ``pack_tensor``; blocks are zero-filled when no values were stored."""
    nsec = [int(x) for x in z[f"{name}.nsec"]]
    qs = [tuple(int(v) for v in r) for r in z[f"{name}.qshape"]]
    ds = [int(v) for v in z[f"{name}.dshape"]]
    qshape, dshape, o = [], [], 0
    for n in nsec:
        qshape.append(qs[o:o + n])
        dshape.append(ds[o:o + n])
        o += n
    rank = len(nsec)
    strides = [1] * rank
    for i in range(rank - 2, -1, -1):
        strides[i] = strides[i + 1] * nsec[i + 1]
    data = z[f"{name}.data"] if f"{name}.data" in z else None
    blocks, off = {}, 0
    for tag in (int(x) for x in z[f"{name}.tags"]):
        shape = tuple(dshape[i][(tag // strides[i]) % nsec[i]] for i in range(rank))
        size = int(np.prod(shape, dtype=np.int64))
        blocks[tag] = (data[off:off + size].reshape(shape).copy() if data is not None else np.zeros(shape))
        off += size
    q = tuple(int(v) for v in z[f"{name}.q"])
    return {"q": q, "qshape": qshape, "dshape": dshape, "blocks": blocks}


def pack_tasks(name: str, tasks) -> Dict[str, np.ndarray]:
    """A task list [(c, [(a, b), ...]), ...] as CSR arrays."""
    c = np.array([t[0] for t in tasks], dtype=np.int64)
    ptr = np.zeros(len(tasks) + 1, dtype=np.int64)
    ptr[1:] = np.cumsum([len(t[1]) for t in tasks])
    ab = np.array([p for t in tasks for p in t[1]], dtype=np.int64).reshape(-1, 2)
    return {f"{name}.c": c, f"{name}.ptr": ptr, f"{name}.ab": ab}


def unpack_tasks(z, name: str):
    c, ptr, ab = z[f"{name}.c"], z[f"{name}.ptr"], z[f"{name}.ab"]
    return [(int(c[i]), [(int(a), int(b)) for a, b in ab[ptr[i]:ptr[i + 1]]]) for i in range(len(c))]
