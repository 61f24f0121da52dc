"""CPU oracle for the two-site DMRG hot path (test infrastructure only).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package; the product path never does.
"""
from .qsd import QSDArray  # noqa: F401


def from_site_dict(d) -> "QSDArray":
    """Oracle tensor from the neutral MPO/site exchange dictionary."""
    a = QSDArray(tuple(d["q"]), d["qshape"], d["dshape"])
    a.blocks = {int(t): b.copy() for t, b in d["blocks"].items()}
    return a
