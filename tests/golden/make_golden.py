"""Regenerate the golden fixtures under tests/golden/ (run in the build container).

* ``reference_energies.json``: the known-answer energies the reference's own test
  logs hold (read as text from the mpsxx tree when it is present) plus the
  oracle's energies on the same Hamiltonians;
* ``hubbard12_u4_m64.json``: oracle sweep energies of the 12-site Hubbard chain
  (U=4, t=1, half filling, M=64, tole 1e-10, 4 sweeps) and its exact ground state.

Usage: python tests/golden/make_golden.py --reference-root PATH   (or MPSXX_REFERENCE_ROOT)
"""
from __future__ import annotations

import json
import os
import re
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import dmrg as od  # noqa: E402
from oracle import from_site_dict  # noqa: E402
from oracle.ed import hubbard_ground_energy  # noqa: E402
from mpsxx_gb300.mpogen import hubbard_mpo  # noqa: E402


def sweep_energies_from_log(path: str):
    """Final 'Sweep Energy' lines (one per root) of a reference run log."""
    vals = []
    with open(path) as f:
        for line in f:
            m = re.match(r"\s*Sweep Energy =\s*(-?\d+\.\d+)\s*$", line)
            if m:
                vals.append(m.group(1))
    return vals


def main():
    ref_root = os.environ.get("MPSXX_REFERENCE_ROOT", "")
    if "--reference-root" in sys.argv:
        ref_root = sys.argv[sys.argv.index("--reference-root") + 1]
    if not ref_root:
        sys.exit("--reference-root PATH (or MPSXX_REFERENCE_ROOT) is required")
    out = {}
    tests = os.path.join(ref_root, "dmrg", "tests")
    if os.path.isdir(tests):
        out["HUBBARD12_M200_roots"] = {"source": "dmrg/tests/hub12_dmrg.out",
                                       "energies": sweep_energies_from_log(os.path.join(tests, "hub12_dmrg.out"))}
        out["FCIDUMP12_M200_roots"] = {"source": "dmrg/tests/twodot.out",
                                       "energies": sweep_energies_from_log(os.path.join(tests, "twodot.out"))}
        out["INTGEN6_M200"] = {"source": "dmrg/tests/dmrg.out",
                               "energies": sweep_energies_from_log(os.path.join(tests, "dmrg.out"))[-1:]}
        # integral lines of the 16-orbital FCIDUMP that intgen.cpp wrote (header and core line excluded)
        import hashlib

        body = open(os.path.join(tests, "FCIDUMP")).read().splitlines()[4:-1]
        out["INTGEN16_FCIDUMP"] = {"source": "dmrg/tests/FCIDUMP", "lines": len(body),
                                   "sha256": hashlib.sha256("".join(l + "\n" for l in body).encode()).hexdigest()}
    # HUBBARD12: U=1, h_{i+1,i}=+1, 12 electrons (dmrg/tests/HUBBARD12)
    t0 = time.time()
    mpo = [from_site_dict(s) for s in hubbard_mpo(12, 1.0, 1.0)]
    st, logs = od.dmrg(mpo, 12, 0, 200, 1e-8, 10)
    out["HUBBARD12_M200_oracle"] = {"energy": logs[-1].energy, "sweeps": len(logs), "tole": 1e-8,
                                    "seconds": time.time() - t0}
    out["HUBBARD12_exact"] = {"energy": float(hubbard_ground_energy(12, 1.0, 1.0, 6, 6)[0])}
    with open(os.path.join(HERE, "reference_energies.json"), "w") as f:
        json.dump(out, f, indent=1)
    if "--reference-only" in sys.argv:
        return
    # config: Hubbard L=12, U=4, M=64, 4 sweeps, tole 1e-10
    mpo = [from_site_dict(s) for s in hubbard_mpo(12, -1.0, 4.0)]
    st = od.make_initial_state(mpo, 12, 0, 64)
    sweeps = []
    for it in range(4):
        log = od.make_sweep(st, 1e-10)
        sweeps.append({"energy": log.energy, "bond_energies": log.bond_energies, "n_sigma": log.n_sigma})
    ed = float(hubbard_ground_energy(12, -1.0, 4.0, 6, 6)[0])
    with open(os.path.join(HERE, "hubbard12_u4_m64.json"), "w") as f:
        json.dump({"L": 12, "U": 4.0, "t": -1.0, "M": 64, "tole": 1e-10, "sweeps": sweeps, "exact": ed}, f, indent=1)
    print("done")


if __name__ == "__main__":
    main()
