"""Generate the golden fixtures that pin the oracle and the CUDA path to the mpsxx
reference itself.

The reference is built from its own sources (``make -C oracle/ref``: stand-in Boost
headers, scipy's OpenBLAS) and run through its own programs: ``mpogen.x`` writes the
site MPOs from an FCIDUMP, ``dmrg.x`` sweeps with every bond's inputs and outputs
dumped (``oracle/ref/hooks_impl.cpp``), and ``ref_ops.x ops`` re-runs the hot-path
functions on a dumped bond, recording ST_Gemm_thread's task lists.

    python tests/golden/make_ref_fixtures.py --reference-root <mpsxx tree> --work <scratch dir>

Writes tests/golden/ref/{runs.json, tasks.npz, bonds.npz, mpo_qc8.npz, mpo_c2_bond.npz}.
Cases: C1 (Hubbard L=12, t=1, U=4, half filling, M=64, tole 1e-10, 4 sweeps), a
synthetic QC Hamiltonian (n=8, K=16, seed 1, 8 electrons, M=64, tole 1e-9,
3 sweeps) and the reference's FCIDUMP12 test input (M=64, 2 sweeps, energies only);
and the reference's MPO of C2 (n=20, K=40, seed 1), of which the two sites of the
middle bond (9, 10) are kept as the bench's operator.
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import re
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_io  # noqa: E402

OUT = os.path.join(HERE, "ref")
REF_BIN = os.path.join(ROOT, "oracle", "_ref")


def run(cmd, cwd, env=None, log=None):
    e = dict(os.environ)
    e.update(env or {})
    with open(log or os.devnull, "w") as f:
        subprocess.run(cmd, cwd=cwd, env=e, stdout=f, stderr=subprocess.STDOUT, check=True)


def hubbard_fcidump(path, L, t, U):
    from mpsxx_gb300 import mpogen

    h = np.zeros((L, L))
    for i in range(L - 1):
        h[i, i + 1] = h[i + 1, i] = -t
    eri = np.zeros((L, L, L, L))
    for i in range(L):
        eri[i, i, i, i] = U
    mpogen.write_fcidump(path, h, eri, L, 0, 0.0)


def qc_fcidump(path, n, K, seed):
    from mpsxx_gb300 import mpogen

    h1, eri = mpogen.synthetic_qc_integrals(n, K, seed)
    mpogen.write_fcidump(path, h1, eri, n, 0, 0.0)


def dmrg_case(work, name, fcidump_writer, N, elec, M, tole, maxiter, dump, threads):
    d = os.path.join(work, name)
    if os.path.isdir(d):
        shutil.rmtree(d)
    os.makedirs(d)
    fcidump_writer(os.path.join(d, "FCIDUMP"))
    run([os.path.join(REF_BIN, "mpogen.x"), "-f", "FCIDUMP", "-s", "."], d, log=os.path.join(d, "mpogen.log"))
    with open(os.path.join(d, "dmrg.conf"), "w") as f:
        f.write(f"N {N}\nM {M}\nelec {elec}\nspin 0\nnroots 1\ntwosite\nmaxiter {maxiter}\ntole {tole:.1e}\n")
    env = {"OMP_NUM_THREADS": str(threads), "OPENBLAS_NUM_THREADS": "1"}
    if dump:
        env["MPSXX_REF_DUMP"] = os.path.join(d, "dump")
    run([os.path.join(REF_BIN, "dmrg.x"), "-i", "dmrg.conf", "-s", "."], d, env=env, log=os.path.join(d, "dmrg.log"))
    log = open(os.path.join(d, "dmrg.log")).read()
    sweeps = [float(x) for x in re.findall(r"Sweep Energy =\s+(-?[0-9.]+) \( delta", log)]
    bonds = [float(x) for x in re.findall(r"\n\t\t\tEnergy =\s+(-?[0-9.]+)", log)]
    return d, {"N": N, "elec": elec, "M": M, "tole": tole, "maxiter": maxiter, "sweep_energies": sweeps,
               "bond_energies": bonds}


def meta(bdir):
    m = {}
    for line in open(os.path.join(bdir, "meta.txt")):
        k, v = line.split()
        m[k] = float(v)
    return m


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=os.environ.get("MPSXX_REFERENCE_ROOT"),
                    help="the mpsxx source tree (or MPSXX_REFERENCE_ROOT)")
    ap.add_argument("--work", required=True, help="scratch directory for the reference runs")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    if not args.reference_root:
        sys.exit("--reference-root (or MPSXX_REFERENCE_ROOT) is required")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={args.reference_root}",
                    f"-j{args.threads}"], check=True, stdout=subprocess.DEVNULL)
    args.work = os.path.abspath(args.work)
    os.makedirs(args.work, exist_ok=True)
    os.makedirs(OUT, exist_ok=True)

    runs, tasks, bonds = {}, {}, {}
    cases = [
        ("c1", lambda p: hubbard_fcidump(p, 12, 1.0, 4.0), 12, 12, 64, 1e-10, 4, True),
        ("qc8", lambda p: qc_fcidump(p, 8, 16, 1), 8, 8, 64, 1e-9, 3, True),
        ("fcidump12", lambda p: shutil.copy(os.path.join(args.reference_root, "dmrg", "tests", "FCIDUMP12"), p),
         12, 12, 64, 1e-8, 2, False),
    ]
    keep = {"c1": {70, 75, 80, 86}, "qc8": None}
    for name, writer, N, elec, M, tole, maxiter, dump in cases:
        d, rec = dmrg_case(args.work, name, writer, N, elec, M, tole, maxiter, dump, args.threads)
        runs[name] = rec
        if not dump:
            continue
        bdirs = sorted(glob.glob(os.path.join(d, "dump", "bond_*")))
        rec["bond_meta"] = []
        nb = 2 * (N - 1)
        sel = keep[name] if keep[name] is not None else {len(bdirs) - nb + N // 2 - 1, len(bdirs) - N // 2}
        for k, b in enumerate(bdirs):
            subprocess.run([os.path.join(REF_BIN, "ref_ops.x"), "ops", b], check=True, stdout=subprocess.DEVNULL,
                           env=dict(os.environ, OMP_NUM_THREADS="1"))
            m = meta(b)
            rec["bond_meta"].append({"forward": int(m["forward"]), "energy": m["energy"], "M": int(m["M"])})
            key = f"{name}/{k:03d}"
            tl = ref_io.read_tasks(os.path.join(b, "tasks_sigma.ref.txt"))
            tl.update(ref_io.read_tasks(os.path.join(b, "tasks_renorm.ref.txt")))
            for g, lst in tl.items():
                tasks.update(ref_io.pack_tasks(f"{key}/{g}", lst))
            u = "lmat" if m["forward"] else "rmat"
            for t in ("mL", "mR", "psi", u):
                tasks.update(ref_io.pack_tensor(f"{key}/{t}", ref_io.read_qsd(os.path.join(b, f"{t}.ref.qsd")),
                                                with_data=False))
            tasks[f"{key}/forward"] = np.array(int(m["forward"]))
            if k in sel:
                for t in ("lmpo", "rmpo", "lopr", "ropr", "lsopr", "rsopr", "lwfn", "rwfn", "out_env", "out_lwfn",
                          "out_rwfn"):
                    bonds.update(ref_io.pack_tensor(f"{key}/{t}", ref_io.read_qsd(os.path.join(b, f"{t}.qsd"))))
                for t in ("psi", "sigma", "diag", "lmat", "rmat", "env"):
                    bonds.update(ref_io.pack_tensor(f"{key}/{t}", ref_io.read_qsd(os.path.join(b, f"{t}.ref.qsd"))))
                bonds[f"{key}/meta"] = np.array([m["forward"], m["M"], m["tole"], m["energy"]])
        if name == "qc8":
            mdir = os.path.join(d, "mpo_qsd")
            os.makedirs(mdir, exist_ok=True)
            subprocess.run([os.path.join(REF_BIN, "ref_ops.x"), "dump_mpo", d, str(N), mdir], check=True)
            mpo = {}
            for i in range(N):
                mpo.update(ref_io.pack_tensor(f"site{i}", ref_io.read_qsd(os.path.join(mdir, f"mpo_{i}.qsd"))))
            np.savez_compressed(os.path.join(OUT, "mpo_qc8.npz"), **mpo)
    # C2's operator: the reference's complementary-operator MPO for the synthetic n=20
    # Hamiltonian; the two sites of the middle bond are the bench's H_eff*psi operands
    d = os.path.join(args.work, "c2_mpo")
    os.makedirs(d, exist_ok=True)
    qc_fcidump(os.path.join(d, "FCIDUMP"), 20, 40, 1)
    run([os.path.join(REF_BIN, "mpogen.x"), "-f", "FCIDUMP", "-s", "."], d, log=os.path.join(d, "mpogen.log"))
    mdir = os.path.join(d, "mpo_qsd")
    os.makedirs(mdir, exist_ok=True)
    subprocess.run([os.path.join(REF_BIN, "ref_ops.x"), "dump_mpo", d, "20", mdir], check=True)
    sites = [ref_io.read_qsd(os.path.join(mdir, f"mpo_{i}.qsd")) for i in range(20)]
    runs["c2_mpo"] = {"bond_dims": [len(s["qshape"][3]) for s in sites[:-1]],
                      "nnz": [len(s["blocks"]) for s in sites]}
    mpo = {}
    for i in (9, 10):
        mpo.update(ref_io.pack_tensor(f"site{i}", sites[i]))
    np.savez_compressed(os.path.join(OUT, "mpo_c2_bond.npz"), **mpo)
    with open(os.path.join(OUT, "runs.json"), "w") as f:
        json.dump(runs, f, indent=1)
    np.savez_compressed(os.path.join(OUT, "tasks.npz"), **tasks)
    np.savez_compressed(os.path.join(OUT, "bonds.npz"), **bonds)
    for fn in sorted(os.listdir(OUT)):
        print(fn, os.path.getsize(os.path.join(OUT, fn)))


if __name__ == "__main__":
    main()
