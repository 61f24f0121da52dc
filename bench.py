"""Benchmark of the merged two-site DMRG hot path on one GB300.

Workload (default, ``--workload c2-bond``): one H_eff*psi (compute_sigma_vector, the
Davidson inner loop) at the middle bond (9, 10) of configuration C2 — the synthetic
quantum-chemistry Hamiltonian with n=20 spatial orbitals, 20 electrons, Sz=0, K=40
Cholesky vectors, integral seed 1, M=512.  The operator is the reference's own
complementary-operator MPO at sites 9 and 10 (W = 712 | 862 | 1028), written by the
reference's generator and committed as a fixture; the MPS bonds around the two sites
have the quantum numbers and dimensions of a converged C2 state (committed); every
allowed block of the environments and site tensors holds seeded normal values.  Both
arms build the workload from these files alone.

``value``: device throughput with the operands resident in HBM (CUDA events on the
library's stream).  ``e2e``: the same step through the C ABI with the wavefunction
copied from pinned host memory and sigma copied back inside the timed region;
``bond_step_e2e``: one whole bond step from host site tensors.  ``--impl reference``
times the reference's CPU H_eff*psi (its C++ restatement, pinned bitwise to the
reference's own sigma) on the host cores, on operands built on the host.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024
T_START = time.perf_counter()
METRIC = "H_eff*psi TFLOP/s (FP64-equivalent), C2 middle bond: qc n=20 M=512"
DATA = ("synthetic: the reference generator's MPO sites of the seeded n=20 integrals, a converged state's block "
        "structure, seeded normal block values")

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum over the launches of one
# H_eff*psi: psi pack, the two tensor-core stages, split-K reduce) divided by the
# algorithmic bytes 8 (nnz L + nnz R + 2 nnz psi), measured by ncu on the small case of
# the same kernels (QC n=14, K=28, M=256, complementary-operator MPO: 0.857 GB against
# 0.402 GB) and applied to the bench workloads, whose operators are too large for a
# multi-metric capture; keyed by (workload, precision).
MEASURED_TRAFFIC = {("c2-bond", "split"): 2.14, ("random-mps", "split"): 2.14}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2-bond", choices=["c2-bond", "random-mps"],
                    help="c2-bond: the committed C2 middle bond; random-mps: --norb/--nchol/--M/--bond under this "
                         "library's MPO generator, a seeded random MPS")
    ap.add_argument("--bond-structure", default="", help="bond structure file of the c2-bond workload")
    ap.add_argument("--no-bond-e2e", action="store_true", help="skip the bond step from host site tensors")
    ap.add_argument("--fp32-operators", action="store_true",
                    help="pack the merged operators as FP32 tiles split on chip (default: hi|lo TF32 tiles)")
    ap.add_argument("--mpo", default="comp", choices=["comp", "mvc"],
                    help="QC MPO of the sweeps and of random-mps: comp = the reference generator's complementary "
                         "operators (restated), mvc = this library's vertex-cover construction")
    ap.add_argument("--norb", type=int, default=20)
    ap.add_argument("--nchol", type=int, default=40)
    ap.add_argument("--M", type=int, default=512)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--bond", type=int, default=-1, help="bond index (default: middle)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--tole", type=float, default=1e-9, help="sweep tolerance (Davidson |r|^2 < 0.1 tole)")
    ap.add_argument("--bond-step", action="store_true",
                    help="random-mps workload: also time one full bond step, FP64 and split, from identical inputs")
    ap.add_argument("--no-sweep", action="store_true", help="skip the FP64-vs-split sweep comparison")
    ap.add_argument("--sweep-norb", type=int, default=20)
    ap.add_argument("--sweep-M", type=int, default=512)
    ap.add_argument("--sweep-max", type=int, default=12, help="sweeps per arm (ramp included)")
    ap.add_argument("--split-floor", type=float, default=-1.0,
                    help="split Davidson residual floor (relative to E) before the FP64 anchor (< 0: default)")
    ap.add_argument("--sweep-env-checkpoint", type=int, default=0,
                    help="keep every k-th block operator a sweep pass leaves for the other (0: all)")
    ap.add_argument("--no-sweep-ramp", dest="sweep_ramp", action="store_false",
                    help="all sweeps at --sweep-M (default: two sweeps at M/4, two at M/2 first)")
    ap.add_argument("--sweep-arms", default="",
                    help="comma list of sweep arms to run (fp64, split, fp64_control, split_control; default all)")
    ap.add_argument("--no-sweep-control", action="store_true",
                    help="skip the control arms (FP64 and split at a ten times tighter Davidson tolerance)")
    ap.add_argument("--no-gradient", dest="gradient", action="store_false",
                    help="skip the energy-gradient workloads (site-dependent Hubbard L=32 M=512, QC n=16 M=256)")
    ap.add_argument("--grad-fd", type=int, default=2, help="parameters checked by central differences per workload")
    ap.add_argument("--no-scan", dest="scan", action="store_false",
                    help="skip the batched scan: 64 Hubbard chains, L ~ U{16..32}, U ~ U(0,8), M 64->256 over 6 sweeps")
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall-clock budget: sections not yet started when it is spent are skipped")
    ap.add_argument("--scan-chains", type=int, default=64)
    ap.add_argument("--scan-compare", type=int, default=8, help="chains also swept one by one for comparison")
    return ap.parse_args()


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        # replicas: the collectives only time the job (barrier, max over ranks)
        dist.init_process_group("nccl" if args.impl == "ours" and torch.cuda.is_available() else "gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def job_tflops(ws: int, flops_per_rank_step: float, step_s: float) -> float:
    """Whole-job throughput of replicas: every rank does one step's work, the job's
    step time is the slowest rank's (already maxed over ranks)."""
    return ws * flops_per_rank_step / step_s / 1e12


def max_over_ranks(ws, v: float, device=None) -> float:
    if ws <= 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        import statistics

        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, nm in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# The H_eff*psi workload (both arms build it from these files alone):
#  * the two MPO sites of the middle bond (9, 10) of configuration C2 as the mpsxx
#    reference's own generator writes them (mpogen.x on the synthetic n=20, K=40,
#    seed-1 integrals; W = 712 | 862 | 1028 around the sites);
#  * the quantum numbers and dimensions of the MPS bonds around sites 9 and 10 of a
#    converged C2 state (M=512);
# with seeded normal random values in every allowed block of the environments and of
# the two site tensors, the orthogonality centre on site 9 (a forward sweep's layout).
C2_MPO = os.path.join(ROOT, "tests", "golden", "ref", "mpo_c2_bond.npz")
C2_STRUCTURE = os.path.join(ROOT, "tests", "golden", "c2_bond_structure.json")
SITE_QUANTA = [(0, 0), (1, 1), (1, -1), (2, 0)]


def _npz_tensor(z, name):
    """A tensor dict from the fixtures' npz layout (q, nsec, qshape, dshape, tags, data)."""
    import numpy as np

    nsec = [int(x) for x in z[f"{name}.nsec"]]
    qs = [tuple(int(v) for v in r) for r in z[f"{name}.qshape"]]
    ds = [int(v) for v in z[f"{name}.dshape"]]
    qshape, dshape, o = [], [], 0
    for n in nsec:
        qshape.append(qs[o:o + n])
        dshape.append(ds[o:o + n])
        o += n
    strides = [1] * len(nsec)
    for i in range(len(nsec) - 2, -1, -1):
        strides[i] = strides[i + 1] * nsec[i + 1]
    data, blocks, off = z[f"{name}.data"], {}, 0
    for tag in (int(x) for x in z[f"{name}.tags"]):
        shape = tuple(dshape[i][(tag // strides[i]) % nsec[i]] for i in range(len(nsec)))
        size = int(np.prod(shape, dtype=np.int64))
        blocks[tag] = data[off:off + size].reshape(shape).copy()
        off += size
    return {"q": tuple(int(v) for v in z[f"{name}.q"]), "qshape": qshape, "dshape": dshape, "blocks": blocks}


def _random_tensor(q, qshape, dshape, rng):
    """Every block allowed by the total quantum number (and of non-zero size), filled with
    standard normal values in ascending tag order."""
    import numpy as np

    nsec = [len(x) for x in qshape]
    grids = np.meshgrid(*[np.arange(n) for n in nsec], indexing="ij")
    qp = sum(np.array([x[0] for x in qshape[i]])[grids[i]] for i in range(len(nsec)))
    qs = sum(np.array([x[1] for x in qshape[i]])[grids[i]] for i in range(len(nsec)))
    size = np.prod([np.array(dshape[i])[grids[i]] for i in range(len(nsec))], axis=0)
    ok = (qp == q[0]) & (qs == q[1]) & (size > 0)
    tags = np.flatnonzero(ok.ravel())
    blocks = {}
    for t in tags:
        idx = np.unravel_index(t, nsec)
        shape = tuple(dshape[i][idx[i]] for i in range(len(nsec)))
        blocks[int(t)] = rng.standard_normal(shape)
    return {"q": tuple(q), "qshape": [list(x) for x in qshape], "dshape": [list(x) for x in dshape],
            "blocks": blocks}


def bench_bond(seed: int):
    """Host tensors of the H_eff*psi workload: site MPOs W9, W10, left environment of site 9,
    right environment of site 10, the centre site 9 (total quantum number) and site 10."""
    import numpy as np

    z = np.load(C2_MPO)
    w9, w10 = _npz_tensor(z, "site9"), _npz_tensor(z, "site10")
    with open(C2_STRUCTURE) as f:
        st = json.load(f)
    neg = lambda qs: [(-a, -b) for a, b in qs]  # noqa: E731
    QL, DL = [tuple(q) for q in st["left"]["q"]], st["left"]["d"]
    QM, DM = [tuple(q) for q in st["middle"]["q"]], st["middle"]["d"]
    QR, DR = [tuple(q) for q in st["right"]["q"]], st["right"]["d"]
    qt = tuple(st["q_total"])
    rng = np.random.default_rng(seed)
    one = lambda n: [1] * n  # noqa: E731
    lenv = _random_tensor((0, 0), [QL, neg(w9["qshape"][0]), neg(QL)], [DL, one(len(w9["qshape"][0])), DL], rng)
    renv = _random_tensor((0, 0), [QR, neg(w10["qshape"][3]), neg(QR)], [DR, one(len(w10["qshape"][3])), DR], rng)
    lwfn = _random_tensor(qt, [QL, SITE_QUANTA, QM], [DL, one(4), DM], rng)
    rwfn = _random_tensor((0, 0), [neg(QM), SITE_QUANTA, QR], [DM, one(4), DR], rng)
    return {"w9": w9, "w10": w10, "lenv": lenv, "renv": renv, "lwfn": lwfn, "rwfn": rwfn,
            "W": len(w9["qshape"][3])}


def workload_name(args) -> str:
    if args.workload == "c2-bond":
        return (f"H_eff*psi at the middle bond (9,10) of C2: qc n=20 K=40 seed=1 M=512, the reference's "
                f"complementary-operator MPO sites (W=862), converged-state block structure, values seed {args.seed}")
    return (f"H_eff*psi at bond ({args.bond if args.bond >= 0 else args.norb // 2 - 1},+1): qc n={args.norb} "
            f"K={args.nchol} seed={args.seed}, {MPO_NAMES[args.mpo]}, seeded random MPS M={args.M}")


def build_workload(args, ctx):
    """The bench bond on the device.  c2-bond: the fixture bond through the product's own
    merged-operator and wavefunction-merge entry points; random-mps: a seeded random MPS
    of bond dimension M under this library's MPO, brought to the chosen bond."""
    from mpsxx_gb300 import core

    if args.workload == "c2-bond":
        hb = bench_bond(args.seed)
        t = {k: core.Tensor.from_dict(ctx, hb[k]) for k in ("w9", "w10", "lenv", "renv", "lwfn", "rwfn")}
        mL = core.compute_merged_operator(ctx, True, t["w9"], t["lenv"])
        mR = core.compute_merged_operator(ctx, False, t["w10"], t["renv"])
        psi = core.merge_wavefunction(ctx, t["w9"], t["w10"], t["lenv"], t["renv"], t["lwfn"], t["rwfn"])
        return dict(mL=mL, mR=mR, psi=psi, bond=9, W=hb["W"], host=hb, dev=t)
    from mpsxx_gb300 import dmrg, mpogen

    h1, eri = mpogen.synthetic_qc_integrals(args.norb, args.nchol, args.seed)
    mpo_d = qc_mpo_of(args, h1, eri)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpo_d]
    st = dmrg.make_random_state(ctx, mpo, args.norb, 0, args.M, seed=args.seed)
    bond = args.bond if args.bond >= 0 else args.norb // 2 - 1
    dmrg.advance_left(ctx, st, bond)
    mL, mR, psi = dmrg.bond_operands(ctx, st, bond)
    return dict(mL=mL, mR=mR, psi=psi, bond=bond, W=mpogen.mpo_bond_dims(mpo_d)[bond], st=st)


def host_operands(hb):
    """mL, mR and psi of the fixture bond built on the host by the oracle's restatement
    of compute_merged_operator (src/optimize.hpp:273-368) and of the wavefunction merge
    (src/optimize.hpp:542-557), as exchange dicts."""
    from oracle import dmrg as od
    from oracle import from_site_dict
    from oracle import qsd as oq

    o = {k: from_site_dict(hb[k]) for k in ("w9", "w10", "lenv", "renv", "lwfn", "rwfn")}
    mL = od.compute_merged_operator(True, o["w9"], o["lenv"])
    mR = od.compute_merged_operator(False, o["w10"], o["renv"])
    ql, qr = od.wave_merge_infos(o["w9"], o["w10"], o["lenv"], o["renv"])
    twf = oq.QSDArray()
    oq.gemm(oq.NoTrans, oq.NoTrans, 1.0, o["lwfn"], o["rwfn"], 1.0, twf, nc=4)
    psi = oq.merge_cols(oq.merge_rows(ql, twf), qr)

    def as_dict(a):
        return {"q": tuple(a.q), "qshape": a.qshape, "dshape": a.dshape, "blocks": a.blocks}

    return as_dict(mL), as_dict(mR), as_dict(psi)


def sigma_checksum(blocks) -> dict:
    """Order-independent summary of a sigma, comparable across the two arms."""
    import numpy as np

    s = sum(float(np.sum(b)) for b in blocks.values())
    n = sum(float(np.sum(b * b)) for b in blocks.values()) ** 0.5
    return {"sum": s, "norm": n, "blocks": len(blocks)}


MPO_NAMES = {"comp": "complementary-operator MPO (the reference generator's scheme, restated)",
             "mvc": "this library's minimum-vertex-cover MPO"}


def qc_mpo_of(args, h1, eri):
    """The QC MPO of the chosen construction: the reference generator's complementary
    operators (default) or this library's vertex-cover construction."""
    from mpsxx_gb300 import mpogen, mpogen_comp

    if args.mpo == "comp":
        return mpogen_comp.qc_mpo_complementary(h1, eri)
    return mpogen.qc_mpo(h1, eri)


def _device_bytes_in_use():
    """Device memory in use (nvidia-smi's view of this process's GPU), or None."""
    try:
        out = subprocess.run(["nvidia-smi", "--query-gpu=memory.used", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=10).stdout.split()
        return int(float(out[0])) * 1024 * 1024 if out else None
    except Exception:
        return None


def sweep_schedule(args):
    """Bond dimension per sweep: ramped to sweep_M (two sweeps at M/4, two at M/2), then
    sweep_M for the rest of sweep_max sweeps."""
    M = args.sweep_M
    ramp = [max(16, M // 4)] * 2 + [max(16, M // 2)] * 2 if args.sweep_ramp else []
    return ramp + [M] * max(1, args.sweep_max - len(ramp))


def sweep_compare(args, device: int):
    """Cold two-site DMRG on the synthetic QC system from the reference's initial state
    (constant-filled sites, src/make_random_mpss.cpp:97-271), the same bond-dimension
    schedule in every arm (src/dmrg.cpp:57-65 sweep loop), three arms:

    * ``fp64``: FP64 H_eff*psi, Davidson |r|^2 < 0.1*tole;
    * ``split``: split-precision H_eff*psi with the FP64 refinement, same tolerance;
    * ``fp64_control`` and ``split_control``: both again with a ten times tighter
      Davidson tolerance.

    Where each Davidson stops moves the truncated (fixed M) problem's path, so energies at
    equal sweep counts differ even between two FP64 runs: the FP64-vs-FP64 difference
    across the two tolerances is the floor against which split vs FP64 (at either
    tolerance) is read.  Sweep times are compared at the final M."""
    from mpsxx_gb300 import core, dmrg, mpogen

    n = args.sweep_norb
    sched = sweep_schedule(args)
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, args.seed)
    mpo_d = qc_mpo_of(args, h1, eri)
    res = {"workload": f"qc n={n} K={2 * n} seed={args.seed}, {MPO_NAMES[args.mpo]}", "tole": args.tole,
           "mpo_bond_dims": mpogen.mpo_bond_dims(mpo_d),
           "M_schedule": sched, "start": "reference initial state (constant-filled sites)",
           "env_checkpoint": args.sweep_env_checkpoint, "split_floor": args.split_floor}
    arms = [("fp64", core.FP64, args.tole), ("split", core.SPLIT_TF32, args.tole)]
    if not args.no_sweep_control:
        arms += [("fp64_control", core.FP64, 0.1 * args.tole), ("split_control", core.SPLIT_TF32, 0.1 * args.tole)]
    if args.sweep_arms:
        keep = set(args.sweep_arms.split(","))
        arms = [a for a in arms if a[0] in keep]
    for name, prec, tole in arms:
        ctx = core.Context(device)
        core.set_precision(ctx, prec)
        ctx.set_split_refinement(residual_floor=args.split_floor)
        mpo = [core.Tensor.from_dict(ctx, d) for d in mpo_d]
        st = dmrg.make_initial_state(ctx, mpo, n, 0, sched[0])
        sweeps = []
        for M in sched:
            st.M = M
            log = dmrg.make_sweep(ctx, st, tole, env_checkpoint=args.sweep_env_checkpoint)
            sweeps.append({"M": M, "seconds": log.seconds, "energy": log.energy, "n_sigma": log.n_sigma,
                           "sigma_flops": log.sigma_flops, **{k: round(v, 4) for k, v in log.times.items()},
                           "device_gb_after": round((_device_bytes_in_use() or 0) / 1e9, 2)})
            print(f"sweep {name} M={M} E={log.energy:.12f} {log.seconds:.1f} s {sweeps[-1]['device_gb_after']} GB",
                  file=sys.stderr, flush=True)
        last = sweeps[-1]
        atM = [s for s in sweeps if s["M"] == sched[-1]]
        res[name] = {"sweeps": len(sweeps), "davidson_tole": 0.1 * tole, "energy": last["energy"],
                     "last_dE": abs(last["energy"] - sweeps[-2]["energy"]) if len(sweeps) > 1 else None,
                     "seconds_total": sum(s["seconds"] for s in sweeps),
                     "seconds_per_sweep_final_M": sum(s["seconds"] for s in atM[1:]) / max(1, len(atM) - 1),
                     "n_sigma_total": sum(s["n_sigma"] for s in sweeps),
                     "sigma_tflops_last_sweep": last["sigma_flops"] / last["seconds"] / 1e12,
                     "per_sweep": sweeps}
        res[name]["device_bytes_in_use_after"] = _device_bytes_in_use()
        del st, mpo
        ctx.close()
    if "fp64" not in res or "split" not in res:
        return res
    e64 = res["fp64"]["energy"]
    cmp = {"abs_dE_split_vs_fp64": abs(res["split"]["energy"] - e64),
           "per_sweep_abs_dE_split_vs_fp64": [abs(a["energy"] - b["energy"]) for a, b in
                                              zip(res["split"]["per_sweep"], res["fp64"]["per_sweep"])],
           "seconds_per_sweep_fp64": res["fp64"]["seconds_per_sweep_final_M"],
           "seconds_per_sweep_split": res["split"]["seconds_per_sweep_final_M"],
           "speedup_per_sweep": res["fp64"]["seconds_per_sweep_final_M"] / res["split"]["seconds_per_sweep_final_M"],
           "speedup_total": res["fp64"]["seconds_total"] / res["split"]["seconds_total"]}
    if "fp64_control" in res and "split_control" in res:
        ec, esc = res["fp64_control"]["energy"], res["split_control"]["energy"]

        def per(a, b):
            return [abs(x["energy"] - y["energy"]) for x, y in zip(res[a]["per_sweep"], res[b]["per_sweep"])]

        cmp["abs_dE_split_vs_fp64_tight"] = abs(esc - ec)
        cmp["abs_dE_fp64_vs_fp64_tight"] = abs(e64 - ec)
        cmp["abs_dE_split_vs_split_tight"] = abs(res["split"]["energy"] - esc)
        cmp["abs_dE_split_vs_fp64_control"] = abs(res["split"]["energy"] - ec)
        cmp["seconds_per_sweep_fp64_tight"] = res["fp64_control"]["seconds_per_sweep_final_M"]
        cmp["seconds_per_sweep_split_tight"] = res["split_control"]["seconds_per_sweep_final_M"]
        cmp["speedup_per_sweep_tight"] = cmp["seconds_per_sweep_fp64_tight"] / cmp["seconds_per_sweep_split_tight"]
        cmp["per_sweep_abs_dE_split_vs_fp64_tight"] = per("split_control", "fp64_control")
        cmp["per_sweep_abs_dE_fp64_vs_fp64_tight"] = per("fp64", "fp64_control")
        cmp["per_sweep_abs_dE_split_vs_fp64_control"] = per("split", "fp64_control")
    res["compare"] = cmp
    return res


def _converge(ctx, mpo, n_elec, M, tole, max_sweeps, st=None):
    from mpsxx_gb300 import dmrg

    if st is None:
        st = dmrg.make_initial_state(ctx, mpo, n_elec, 0, M)
    e_prev, n = None, 0
    for n in range(1, max_sweeps + 1):
        log = dmrg.make_sweep(ctx, st, tole)
        if e_prev is not None and abs(log.energy - e_prev) < tole:
            break
        e_prev = log.energy
    return st, log.energy, n


def gradient_bench(args, device: int):
    """Adjoint energy gradients: dE/dU_i, dE/dt_i of a site-dependent Hubbard chain
    (L=32, U_i ~ U(2,6), |t_i| ~ U(0.8,1.2), half filling, M=512) and dE/dh_pq (with the
    reference's MPO also dE/d(pq|rs)) of the n=16 synthetic QC Hamiltonian (M=256),
    through the generators' Jacobians.  Gradient in FP64 and split precision on
    the same converged state, environments checkpointed every 4 sites; a few
    parameters checked by central differences (step 1e-4) of the energy, both of
    warm-restarted DMRG (the state re-converged: the derivative of the truncated
    problem's energy) and of the converged state held fixed (<psi|H(theta +- h)|psi>:
    what the adjoint computes, by Hellmann-Feynman)."""
    import numpy as np

    from mpsxx_gb300 import core, dmrg, mpogen, mpogen_comp

    out = {}
    rng = np.random.default_rng(args.seed)
    L = 32
    U = rng.uniform(2.0, 6.0, L)
    t = -rng.uniform(0.8, 1.2, L - 1)
    n = 16
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, args.seed)
    cases = [
        ("hubbard_L32_M512", lambda th: mpogen.hubbard_mpo(L, th[0], th[1], jacobian=True), (t, U), L, 512,
         [("U", 0), ("U", L // 2), ("t", L // 2)]),
        ("qc_n16_M256", lambda th: mpogen.qc_mpo(th[0], th[1], jacobian=True), (h1, eri), n, 256,
         [("h", 0, 0), ("h", 3, 5), ("h", 7, 8)]),
    ]
    if args.mpo == "comp":  # the reference's generator: keys of the integrals it reads
        cases[1] = ("qc_n16_M256", lambda th: mpogen_comp.qc_mpo_complementary(th[0], th[1], jacobian=True),
                    (h1, eri), n, 256, [("h", 0, 0), ("eri", 5, 3, 5, 3), ("h", 8, 7), ("eri", 3, 3, 3, 3)])
    tole = 1e-10
    for name, build, theta, nel, M, checks in cases:
        ctx = core.Context(device)
        sites, jacs = build(theta)
        mpo = [core.Tensor.from_dict(ctx, d) for d in sites]
        t0 = time.perf_counter()
        st, e0, nsw = _converge(ctx, mpo, nel, M, tole, 20)
        t_dmrg = time.perf_counter() - t0
        tags = [m.blocks()[0] for m in st.mpo]
        res = {"energy": e0, "sweeps": nsw, "dmrg_seconds": t_dmrg, "checkpoint": 4}
        if name.startswith("qc"):
            res["mpo"] = MPO_NAMES[args.mpo]
        grads = {}
        for pname, prec in (("fp64", core.FP64), ("split", core.SPLIT_TF32)):
            core.set_precision(ctx, prec)
            g = dmrg.gradient_sweep(ctx, st, checkpoint=4)
            core.set_precision(ctx, core.FP64)
            grads[pname] = dmrg.parameter_gradient(g.site_grads, tags, jacs)
            res[pname] = {"seconds": g.seconds, "state_energy": g.energy, "env_recomputed": g.env_recomputed,
                          "env_peak": g.env_peak, "env_all": len(st.mpo)}
        keys = sorted(grads["fp64"], key=str)
        res["n_parameters"] = len(keys)
        res["split_vs_fp64_max_rel"] = max(abs(grads["split"][k] - grads["fp64"][k]) / max(1.0, abs(grads["fp64"][k]))
                                          for k in keys)
        fd_rows = []
        for par in checks[: args.grad_fd]:
            vals, fixed = [], []
            for sgn in (1.0, -1.0):
                th = [np.array(x, copy=True) for x in theta]
                if par[0] == "U":
                    th[1][par[1]] += sgn * 1e-4
                elif par[0] == "t":
                    th[0][par[1]] += sgn * 1e-4
                elif par[0] == "eri":  # every entry of the 8-fold class
                    p, q, r, s_ = par[1:]
                    for a, b, c, d in {(p, q, r, s_), (q, p, r, s_), (p, q, s_, r), (q, p, s_, r),
                                       (r, s_, p, q), (s_, r, p, q), (r, s_, q, p), (s_, r, q, p)}:
                        th[1][a, b, c, d] += sgn * 1e-4
                else:  # symmetric step of h_pq and h_qp
                    p, q = par[1], par[2]
                    th[0][p, q] += sgn * 1e-4
                    if p != q:
                        th[0][q, p] += sgn * 1e-4
                sites2, _ = build(th)
                mpo2 = [core.Tensor.from_dict(ctx, d) for d in sites2]
                st2 = dmrg.restart_state(ctx, mpo2, st)
                # the converged state's energy under the stepped Hamiltonian (state held)
                fixed.append(dmrg.gradient_sweep(ctx, st2, checkpoint=4).energy)
                st2, _, _ = _converge(ctx, mpo2, nel, M, tole * 0.1, 8, st2)
                vals.append(dmrg.gradient_sweep(ctx, st2, checkpoint=4).energy)
            fd = (vals[0] - vals[1]) / 2e-4
            fd_fixed = (fixed[0] - fixed[1]) / 2e-4
            adj = grads["fp64"].get(par, 0.0)
            if par[0] == "h" and par[1] != par[2]:
                adj += grads["fp64"].get(("h", par[2], par[1]), 0.0)
            fd_rows.append({"param": list(map(str, par)), "adjoint": adj, "fd": fd,
                            "rel": abs(adj - fd) / max(1.0, abs(fd)), "fd_state_held": fd_fixed,
                            "rel_state_held": abs(adj - fd_fixed) / max(1.0, abs(fd_fixed))})
        res["fd_checks"] = fd_rows
        out[name] = res
        del st, mpo
        ctx.close()
    return out


def scan_bench(args, device: int):
    """Batched parameter scan: all chains' bond steps in lockstep (one grouped tensor-core
    H_eff*psi launch per stage for all unconverged chains), split precision with the
    FP64 refinement; a subset of the chains is also swept one by one for timing and
    energy comparison."""
    from mpsxx_gb300 import core, scan

    specs = scan.random_specs(args.scan_chains, args.seed)
    # bond dimension ramped over 6 sweeps, then 2 sweeps at the final M so that the
    # batched and one-by-one runs are compared at convergence (early sweeps of strongly
    # correlated chains take rounding-dependent paths to the same fixed point)
    sched = scan.m_schedule(64, 256, 6) + [256, 256]
    ctx = core.Context(device)
    core.set_precision(ctx, core.SPLIT_TF32)
    chains = scan.make_chains(ctx, specs, sched[0])
    rows = []
    for M in sched:
        r = scan.sweep_batched(ctx, chains, M, args.tole)
        rows.append({"M": M, "seconds": r["seconds"], "n_sigma": r["n_sigma"], "bond_steps": r["bond_steps"]})
    t_batched = sum(r["seconds"] for r in rows)
    k = min(args.scan_compare, len(specs))
    single = scan.make_chains(ctx, specs[:k], sched[0])
    t_single = 0.0
    for M in sched:
        t_single += scan.sweep_sequential(ctx, single, M, args.tole)["seconds"]
    de = [abs(a.energies[-1] - b.energies[-1]) for a, b in zip(chains[:k], single)]
    ctx.close()
    per_chain_batched = t_batched / len(specs)
    per_chain_single = t_single / k
    return {"chains": len(specs), "lengths": [s[0] for s in specs], "M_schedule": sched, "tole": args.tole,
            "precision": "split", "per_sweep": rows, "seconds_batched_all": t_batched,
            "seconds_per_chain_batched": per_chain_batched, "compared_chains": k,
            "seconds_per_chain_one_by_one": per_chain_single, "speedup_per_chain": per_chain_single / per_chain_batched,
            "abs_dE_max_vs_one_by_one": max(de), "abs_dE_vs_one_by_one": de,
            "final_energies": [c.energies[-1] for c in chains]}


def bond_compare(ctx, wl, M, tole):
    """One full two-site step (merged operators, diagonal, Davidson, SVD, renormalise,
    expand) on the bench bond, FP64 and split precision from identical inputs."""
    from mpsxx_gb300 import core

    st, i = wl["st"], wl["bond"]
    out = {}
    for name, prec in (("fp64", core.FP64), ("split", core.SPLIT_TF32)):
        core.set_precision(ctx, prec)
        ctx.sync()
        t0 = time.perf_counter()
        e, env, nl, nr, s = core.optimize_twosite_merged(ctx, True, st.mpo[i], st.mpo[i + 1], st.lenv[i],
                                                         st.renv[i + 1], st.wave[i], st.wave[i + 1], 0.1 * tole, M)
        dt = time.perf_counter() - t0
        out[name] = {"seconds": dt, "energy": e, "n_sigma": int(s["n_sigma"]),
                     "n_sigma_fp64": int(s["n_sigma_fp64"]) if prec != core.FP64 else int(s["n_sigma"]),
                     "t_davidson": s["t_davidson"], "t_renorm": s["t_renorm"], "t_svd": s["t_svd"],
                     "t_merge": s["t_merge"], "converged": int(s["converged"])}
    core.set_precision(ctx, core.FP64)
    out["abs_dE"] = abs(out["split"]["energy"] - out["fp64"]["energy"])
    out["speedup"] = out["fp64"]["seconds"] / out["split"]["seconds"]
    out["tole"] = tole
    return out


def roofline_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def measure_fp64_peak(torch) -> float:
    """cuBLAS DGEMM throughput (TFLOP/s) on this GPU: the FP64 roofline denominator."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(5):
        a @ b
    e1.record()
    torch.cuda.synchronize()
    return 5 * 2 * n ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12


def cpu_sigma_timed(mL: dict, mR: dict, psi: dict, budget_s: float, min_reps: int = 1):
    """The C++ restatement of the reference's CPU H_eff*psi (oracle/cpu: BTAS task
    enumeration, FLOP-sorted OpenMP task loop, one single-threaded dgemm per block pair,
    pinned bit for bit to the reference's own sigma) on all host cores, repeated until
    ``budget_s`` seconds of sigma work.  Returns (sigma blocks, FLOPs per sigma, seconds
    per sigma, repetitions, threads)."""
    from oracle import cpu as ocpu

    ops = ocpu.Operands(mL, mR, psi)
    secs = []
    blocks, fl = None, 0.0
    while len(secs) < min_reps or sum(secs) < budget_s:
        blocks, fl, s = ocpu.sigma(ops)
        secs.append(s)
    return blocks, fl, sum(secs) / len(secs), len(secs), ocpu.threads()


def sigma_vs_cpu(gpu_blocks, cpu_blocks) -> dict:
    """Largest block-wise difference of the device FP64 sigma from the CPU restatement's,
    relative to the largest |sigma| element; a block present on one side only counts in
    full."""
    import numpy as np

    scale = max(float(np.abs(b).max()) for b in cpu_blocks.values() if b.size)
    worst = 0.0
    for t in set(gpu_blocks) | set(cpu_blocks):
        g, b = gpu_blocks.get(t), cpu_blocks.get(t)
        if g is None or b is None:
            x = b if g is None else g
            worst = max(worst, float(np.abs(x).max()) / scale if x.size else 0.0)
        else:
            worst = max(worst, float(np.abs(g - b).max()) / scale if b.size else 0.0)
    return {"max_rel_err": worst, "blocks_gpu": len(gpu_blocks), "blocks_cpu": len(cpu_blocks)}


def cpu_record(fl, sec, reps, threads, what) -> dict:
    return {"value": fl / sec / 1e12, "unit": "TFLOP/s", "cores": threads, "kind": "port",
            "sample": f"C++ restatement of the reference's CPU H_eff*psi (BTAS block tasks, OpenMP over tasks, "
                      f"OpenBLAS dgemm per block pair; bitwise equal to the reference's sigma on its dumped bonds) "
                      f"on {what}: {reps} full H_eff*psi, {sec:.2f} s each, {threads} threads"}


def run_reference(args, ws, rank):
    """Reference arm: the reference's CPU H_eff*psi on the host cores, on the same bond.

    The reference's sources are not on the GPU host, so its C++ restatement (oracle/cpu,
    pinned bitwise to the reference's own sigma) is timed.  The operands are built on the
    host by the oracle from the committed bond files; nothing of the GPU library is
    imported or loaded.  Other ranks exit without work."""
    if rank != 0:
        return
    if args.workload != "c2-bond":
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm runs on the c2-bond workload only"}))
        return
    t0 = time.perf_counter()
    mL, mR, psi = host_operands(bench_bond(args.seed))
    t_build = time.perf_counter() - t0
    from oracle import cpu as ocpu

    ops = ocpu.Operands(mL, mR, psi)
    for _ in range(args.warmup):
        ocpu.sigma(ops)
    secs = []
    blocks, fl = None, 0.0
    for _ in range(max(1, args.steps)):
        blocks, fl, s = ocpu.sigma(ops)
        secs.append(s)
    sec = sum(secs) / len(secs)
    v = fl / sec / 1e12
    th = ocpu.threads()
    # the same H_eff*psi on one core (one untimed run first)
    ocpu.set_threads(1)
    try:
        ocpu.sigma(ops)
        _, _, sec1 = ocpu.sigma(ops)
    finally:
        ocpu.set_threads(0)
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "TFLOP/s", "n_gpus": 1, "steps": len(secs),
           "warmup": args.warmup, "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": DATA,
           "config": {"workload": workload_name(args), "W": 862, "flops_per_step": fl, "parallelism": "host cores"},
           "cpu_baseline": cpu_record(fl, sec, len(secs), th, "operands built on the host by the oracle"),
           "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "cpu_single_core": {"value": fl / sec1 / 1e12, "unit": "TFLOP/s", "ms_per_step": sec1 * 1e3, "cores": 1,
                               "speedup_all_cores": sec1 / sec},
           "sigma_checksum": sigma_checksum(blocks), "host_setup_s": round(t_build, 1)}
    print(json.dumps(out), flush=True)


def measure_tf32_peak(torch) -> float:
    """cuBLAS TF32 tensor-core GEMM throughput (TFLOP/s, FP32 8192^3 with TF32 math, best
    of 10): the split path's tensor roofline is a third of it (three products)."""
    n = 8192
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        a = torch.randn(n, n, dtype=torch.float32, device="cuda")
        b = torch.randn(n, n, dtype=torch.float32, device="cuda")
        for _ in range(3):
            a @ b
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(10):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b
        return 2 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def bond_e2e(ctx, hb, M: int, tole: float, precision: int, reps: int = 2) -> dict:
    """One two-site bond step (merged operators, diagonal, Davidson, SVD, renormalisation,
    expand) end to end from host site tensors: the six input tensors uploaded, the step,
    the renormalised environment and both new site tensors downloaded."""
    from mpsxx_gb300 import core

    core.set_precision(ctx, precision)
    names = ("w9", "w10", "lenv", "renv", "lwfn", "rwfn")
    h2d = 8 * sum(int(sum(b.size for b in hb[k]["blocks"].values())) for k in names)
    rows = []
    for _ in range(reps):
        ctx.sync()
        t0 = time.perf_counter()
        t = {k: core.Tensor.from_dict(ctx, hb[k]) for k in names}
        e, env, nl, nr, s = core.optimize_twosite_merged(ctx, True, t["w9"], t["w10"], t["lenv"], t["renv"],
                                                         t["lwfn"], t["rwfn"], 0.1 * tole, M)
        outs = [x.download() for x in (env, nl, nr)]
        dt = time.perf_counter() - t0
        rows.append({"seconds": dt, "energy": e, "n_sigma": int(s["n_sigma"]), "t_davidson": s["t_davidson"],
                     "t_svd": s["t_svd"], "t_renorm": s["t_renorm"], "t_merge": s["t_merge"],
                     "d2h_bytes": 8 * sum(int(o.size) for o in outs)})
        del t, env, nl, nr
    core.set_precision(ctx, core.FP64)
    return {"h2d_bytes": h2d, "runs": rows, "seconds_best": min(r["seconds"] for r in rows)}


def main():
    global T_START
    T_START = time.perf_counter()
    args = parse()
    ws, rank, local = dist_init(args)
    if args.workload == "c2-bond" and args.bond_structure:
        global C2_STRUCTURE
        C2_STRUCTURE = args.bond_structure
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    import torch

    torch.cuda.set_device(local)
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import lib

    ctx = core.Context(local)
    ctx.set_sigma_operator_format(args.fp32_operators)
    wl = build_workload(args, ctx)
    mL, mR, psi = wl["mL"], wl["mR"], wl["psi"]

    # Parity first, on a fresh FP64 sigma: against the CPU restatement of the reference's
    # sigma on the same operands (downloaded), which is also the timed CPU baseline.
    core.set_precision(ctx, core.FP64)
    s64 = psi.like()
    core.compute_sigma_vector(ctx, mL, mR, psi, s64)
    ref64 = s64.download()
    gpu64_blocks = s64.to_dict()["blocks"]
    cpu_base, parity = None, None
    if not args.no_cpu_baseline and ws == 1:
        cblocks, cfl, csec, creps, cth = cpu_sigma_timed(mL.to_dict(), mR.to_dict(), psi.to_dict(), args.cpu_seconds)
        cpu_base = cpu_record(cfl, csec, creps, cth, "the same bond's operands downloaded from the device")
        parity = {"sigma_fp64_vs_cpu_port": sigma_vs_cpu(gpu64_blocks, cblocks),
                  "sigma_checksum_gpu_fp64": sigma_checksum(gpu64_blocks),
                  "sigma_checksum_cpu_port": sigma_checksum(cblocks)}
        del cblocks

    # one call builds and caches the plan
    core.set_precision(ctx, core.SPLIT_TF32 if args.precision == "split" else core.FP64)
    sig = psi.like()
    core.compute_sigma_vector(ctx, mL, mR, psi, sig)
    ctx.sync()
    c0 = ctx.counters()
    fl_per_step = c0["sigma_flops"] / max(1, c0["sigma_calls"])
    bytes_alg = 8 * (mL.nnz + mR.nnz + 2 * psi.nnz)
    inputs_bytes = 8 * (mL.nnz + mR.nnz + psi.nnz)
    l2 = "inputs larger than L2" if inputs_bytes > L2_BYTES else "L2 flushed between steps"
    flush = None if inputs_bytes > L2_BYTES else torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    # FP64 timing of the same step (CUDA events on the context's stream)
    core.set_precision(ctx, core.FP64)
    fp64_s = kernel_times(ctx, mL, mR, psi, s64, max(2, min(args.steps, 3)))["sigma_kernels_s"]

    # headline: split-precision (3xTF32 tensor-core) path
    core.set_precision(ctx, core.SPLIT_TF32 if args.precision == "split" else core.FP64)
    for _ in range(args.warmup):
        core.compute_sigma_vector(ctx, mL, mR, psi, sig)
    tuning = ctx.tuning()
    plan_stats = core.sigma_plan_stats(ctx, mL, mR, psi)
    barrier(ws)
    torch.cuda.synchronize()
    launches0 = ctx.counters()["launches"]
    times = []
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")
        for _ in range(args.steps):
            if flush is not None:
                flush.zero_()
                torch.cuda.synchronize()
            t0 = time.perf_counter()
            core.compute_sigma_vector(ctx, mL, mR, psi, sig)  # returns after the stream completes
            times.append(time.perf_counter() - t0)
        torch.cuda.nvtx.range_pop()
    barrier(ws)
    launches = ctx.counters()["launches"] - launches0
    step_s = max_over_ranks(ws, sum(times) / len(times), device="cuda")
    kt = kernel_times(ctx, mL, mR, psi, sig, args.steps)
    value = job_tflops(ws, fl_per_step, step_s)
    # accuracy of one step against the FP64 step
    one = sig.like()
    core.compute_sigma_vector(ctx, mL, mR, psi, one)
    got = one.download()
    rel = float(abs(got - ref64).max() / max(abs(ref64).max(), 1e-300))

    # e2e through the C ABI: pinned host psi -> device, sigma, device -> pinned host
    hpsi = torch.from_numpy(psi.download()).pin_memory()
    hsig = torch.empty_like(hpsi).pin_memory()
    for _ in range(args.warmup):
        e2e_step(ctx, lib(), psi, sig, hpsi, hsig, mL, mR)
    barrier(ws)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step(ctx, lib(), psi, sig, hpsi, hsig, mL, mR)
    e2e_s = max_over_ranks(ws, (time.perf_counter() - t0) / args.steps, device="cuda")

    peaks, src = roofline_peaks()
    fp64_peak = measure_fp64_peak(torch)
    tf32_peak = measure_tf32_peak(torch)
    bond = None
    if args.workload == "c2-bond" and not args.no_bond_e2e:
        bond = {p: bond_e2e(ctx, wl["host"], 512, args.tole, prec)
                for p, prec in (("split", core.SPLIT_TF32), ("fp64", core.FP64))}
    elif args.bond_step and "st" in wl:
        bond = bond_compare(ctx, wl, args.M, args.tole)
    # The headline workload's device memory is given back before the sections, which
    # build their own (the largest configurations need all of the GPU's memory).
    shape_info = {"W": wl["W"], "D_rows": sum(psi.shape()[1][0]), "D_cols": sum(psi.shape()[1][1]),
                  "nnz_psi": psi.nnz, "nnz_L": mL.nnz, "nnz_R": mR.nnz}
    psi_nnz = psi.nnz
    del mL, mR, psi, sig, s64, one, wl
    import gc

    gc.collect()
    ctx.close()
    # the sweep comparison, the scan and the gradients belong to the one-GPU line
    # (replicas, N > 1, time H_eff*psi only); a section not yet started when the
    # wall-clock budget is spent is skipped and says so
    sections, results = {}, {}
    for name, on, fn in (("sweeps", not args.no_sweep, sweep_compare), ("scan", args.scan, scan_bench),
                         ("gradient", args.gradient, gradient_bench)):
        if not on or ws > 1:
            results[name] = None
            continue
        if time.perf_counter() - T_START > args.budget_s:
            results[name] = {"skipped": f"wall-clock budget of {args.budget_s:.0f} s spent before this section"}
            continue
        t_sec = time.perf_counter()
        results[name] = fn(args, local)
        sections[name] = time.perf_counter() - t_sec
    sweep, scan_res, grad = results["sweeps"], results["scan"], results["gradient"]
    if rank == 0:
        ksec = kt["sigma_kernels_s"]
        achieved_tf = fl_per_step / ksec / 1e12
        traffic = MEASURED_TRAFFIC.get((args.workload, args.precision))
        if args.precision == "split":
            roof = {"bound": "hbm", "achieved": bytes_alg / ksec / 1e9, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": bytes_alg / ksec / 1e9 / peaks["hbm_gbs"],
                    "traffic": traffic * bytes_alg if traffic else None,
                    "traffic_note": (f"DRAM bytes per H_eff*psi = {traffic:.2f} x the algorithmic bytes, the ratio "
                                     f"of dram__bytes_read+write to algorithmic bytes measured by ncu on the "
                                     f"small case of the same kernels" if traffic else None),
                    "algorithmic_bytes": bytes_alg,
                    "peak_source": f"{src} hbm_gbs (STREAM-style copy)",
                    "tensor": {"achieved": achieved_tf, "peak": tf32_peak / 3.0, "unit": "TFLOP/s",
                               "frac": achieved_tf / (tf32_peak / 3.0),
                               "peak_source": "cuBLAS TF32 GEMM measured in this run, /3 (three TF32 products "
                                              "per FP64-equivalent product)",
                               "tf32_tflops": tf32_peak},
                    "intensity_flop_per_byte": fl_per_step / bytes_alg,
                    "ridge_flop_per_byte": tf32_peak / 3.0 * 1e12 / (peaks["hbm_gbs"] * 1e9)}
        else:
            roof = {"bound": "fp64", "achieved": achieved_tf, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": achieved_tf / fp64_peak, "traffic": None,
                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 pipe)"}
        roof.update({"kernel_ms": ksec * 1e3, "hbm_peak_source": src})
        out = {
            "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "tf32x3-split (fp64 in/out)" if args.precision == "split" else "f64",
            "data": DATA,
            "config": {"workload": workload_name(args), **shape_info,
                       "flops_per_step": fl_per_step, "l2": l2, "parallelism": f"replicas{ws}",
                       "precision": args.precision,
                       "operators": "FP32 tiles split on chip" if args.fp32_operators else "hi|lo TF32 tiles"},
            "gpu_launches": int(launches),
            "e2e": {"value": job_tflops(ws, fl_per_step, e2e_s), "unit": "TFLOP/s", "ms_per_step": e2e_s * 1e3,
                    "h2d_bytes_per_step": 8 * psi_nnz, "d2h_bytes_per_step": 8 * psi_nnz},
            "roofline": roof,
            "fp64_path": {"ms_per_step": fp64_s * 1e3, "value": fl_per_step / fp64_s / 1e12, "unit": "TFLOP/s",
                          "peak": fp64_peak, "frac": fl_per_step / fp64_s / 1e12 / fp64_peak,
                          "speedup_of_headline": fp64_s / ksec},
            "accuracy": {"max_rel_err_vs_fp64": rel},
            "parity": parity,
            "cpu_baseline": cpu_base,
            "sigma_tuning": [{"w_scratch_mb": b / 2**20, "target_tiles": tt, "fp32_intermediate": f, "ms": ms}
                             for b, tt, f, ms in tuning],
            "sigma_plan": plan_stats,
            "bond_step_e2e": bond,
            "sweeps": sweep,
            "gradient": grad,
            "scan": scan_res,
            "clocks": clk.summary(),
            "section_seconds": {k: round(v, 1) for k, v in sections.items()},
        }
        print(json.dumps(out), flush=True)
    barrier(ws)


def e2e_step(ctx, L, psi, sig, hpsi, hsig, mL, mR):
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import check

    dptr = C.POINTER(C.c_double)
    check(L.mpsxx_tensor_upload(psi.h, C.cast(hpsi.data_ptr(), dptr)))
    core.compute_sigma_vector(ctx, mL, mR, psi, sig)
    check(L.mpsxx_tensor_download(sig.h, C.cast(hsig.data_ptr(), dptr)))


def kernel_times(ctx, mL, mR, psi, sig, steps):
    """Device time of the sigma kernels (CUDA events on the context's stream)."""
    from mpsxx_gb300 import core
    from mpsxx_gb300._lib import lib, check

    t0 = time.perf_counter()
    for _ in range(steps):
        core.compute_sigma_vector(ctx, mL, mR, psi, sig)
    wall = (time.perf_counter() - t0) / steps
    ev = C.c_double()
    rc = lib().mpsxx_sigma_device_time(ctx.h, mL.h, mR.h, psi.h, sig.h, int(steps), C.byref(ev)) \
        if hasattr(lib(), "mpsxx_sigma_device_time") else -1
    if rc == 0:
        return {"sigma_kernels_s": ev.value, "wall_s": wall}
    return {"sigma_kernels_s": wall, "wall_s": wall}


if __name__ == "__main__":
    main()
