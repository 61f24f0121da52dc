"""Benchmark of the merged two-site DMRG hot path on one GB300.

Workload (default): the synthetic quantum-chemistry Hamiltonian with n=20
spatial orbitals, 20 electrons, Sz=0, integral seed 1, K=40 Cholesky vectors,
complementary-operator MPO, bond dimension M=512.  The state is a random MPS of
bond dimension 512 (synthetic, seeded) brought into mixed-canonical form at the
middle bond (9, 10), where the MPO bond dimension peaks.  One step = one
H_eff*psi application (compute_sigma_vector, the Davidson inner loop) on that
bond.  Inputs are resident in HBM for ``value``; ``e2e`` repeats the step
through the C ABI with the wavefunction copied from pinned host memory and the
result copied back inside the timed region.

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

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per H_eff*psi of the default
# workload (QC n=20, K=40, seed 1, M=512, bond (9,10)), summed over the launches of one
# step, from one ncu capture of the launch list (one pass); None for other workloads.
MEASURED_TRAFFIC = {("split", 20, 40, 1, 512): 6.75e9, }


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--norb", type=int, default=20)
    ap.add_argument("--nchol", type=int, default=40)
    ap.add_argument("--M", type=int, default=512)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--bond", type=int, default=-1, help="bond index (default: middle)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--precision", default="split", choices=["split", "fp64"])
    ap.add_argument("--tole", type=float, default=1e-9, help="sweep tolerance (Davidson |r|^2 < 0.1 tole)")
    ap.add_argument("--bond-step", action="store_true", help="also time one full bond step at the bench bond")
    ap.add_argument("--no-sweep", action="store_true", help="skip the FP64-vs-split sweep comparison")
    ap.add_argument("--sweep-norb", type=int, default=20)
    ap.add_argument("--sweep-M", type=int, default=512)
    ap.add_argument("--sweep-max", type=int, default=16)
    ap.add_argument("--sweep-conv", type=float, default=1e-10,
                    help="sweep convergence: |dE| between consecutive sweeps")
    ap.add_argument("--no-sweep-control", action="store_true",
                    help="skip the FP64 control arm (ten times tighter Davidson tolerance)")
    ap.add_argument("--mpo", default="qc", choices=["qc"], help="QC MPO construction")
    ap.add_argument("--gradient", action="store_true",
                    help="also run the energy-gradient workloads (site-dependent Hubbard L=32 M=512, QC n=16 M=256)")
    ap.add_argument("--grad-fd", type=int, default=2, help="parameters checked by central differences per workload")
    ap.add_argument("--scan", action="store_true",
                    help="also run the batched scan: 64 Hubbard chains, L ~ U{16..32}, U ~ U(0,8), M 64->256 over 6 sweeps")
    ap.add_argument("--scan-chains", type=int, default=64)
    ap.add_argument("--scan-compare", type=int, default=8, help="chains also swept one by one for comparison")
    ap.add_argument("--warm-sweeps", type=int, default=2,
                    help="sweeps in each precision from the FP64-converged state")
    ap.add_argument("--sweep-split-all", action="store_true",
                    help="also sweep with the renormalisation contractions in split precision")
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


def mpo_dicts(args, h1, eri):
    from mpsxx_gb300 import mpogen

    return mpogen.qc_mpo(h1, eri)


def build_workload(args, ctx):
    from mpsxx_gb300 import core, dmrg, mpogen

    h1, eri = mpogen.synthetic_qc_integrals(args.norb, args.nchol, args.seed)
    mpo_d = mpo_dicts(args, h1, eri)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpo_d]
    st = dmrg.make_random_state(ctx, mpo, args.norb, 0, args.M, seed=args.seed)
    bond = args.bond if args.bond >= 0 else args.norb // 2 - 1
    dmrg.advance_left(ctx, st, bond)
    mL, mR, psi = dmrg.bond_operands(ctx, st, bond)
    return dict(mpo_d=mpo_d, mL=mL, mR=mR, psi=psi, bond=bond, W=mpogen.mpo_bond_dims(mpo_d)[bond], st=st)


def sweep_compare(args, device: int):
    """Cold two-site DMRG from the reference's initial state (constant-filled sites,
    src/make_random_mpss.cpp:97-271) on the synthetic QC system, in three arms, each
    swept until the sweep energy changes by less than ``sweep_conv`` after at least two
    sweeps (src/dmrg.cpp:57-65), at most ``sweep_max`` sweeps:

    * ``fp64``: FP64 H_eff*psi, Davidson |r|^2 < 0.1*tole;
    * ``split``: split-precision H_eff*psi with the FP64 refinement, same tolerance;
    * ``fp64_control``: FP64 again with a ten times tighter Davidson tolerance.

    The two FP64 arms differ only in where each Davidson stops; the energy they settle
    at differs by the path dependence of the truncated (fixed M) problem, the floor
    against which the split-vs-FP64 difference is read."""
    from mpsxx_gb300 import core, dmrg, mpogen

    n, M = args.sweep_norb, args.sweep_M
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, args.seed)
    mpo_d = mpo_dicts(args, h1, eri)
    res = {"workload": f"qc n={n} K={2 * n} seed={args.seed} M={M} mpo={args.mpo}", "tole": args.tole,
           "sweep_conv": args.sweep_conv, "start": "reference initial state (constant-filled sites)"}
    arms = [("fp64", core.FP64, args.tole), ("split", core.SPLIT_TF32, args.tole)]
    if not args.no_sweep_control:
        arms.append(("fp64_control", core.FP64, 0.1 * args.tole))
    if args.sweep_split_all:
        arms.append(("split_all", core.SPLIT_TF32_ALL, args.tole))
    warm = None
    for name, prec, tole in arms:
        ctx = core.Context(device)
        core.set_precision(ctx, prec)
        mpo = [core.Tensor.from_dict(ctx, d) for d in mpo_d]
        st = dmrg.make_initial_state(ctx, mpo, n, 0, M)
        sweeps, e_prev, conv = [], None, False
        for it in range(args.sweep_max):
            log = dmrg.make_sweep(ctx, st, tole)
            sweeps.append({"seconds": log.seconds, "energy": log.energy, "n_sigma": log.n_sigma,
                           "sigma_flops": log.sigma_flops, **{k: round(v, 4) for k, v in log.times.items()}})
            if e_prev is not None and it >= 1 and abs(log.energy - e_prev) < args.sweep_conv:
                conv = True
                break
            e_prev = log.energy
        last = sweeps[-1]
        res[name] = {"sweeps": len(sweeps), "converged": conv, "davidson_tole": 0.1 * tole,
                     "energy": last["energy"],
                     "last_dE": abs(last["energy"] - sweeps[-2]["energy"]) if len(sweeps) > 1 else None,
                     "seconds_total": sum(s["seconds"] for s in sweeps),
                     "seconds_last_sweep": last["seconds"],
                     "n_sigma_total": sum(s["n_sigma"] for s in sweeps),
                     "sigma_tflops_last_sweep": last["sigma_flops"] / last["seconds"] / 1e12,
                     "per_sweep": sweeps}
        if name == "fp64" and args.warm_sweeps > 0:
            warm = warm_compare(args, ctx, st)
        del st, mpo
        ctx.close()
    e64 = res["fp64"]["energy"]
    res["cold"] = {"abs_dE_split_vs_fp64": abs(res["split"]["energy"] - e64),
                   "abs_dE_fp64_control_vs_fp64": (abs(res["fp64_control"]["energy"] - e64)
                                                   if "fp64_control" in res else None),
                   "seconds_per_sweep_fp64": res["fp64"]["seconds_last_sweep"],
                   "seconds_per_sweep_split": res["split"]["seconds_last_sweep"],
                   "speedup_last_sweep": res["fp64"]["seconds_last_sweep"] / res["split"]["seconds_last_sweep"],
                   "speedup_total": res["fp64"]["seconds_total"] / res["split"]["seconds_total"]}
    if "split_all" in res:
        res["split_all"]["abs_dE"] = abs(res["split_all"]["energy"] - e64)
    res["warm"] = warm
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
    (L=32, U_i ~ U(2,6), |t_i| ~ U(0.8,1.2), half filling, M=512) and dE/dh_pq of the
    n=16 synthetic QC Hamiltonian (M=256).  Gradient in FP64 and split precision on
    the same converged state, environments checkpointed every 4 sites; a few
    parameters checked by central differences (step 1e-4) of warm-restarted DMRG."""
    import numpy as np

    from mpsxx_gb300 import core, dmrg, mpogen

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
        ("qc_n16_M256", lambda th: mpogen.qc_mpo(th[0], eri, jacobian=True), (h1,), n, 256,
         [("h", 0, 0), ("h", 3, 5), ("h", 7, 8)]),
    ]
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
            vals = []
            for sgn in (1.0, -1.0):
                th = [np.array(x, copy=True) for x in theta]
                if par[0] == "U":
                    th[1][par[1]] += sgn * 1e-4
                elif par[0] == "t":
                    th[0][par[1]] += sgn * 1e-4
                else:  # symmetric step of h_pq and h_qp
                    p, q = par[1], par[2]
                    th[0][p, q] += sgn * 1e-4
                    if p != q:
                        th[0][q, p] += sgn * 1e-4
                sites2, _ = build(th)
                mpo2 = [core.Tensor.from_dict(ctx, d) for d in sites2]
                st2 = dmrg.restart_state(ctx, mpo2, st)
                st2, _, _ = _converge(ctx, mpo2, nel, M, tole * 0.1, 8, st2)
                vals.append(dmrg.gradient_sweep(ctx, st2, checkpoint=4).energy)
            fd = (vals[0] - vals[1]) / 2e-4
            adj = grads["fp64"].get(par, 0.0)
            if par[0] == "h" and par[1] != par[2]:
                adj += grads["fp64"].get(("h", par[2], par[1]), 0.0)
            fd_rows.append({"param": list(map(str, par)), "adjoint": adj, "fd": fd,
                            "rel": abs(adj - fd) / max(1.0, abs(fd))})
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


def warm_compare(args, ctx, st):
    """From the FP64-converged state, the same number of further sweeps in FP64 and
    in split precision (identical start, same fixed point): energies sweep by sweep
    and sweep times at convergence."""
    from mpsxx_gb300 import core, dmrg

    out = {}
    for name, prec in (("fp64", core.FP64), ("split", core.SPLIT_TF32)):
        core.set_precision(ctx, prec)
        s2 = dmrg.DeviceState(st.mpo, list(st.wave), list(st.lenv), list(st.renv), st.M)
        rows = []
        for _ in range(args.warm_sweeps):
            log = dmrg.make_sweep(ctx, s2, args.tole)
            rows.append({"seconds": log.seconds, "energy": log.energy, "n_sigma": log.n_sigma,
                         "n_sigma_fp64": int(log.times.get("n_sigma_fp64", 0)), "sigma_flops": log.sigma_flops})
        out[name] = rows
    core.set_precision(ctx, core.FP64)
    de = [abs(a["energy"] - b["energy"]) for a, b in zip(out["split"], out["fp64"])]
    t64 = sum(r["seconds"] for r in out["fp64"])
    t32 = sum(r["seconds"] for r in out["split"])
    out["abs_dE_per_sweep"] = de
    out["abs_dE_max"] = max(de)
    out["seconds_per_sweep_fp64"] = t64 / len(out["fp64"])
    out["seconds_per_sweep_split"] = t32 / len(out["split"])
    out["speedup"] = t64 / t32
    return out


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


def cpu_sigma_oracle(wl):
    """The oracle's H_eff*psi on the same bond (host cores, NumPy BLAS threads): every
    block task of both Gemm's, timed as one whole step.  Returns the baseline record and
    the oracle's sigma blocks {tag: ndarray} for the parity check."""
    from oracle import dmrg as od
    from oracle import qsd as oq

    def to_oracle(t):
        d = t.to_dict()
        a = oq.QSDArray(d["q"], d["qshape"], d["dshape"])
        a.blocks = d["blocks"]
        return a

    mL, mR, psi = to_oracle(wl["mL"]), to_oracle(wl["mR"]), to_oracle(wl["psi"])
    cores = os.cpu_count() or 1
    tasks = []
    out = oq.QSDArray()
    t0 = time.perf_counter()
    scr = od.compute_sigma_vector(mL, mR, psi, out, tasks)
    dt = time.perf_counter() - t0
    fl = sigma_task_flops(tasks, mL, mR, psi, scr)
    rec = {"value": fl / dt / 1e12, "unit": "TFLOP/s", "cores": cores, "kind": "port",
           "sample": f"oracle (NumPy) H_eff*psi on all {len(psi.blocks)} psi blocks of the same bond, "
                     f"one full step of {dt:.1f} s, NumPy BLAS threads on {cores} cores"}
    return rec, out.blocks


def sigma_vs_oracle(gpu_blocks, oracle_blocks) -> dict:
    """Largest block-wise difference of the device FP64 sigma from the oracle's, relative
    to the largest |sigma| element."""
    import numpy as np

    scale = max(float(np.abs(b).max()) for b in oracle_blocks.values() if b.size)
    worst = 0.0
    for t, b in oracle_blocks.items():
        g = gpu_blocks.get(t)
        if g is None:
            worst = max(worst, float(np.abs(b).max()) / scale)
        else:
            worst = max(worst, float(np.abs(g - b).max()) / scale)
    extra = [t for t in gpu_blocks if t not in oracle_blocks and np.abs(gpu_blocks[t]).max() > 0]
    return {"max_rel_err": worst, "blocks": len(oracle_blocks), "extra_nonzero_blocks": len(extra)}


def sigma_task_flops(tasks, mL, mR, psi, scr) -> float:
    """2*m*n*k summed over the enumerated (A, B) pairs of both sigma Gemm's."""
    fl = 0.0
    for name, tl in tasks:
        for _, pairs in tl:
            for ta, tb in pairs:
                if name == "LxPsi":
                    a, b = mL.blocks[ta], psi.blocks[tb]
                    fl += 2.0 * a.shape[0] * a.shape[2] * b.shape[1]
                else:
                    a, b = scr.blocks[ta], mR.blocks[tb]
                    fl += 2.0 * a.shape[0] * a.shape[2] * b.shape[0]
    return fl


def run_reference(args, ws, rank):
    """Reference arm: the reference's CPU algorithm for the path on the host cores.

    The reference (C++ over Boost, BTAS and MKL) does not build in this image (no
    Boost, no CBLAS/LAPACKE headers), so its NumPy restatement (the oracle port)
    is timed; the workload is built on the GPU machine through the product path and
    copied to the host first."""
    if rank != 0:
        return
    from mpsxx_gb300 import core

    ctx = core.Context(0)
    wl = build_workload(args, ctx)
    samples = []
    for _ in range(max(1, args.steps)):
        s, _ = cpu_sigma_oracle(wl)
        samples.append(s["value"])
    v = sum(samples) / len(samples)
    out = {"impl": "reference", "metric": "H_eff*psi TFLOP/s (FP64-equivalent), n=20 QC, M=512, middle bond",
           "value": v, "unit": "TFLOP/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": f"qc n={args.norb} K={args.nchol} seed={args.seed} M={args.M} bond={wl['bond']}",
                      "W": wl["W"]},
           "cpu_baseline": {"value": v, "unit": "TFLOP/s", "cores": os.cpu_count() or 1, "kind": "port",
                            "sample": s["sample"]},
           "e2e": {"value": v, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_init(args)
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
    wl = build_workload(args, ctx)
    mL, mR, psi = wl["mL"], wl["mR"], wl["psi"]
    sig = psi.like()
    # one call builds and caches the plan
    core.compute_sigma_vector(ctx, mL, mR, psi, sig)
    ctx.sync()
    c0 = ctx.counters()
    fl_per_step = c0["sigma_flops"] / max(1, c0["sigma_calls"])
    bytes_alg = 8 * (mL.nnz + mR.nnz + 2 * psi.nnz)
    inputs_bytes = 8 * (mL.nnz + mR.nnz + psi.nnz)
    l2 = "inputs larger than L2" if inputs_bytes > L2_BYTES else "L2 flushed between steps"
    flush = None if inputs_bytes > L2_BYTES else torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")

    # FP64 reference timing of the same step (CUDA events on the context's stream)
    core.set_precision(ctx, core.FP64)
    s64 = sig.like()
    core.compute_sigma_vector(ctx, mL, mR, psi, s64)
    ref64 = s64.download()
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
    # accuracy of this step against the FP64 step
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
    bond = bond_compare(ctx, wl, args.M, args.tole) if args.bond_step else None
    # the sweep comparison and the CPU baseline belong to the one-GPU line; replicas
    # (N > 1) time H_eff*psi only
    sections = {}
    t_sec = time.perf_counter()
    sweep = sweep_compare(args, local) if not args.no_sweep and ws == 1 else None
    sections["sweeps"] = time.perf_counter() - t_sec
    t_sec = time.perf_counter()
    grad = gradient_bench(args, local) if args.gradient else None
    sections["gradient"] = time.perf_counter() - t_sec
    t_sec = time.perf_counter()
    scan_res = scan_bench(args, local) if args.scan else None
    sections["scan"] = time.perf_counter() - t_sec
    out = None
    if rank == 0:
        achieved = fl_per_step / kt["sigma_kernels_s"] / 1e12
        if args.precision == "split":
            # TF32 dense rate = half the measured BF16 rate; 3 products per FP64-equivalent product
            tf32 = peaks["bf16_tflops"] / 2.0
            traffic = MEASURED_TRAFFIC.get((args.precision, args.norb, args.nchol, args.seed, args.M))
            roof = {"bound": "tensor", "achieved": achieved, "peak": tf32 / 3.0, "unit": "TFLOP/s",
                    "frac": achieved / (tf32 / 3.0), "traffic": traffic,
                    "traffic_note": "DRAM bytes per H_eff*psi (all launches of the step) from ncu; algorithmic "
                                    "bytes are hbm_algorithmic_bytes" if traffic else None,
                    "hbm_algorithmic_bytes": bytes_alg,
                    "peak_source": f"{src} bf16_tflops/2 (TF32 dense) /3 (3-product split), FP64-equivalent"}
        else:
            roof = {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                    "frac": achieved / fp64_peak, "traffic": None,
                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run (FP64 CUDA-core pipe)"}
        roof.update({"kernel_ms": kt["sigma_kernels_s"] * 1e3,
                     "hbm_algorithmic_gbs": bytes_alg / kt["sigma_kernels_s"] / 1e9,
                     "hbm_peak_gbs": peaks.get("hbm_gbs"), "hbm_peak_source": src})
        out = {
            "metric": "H_eff*psi TFLOP/s (FP64-equivalent), n=20 QC, M=512, middle bond",
            "value": value, "unit": "TFLOP/s", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "tf32x3-split (fp64 in/out)" if args.precision == "split" else "f64",
            "data": "synthetic: seeded integrals, seeded random MPS of bond dimension 512",
            "config": {"workload": f"qc n={args.norb} K={args.nchol} seed={args.seed} M={args.M} "
                                   f"bond=({wl['bond']},{wl['bond'] + 1})",
                       "W": wl["W"], "D_rows": sum(psi.shape()[1][0]), "D_cols": sum(psi.shape()[1][1]),
                       "nnz_psi": psi.nnz, "nnz_L": mL.nnz, "nnz_R": mR.nnz, "flops_per_step": fl_per_step,
                       "l2": l2, "parallelism": f"replicas{ws}", "precision": args.precision},
            "gpu_launches": int(launches),
            "e2e": {"value": job_tflops(ws, fl_per_step, e2e_s), "unit": "TFLOP/s", "ms_per_step": e2e_s * 1e3,
                    "h2d_bytes_per_step": 8 * psi.nnz, "d2h_bytes_per_step": 8 * psi.nnz},
            "roofline": roof,
            "fp64_path": {"ms_per_step": fp64_s * 1e3, "value": fl_per_step / fp64_s / 1e12, "unit": "TFLOP/s",
                          "peak": fp64_peak, "frac": fl_per_step / fp64_s / 1e12 / fp64_peak,
                          "speedup_of_headline": fp64_s / kt["sigma_kernels_s"]},
            "accuracy": {"max_rel_err_vs_fp64": rel},
            "sigma_tuning": [{"w_scratch_mb": b / 2**20, "target_tiles": tt, "fp32_intermediate": f, "ms": ms}
                             for b, tt, f, ms in tuning],
            "sigma_plan": plan_stats,
            "bond_step": bond,
            "sweeps": sweep,
            "gradient": grad,
            "scan": scan_res,
            "clocks": clk.summary(),
            "section_seconds": {k: round(v, 1) for k, v in sections.items()},
        }
        if not args.no_cpu_baseline and ws == 1:
            rec, oblocks = cpu_sigma_oracle(wl)
            out["cpu_baseline"] = rec
            # a fresh FP64 sigma (the timing loops above accumulate into their outputs)
            core.set_precision(ctx, core.FP64)
            s_par = psi.like()
            core.compute_sigma_vector(ctx, mL, mR, psi, s_par)
            core.set_precision(ctx, core.SPLIT_TF32 if args.precision == "split" else core.FP64)
            out["parity"] = {"sigma_vs_oracle_c2": sigma_vs_oracle(s_par.to_dict()["blocks"], oblocks)}
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
