"""Record the block structure of the C2 middle bond of a converged DMRG state.

C2: synthetic QC Hamiltonian n=20, 20 electrons, Sz=0, K=40 Cholesky vectors,
seed 1, M=512.  Split-precision two-site sweeps from the reference's initial
state until the sweep energy changes by less than 1e-7 (at most 12 sweeps),
then the orthogonality centre is moved to site 9 by forward canonicalisation.
The quantum numbers and dimensions of the three MPS bonds around sites 9 and
10 are written to tests/golden/c2_bond_structure.json; the bench builds its
H_eff*psi workload from them (seeded random values) in both of its arms.

    python tests/golden/make_c2_structure.py      (needs a GPU)
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    import __graft_entry__

    __graft_entry__.build()
    from mpsxx_gb300 import core, dmrg, mpogen

    n, M, bond = 20, 512, 9
    h1, eri = mpogen.synthetic_qc_integrals(n, 2 * n, 1)
    ctx = core.Context(0)
    core.set_precision(ctx, core.SPLIT_TF32)
    mpo = [core.Tensor.from_dict(ctx, d) for d in mpogen.qc_mpo(h1, eri)]
    st = dmrg.make_initial_state(ctx, mpo, n, 0, M)
    energies = []
    for _ in range(12):
        energies.append(dmrg.make_sweep(ctx, st, 1e-9).energy)
        if len(energies) > 1 and abs(energies[-1] - energies[-2]) < 1e-7:
            break
    dmrg.advance_left(ctx, st, bond)
    left, right = st.wave[bond], st.wave[bond + 1]
    lq, ld = left.shape()
    rq, rd = right.shape()
    out = {"workload": "qc n=20 K=40 seed=1 M=512, middle bond (9,10) of the converged state",
           "sweep_energies": energies, "q_total": list(left.q),
           "left": {"q": [list(q) for q in lq[0]], "d": ld[0]},
           "middle": {"q": [list(q) for q in lq[2]], "d": ld[2]},
           "right": {"q": [list(q) for q in rq[2]], "d": rd[2]},
           "right_site_left_index": {"q": [list(q) for q in rq[0]], "d": rd[0]},
           "lenv": {k: v for k, v in zip(("qshape", "dshape"), st.lenv[bond].shape())},
           "renv": {k: v for k, v in zip(("qshape", "dshape"), st.renv[bond + 1].shape())}}
    out["lenv"]["qshape"] = [[list(q) for q in x] for x in out["lenv"]["qshape"]]
    out["renv"]["qshape"] = [[list(q) for q in x] for x in out["renv"]["qshape"]]
    path = os.path.join(HERE, "c2_bond_structure.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(path, "sectors", len(ld[0]), len(ld[2]), len(rd[2]), "dims", sum(ld[0]), sum(ld[2]), sum(rd[2]))


if __name__ == "__main__":
    main()
