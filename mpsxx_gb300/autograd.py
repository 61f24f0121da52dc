"""torch.autograd verification harness over the C ABI.

E(theta) is the DMRG ground-state energy of a parameterised Hamiltonian family;
its backward is the adjoint gradient: dE/dW from the merged-operator adjoint at
every bond (``dmrg.gradient_sweep``), pulled through the MPO generator's
parameter Jacobian (``dmrg.parameter_gradient``).  Consecutive evaluations restart
from the previous converged state with the new Hamiltonian, so finite-difference
checks cost a few sweeps each.  The harness is for verification: parameters live
on the host, the work runs on the context's device.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import core, dmrg, mpogen


class DMRGEnergy(torch.autograd.Function):
    """E = model(theta); dE/dtheta from the adjoint (no second derivatives)."""

    @staticmethod
    def forward(fctx, theta: torch.Tensor, model) -> torch.Tensor:
        e, grad = model.energy_and_gradient(theta.detach().cpu().double().numpy())
        fctx.save_for_backward(torch.as_tensor(grad, dtype=theta.dtype, device=theta.device))
        return theta.new_tensor(e)

    @staticmethod
    def backward(fctx, g_e: torch.Tensor):
        (grad,) = fctx.saved_tensors
        return g_e * grad, None


class HubbardChain:
    """Open Hubbard chain with site-dependent parameters, theta = (t_0..t_{L-2}, U_0..U_{L-1});
    t_i is the one-electron integral h_{i,i+1}."""

    def __init__(self, ctx: core.Context, L: int, n_elec: int, M: int, tole: float = 1e-10, max_sweeps: int = 12,
                 warm_sweeps: int = 4, checkpoint: int = 4, precision: int = core.FP64):
        self.ctx, self.L, self.n_elec, self.M = ctx, L, n_elec, M
        self.tole, self.max_sweeps, self.warm_sweeps = tole, max_sweeps, warm_sweeps
        self.checkpoint, self.precision = checkpoint, precision
        self.state: Optional[dmrg.DeviceState] = None
        self.last = None

    def split(self, theta: np.ndarray):
        return theta[: self.L - 1], theta[self.L - 1:]

    def energy_and_gradient(self, theta: np.ndarray):
        ctx = self.ctx
        t, U = self.split(theta)
        sites, jacs = mpogen.hubbard_mpo(self.L, t, U, jacobian=True)
        saved = core.get_precision(ctx)
        core.set_precision(ctx, self.precision)
        try:
            mpo = [core.Tensor.from_dict(ctx, d) for d in sites]
            if self.state is None:
                st = dmrg.make_initial_state(ctx, mpo, self.n_elec, 0, self.M)
                nmax = self.max_sweeps
            else:
                st = dmrg.restart_state(ctx, mpo, self.state)
                nmax = self.warm_sweeps
            e_prev = None
            for it in range(nmax):
                log = dmrg.make_sweep(ctx, st, self.tole)
                if e_prev is not None and abs(log.energy - e_prev) < self.tole:
                    break
                e_prev = log.energy
            self.state = st
            g = dmrg.gradient_sweep(ctx, st, checkpoint=self.checkpoint)
        finally:
            core.set_precision(ctx, saved)
        tags = [m.blocks()[0] for m in st.mpo]
        dE = dmrg.parameter_gradient(g.site_grads, tags, jacs)
        grad = np.array([dE.get(("t", k), 0.0) for k in range(self.L - 1)] +
                        [dE.get(("U", k), 0.0) for k in range(self.L)])
        self.last = g
        return g.energy, grad

    def __call__(self, theta: torch.Tensor) -> torch.Tensor:
        return DMRGEnergy.apply(theta, self)
