"""Differentiable Cahn-Hilliard IMEX trajectories on the GPU.

The reference differentiates its spectral solver with JAX/diffrax forward mode
for parameter estimation (evoxels/inversion.py:51-124).  Here the gradient
comes from a hand-written adjoint of each IMEX step (``evx_ch_adjoint``), with
gradients with respect to the initial field, the mobility ``D`` and the
gradient-energy parameter ``eps`` (``kappa = 2*eps``; the default bulk term
``18/eps`` also depends on ``eps`` unless ``mu_hom`` pins it).

Memory: states are checkpointed every ``checkpoint_every`` steps during the
forward pass; the backward pass recomputes one segment at a time into a
``(K+1)``-state buffer and runs the adjoint through it.  With
``checkpoint_every >= nsteps`` the whole trajectory is kept and nothing is
recomputed.
"""

from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib
from .problem_definition import CahnHilliard
from .timesteppers import get_plan
from .voxelgrid import VoxelGridGB300, cuda_stream, normalize_bc


class CahnHilliardAdjoint:
    """Forward trajectory + adjoint driver on one grid.

    ``pinned_w``: when given, the bulk term is ``pinned_w*c(1-c)(1-2c)``
    independent of ``eps`` (the reference's callable ``mu_hom`` pinned to a
    fixed coefficient); otherwise it is ``18/eps*c(1-c)(1-2c)``.

    ``spectral``: keep each forward step's increment spectrum beside the
    trajectory (when the grid has the x-pass, power-of-two ``Nx``) so the
    adjoint forms the mobility gradient sums by Parseval in k-space; this
    costs one more field-sized buffer per step and saves an inverse FFT and
    two field reads per adjoint step.

    ``bc``: the problem's boundary conditions; a Neumann or Dirichlet x axis
    selects the mirrored-x step (y and z periodic, as the reference's FFT
    steppers require); its parameter gradients use the real-space sums.
    """

    def __init__(self, vg: VoxelGridGB300, dt=0.1, A=0.25, pinned_w=None, spectral=True, bc=None):
        self.vg = vg
        self.dt = float(dt)
        self.A = float(A)
        self.pinned_w = pinned_w
        self.bc = None if bc is None else normalize_bc(bc, vg.convention)
        if self.bc is not None and all(kind == "periodic" for kind, _ in self.bc):
            self.bc = None
        self.mirrored = self.bc is not None
        self.plan = get_plan(vg, grads=not self.mirrored, bc=self.bc)
        self.spec_floats = int(_lib.lib().evx_ch_spectrum_floats(self.plan.handle)) if spectral else 0
        self.n = int(np.prod(vg.shape))
        self._pcache = {}
        self._mse_scratch = torch.empty(int(_lib.lib().evx_mse_scratch_bytes(self.n)), dtype=torch.uint8,
                                        device=vg.device)

    def params(self, D, eps):
        key = (float(D), float(eps))
        p = self._pcache.get(key)
        if p is None:
            p = self._pcache[key] = self._make_params(*key)
        return p

    def _make_params(self, D, eps):
        mu = None if self.pinned_w is None else (lambda c, lib=None, w=self.pinned_w: w * c * (1 - c) * (1 - 2 * c))
        kw = {} if self.bc is None else {"bc": self.bc}
        prob = CahnHilliard(self.vg, eps=float(eps), D=float(D), mu_hom=mu, A=self.A, **kw)
        if self.bc is not None:
            prob.verify_fft_bc_config()
        return prob.evx_params(self.dt)

    def new_spectra(self, nsteps):
        """Buffer for ``nsteps`` stored increment spectra, or None when not kept."""
        if not self.spec_floats:
            return None
        return torch.empty(int(nsteps) * self.spec_floats, dtype=torch.float32, device=self.vg.device)

    def forward(self, u0, nsteps, D, eps, traj=None, spectra=None):
        """``nsteps`` IMEX steps; ``traj`` (optional) receives u_1..u_n, ``spectra``
        (optional, from ``new_spectra``) the increment spectra of the steps."""
        out = torch.empty_like(u0)
        p = self.params(D, eps)
        _lib.check(_lib.lib().evx_ch_forward_spectra(
            self.plan.handle, u0.data_ptr(), out.data_ptr(), int(nsteps),
            traj.data_ptr() if traj is not None else None, spectra.data_ptr() if spectra is not None else None,
            p, None, self.plan.workspace.data_ptr(), cuda_stream()), "evx_ch_forward_spectra")
        return out

    def adjoint(self, states, nsteps, lam, D, eps, grads, spectra=None):
        """Adjoint through ``states`` (``nsteps+1`` consecutive fields); accumulates into ``grads``.
        ``spectra``: the forward's stored spectra of the same steps (optional)."""
        out = torch.empty_like(lam)
        p = self.params(D, eps)
        _lib.check(_lib.lib().evx_ch_adjoint_spectra(
            self.plan.handle, states.data_ptr(), spectra.data_ptr() if spectra is not None else None, int(nsteps),
            lam.data_ptr(), out.data_ptr(), p, grads.data_ptr() if grads is not None else None,
            self.plan.workspace.data_ptr(), cuda_stream()), "evx_ch_adjoint_spectra")
        return out

    def mse(self, u, target, lam=None):
        """Device loss ``mean((u-target)^2)`` (float64 tensor) and optional gradient into ``lam``."""
        loss = torch.empty(1, dtype=torch.float64, device=u.device)
        _lib.check(_lib.lib().evx_mse_grad(u.data_ptr(), target.data_ptr(), self.n,
                                           lam.data_ptr() if lam is not None else None, loss.data_ptr(),
                                           self._mse_scratch.data_ptr(), self._mse_scratch.numel(),
                                           cuda_stream()), "evx_mse_grad")
        return loss

    # ------------------------------------------------------------------------
    def run_forward_checkpointed(self, c0, nsteps, D, eps, K):
        """Forward pass.  Returns ``(u_T, saved)``; ``saved`` holds either the whole
        trajectory (K >= nsteps) or the states every K steps."""
        if K >= nsteps:
            traj = torch.empty((nsteps + 1,) + tuple(c0.shape[1:]), dtype=torch.float32, device=c0.device)
            traj[0].copy_(c0[0])
            spectra = self.new_spectra(nsteps)
            self.forward(traj[0:1], nsteps, D, eps, traj=traj[1:], spectra=spectra)
            return traj[nsteps:nsteps + 1], {"traj": traj, "spectra": spectra}
        cps = [c0]
        u = c0
        s = 0
        while s < nsteps:
            m = min(K, nsteps - s)
            u = self.forward(u, m, D, eps)
            s += m
            if s < nsteps:
                cps.append(u)
        return u, {"cps": cps}

    def backward_checkpointed(self, saved, nsteps, lam_T, D, eps, K, want_params=True):
        """Adjoint through all steps; segments are recomputed from their checkpoints."""
        grads = torch.zeros(3, dtype=torch.float64, device=lam_T.device) if want_params else None
        if "traj" in saved:
            return self.adjoint(saved["traj"], nsteps, lam_T, D, eps, grads, saved.get("spectra")), grads
        cps = saved["cps"]
        seg_buf = torch.empty((K + 1,) + tuple(lam_T.shape[1:]), dtype=torch.float32, device=lam_T.device)
        seg_spec = self.new_spectra(K) if want_params else None
        lam = lam_T
        for si in range(len(cps) - 1, -1, -1):
            m = min(K, nsteps - si * K)
            seg_buf[0].copy_(cps[si][0])
            self.forward(seg_buf[0:1], m, D, eps, traj=seg_buf[1:m + 1], spectra=seg_spec)
            lam = self.adjoint(seg_buf[:m + 1], m, lam, D, eps, grads, seg_spec)
        return lam, grads

    def param_grads(self, grads, eps):
        """Map (dL/dD, dL/dkappa, dL/dw) to (dL/dD, dL/deps)."""
        gD, gK, gW = (float(x) for x in grads.tolist())
        _lib.check_device_status("CahnHilliardAdjoint gradients")
        geps = 2.0 * gK
        if self.pinned_w is None:
            geps += -18.0 / float(eps) ** 2 * gW
        return gD, geps

    def loss_and_grads(self, c0, target, nsteps, D, eps, checkpoint_every=None):
        """MSE loss of u_T against ``target`` and gradients w.r.t. c0, D, eps."""
        K = nsteps if not checkpoint_every else int(checkpoint_every)
        uT, saved = self.run_forward_checkpointed(c0, nsteps, D, eps, K)
        lam = torch.empty_like(uT)
        loss = self.mse(uT, target, lam)
        g0, grads = self.backward_checkpointed(saved, nsteps, lam, D, eps, K)
        gD, geps = self.param_grads(grads, eps)     # reads the device status word
        return float(loss), g0, gD, geps


class CahnHilliardIMEXFunction(torch.autograd.Function):
    """``u_T = IMEX^n(c0; D, eps)`` with the hand-written adjoint as its backward.

    ``apply(c0, D, eps, runner, nsteps, checkpoint_every)``: ``c0`` is a
    ``(1, Nx, Ny, Nz)`` float32 CUDA tensor, ``D``/``eps`` 0-d tensors (or
    floats).  Gradients flow to all three.
    """

    @staticmethod
    def forward(ctx, c0, D, eps, runner, nsteps, checkpoint_every):
        Df, ef = float(D), float(eps)
        K = nsteps if not checkpoint_every else int(checkpoint_every)
        c0 = c0.detach().contiguous()
        uT, saved = runner.run_forward_checkpointed(c0, nsteps, Df, ef, K)
        ctx.runner, ctx.nsteps, ctx.K, ctx.Df, ctx.ef = runner, nsteps, K, Df, ef
        ctx.saved = saved
        ctx.D_is_tensor = isinstance(D, torch.Tensor)
        ctx.e_is_tensor = isinstance(eps, torch.Tensor)
        return uT

    @staticmethod
    def backward(ctx, grad_out):
        r = ctx.runner
        lam, grads = r.backward_checkpointed(ctx.saved, ctx.nsteps, grad_out.contiguous().float(), ctx.Df, ctx.ef,
                                             ctx.K, want_params=ctx.needs_input_grad[1] or ctx.needs_input_grad[2])
        gD = geps = None
        if grads is not None:
            d, e = r.param_grads(grads, ctx.ef)
            gD = torch.tensor(d, dtype=torch.float32) if ctx.D_is_tensor else None
            geps = torch.tensor(e, dtype=torch.float32) if ctx.e_is_tensor else None
        ctx.saved = None
        return lam, gD, geps, None, None, None


def ch_imex_trajectory(c0, D, eps, nsteps, runner, checkpoint_every=None):
    """Differentiable ``nsteps`` IMEX steps (see ``CahnHilliardIMEXFunction``)."""
    return CahnHilliardIMEXFunction.apply(c0, D, eps, runner, int(nsteps), checkpoint_every)


def default_checkpoint_interval(vg, nsteps, budget_bytes=None, spectrum_bytes=0):
    """Largest K whose (K+1)-state segment buffer, K stored spectra of
    ``spectrum_bytes`` each, and n/K checkpoints fit the budget.

    Default budget: half of the device's free memory.
    """
    field = 4 * int(np.prod(vg.shape))
    if budget_bytes is None:
        free, _ = torch.cuda.mem_get_info(vg.device)
        budget_bytes = free // 2
    best = 1
    for K in range(1, nsteps + 1):
        need = (K + 1) * field + K * spectrum_bytes + math.ceil(nsteps / K) * field
        if need <= budget_bytes:
            best = K
    return best


def fit_parameters(runner, c0, target, nsteps, D0, eps0, iters=20, lr=0.05, checkpoint_every=None):
    """Estimate ``(D, eps)`` from an observed final field (the reference's
    parameter-estimation role, evoxels/inversion.py:126-233, with gradients from
    the hand-written adjoint instead of JAX forward mode).

    Adam on ``log D`` and ``log eps`` (positivity, as the reference's
    ``pos_params``).  Returns ``(D, eps, history)``, history holding
    ``(loss, D, eps)`` per iteration.
    """
    x = np.log(np.array([float(D0), float(eps0)]))
    m = np.zeros(2)
    v = np.zeros(2)
    b1, b2 = 0.9, 0.999
    hist = []
    for it in range(1, iters + 1):
        D, eps = np.exp(x)
        loss, _, gD, geps = runner.loss_and_grads(c0, target, nsteps, D, eps, checkpoint_every)
        hist.append((loss, float(D), float(eps)))
        g = np.array([gD * D, geps * eps])           # chain rule to log-space
        m = b1 * m + (1 - b1) * g
        v = b2 * v + (1 - b2) * g * g
        mh, vh = m / (1 - b1 ** it), v / (1 - b2 ** it)
        x = x - lr * mh / (np.sqrt(vh) + 1e-12)
    D, eps = np.exp(x)
    return float(D), float(eps), hist
