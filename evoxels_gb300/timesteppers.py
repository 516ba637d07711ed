"""Time steppers backed by the CUDA library.

``PseudoSpectralIMEX`` (evoxels/timesteppers.py:64-89) and ``ForwardEuler``
(evoxels/timesteppers.py:32-43) with the reference's ``(problem, dt)``
constructor, ``order`` and functional ``step(t, u) -> u``.  Both add
``advance(u, nsteps)``, which runs ``nsteps`` steps inside the library (the
IMEX update fused into the next step's rhs pass, forward Euler temporally
blocked), and which ``TimeDependentSolver`` uses between output frames.
"""

from __future__ import annotations

import ctypes as C
import threading
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from .problem_definition import CahnHilliard, ReactionDiffusion
from .voxelgrid import cuda_stream, evx_bc


class ChPlan:
    """An ``evx_ch_plan`` plus its device workspace (one per grid shape/spacing/device)."""

    def __init__(self, vg, grads=False, cufft3d=False, fused_yz=False, bc=None):
        self.vg = vg
        self.grid = vg.evx_grid()
        self.grads = grads
        h = C.c_void_p()
        flags = (1 if grads else 0) | (2 if cufft3d else 0) | (4 if fused_yz else 0)
        with torch.cuda.device(vg.device):
            if bc is None:
                _lib.check(_lib.lib().evx_ch_plan_create(C.byref(h), self.grid, flags), "evx_ch_plan_create")
            else:   # normalised BC tuple: the mirrored-x step for a non-periodic x axis
                _lib.check(_lib.lib().evx_ch_plan_create_bc(C.byref(h), self.grid, evx_bc(bc), flags),
                           "evx_ch_plan_create_bc")
        self.handle = h
        nbytes = int(_lib.lib().evx_ch_workspace_bytes(h))
        self.workspace = torch.empty(nbytes, dtype=torch.uint8, device=vg.device)
        self.n = int(np.prod(vg.shape))

    def __del__(self):
        try:
            if self.handle:
                _lib.lib().evx_ch_plan_destroy(self.handle)
                self.handle = None
        except Exception:  # noqa: BLE001 - interpreter shutdown
            pass


_plan_lock = threading.Lock()
_plans = {}


def get_plan(vg, grads=False, cufft3d=False, fused_yz=False, bc=None):
    """Cached plan per grid; ``cufft3d`` forces cuFFT's 3-D transforms instead of the
    (y, z) transforms plus the fused x-pass used for power-of-two ``Nx``; ``fused_yz``
    replaces cuFFT's (y, z) transforms by the fused cluster kernels (opt-in); ``bc``
    (normalised BC tuple) selects the mirrored-x step for a non-periodic x axis."""
    if bc is not None and all(kind == "periodic" for kind, _ in bc):
        bc = None
    bkey = None if bc is None else tuple((k, tuple(float(x) for x in v) if v is not None else None) for k, v in bc)
    key = (vg.shape, vg.spacing, str(vg.device), bool(grads), bool(cufft3d), bool(fused_yz), bkey)
    with _plan_lock:
        p = _plans.get(key)
        if p is None:
            p = ChPlan(vg, grads, cufft3d, fused_yz, bc)
            _plans[key] = p
        return p


def clear_plans():
    with _plan_lock:
        _plans.clear()


class TimeStepper:
    """Interface of evoxels/timesteppers.py:9-29."""

    @property
    def order(self) -> int:
        raise NotImplementedError

    def step(self, t, u):
        raise NotImplementedError


@dataclass
class PseudoSpectralIMEX(TimeStepper):
    """Semi-implicit Fourier step ``u + irfftn(prefac * rfftn(rhs(u)))`` (evoxels/timesteppers.py:64-89)."""
    problem: CahnHilliard
    dt: float

    def __post_init__(self):
        if not isinstance(self.problem, CahnHilliard):
            raise NotImplementedError("evoxels_gb300's spectral step is implemented for CahnHilliard")
        self.problem.verify_fft_bc_config()
        self.pad = self.problem.pad_fft_bc
        self._plan = get_plan(self.problem.vg, bc=self.problem.bc)
        self._params = self.problem.evx_params(self.dt)
        self._nonfinite = None

    @property
    def order(self) -> int:
        return 1

    @property
    def _fft_prefac(self):
        """``dt / (1 - dt*fourier_symbol)`` as a tensor (API parity; the kernels compute it in place)."""
        return self.dt / (1 - self.dt * self.problem.fourier_symbol)

    def _check(self, u):
        u = self.problem.vg.check_field(u)
        if u.shape[0] != 1:
            # the reference transforms over (C, Nx, Ny, Nz) and so couples channels;
            # evoxels_gb300 builds the single-field step only
            raise NotImplementedError("PseudoSpectralIMEX in evoxels_gb300 steps one field (C == 1)")
        return u

    def step(self, t, u):
        u = self._check(u)
        out = torch.empty_like(u)
        p = self._plan
        _lib.check(_lib.lib().evx_ch_step(p.handle, u.data_ptr(), out.data_ptr(), self._params,
                                          p.workspace.data_ptr(), cuda_stream()), "evx_ch_step")
        return out

    def advance(self, u, nsteps, traj=None, nonfinite=None):
        """``nsteps`` steps from ``u`` in one library call; ``traj`` receives u_1..u_n."""
        u = self._check(u)
        out = torch.empty_like(u)
        p = self._plan
        tp = 0
        if traj is not None:
            if traj.dtype != torch.float32 or not traj.is_contiguous() or traj.numel() < nsteps * p.n:
                raise ValueError("traj must be a contiguous float32 tensor holding nsteps fields")
            tp = traj.data_ptr()
        nf = nonfinite.data_ptr() if nonfinite is not None else None
        _lib.check(_lib.lib().evx_ch_forward(p.handle, u.data_ptr(), out.data_ptr(), int(nsteps), tp or None,
                                             self._params, nf, p.workspace.data_ptr(), cuda_stream()),
                   "evx_ch_forward")
        return out


@dataclass
class ForwardEuler(TimeStepper):
    """``u + dt*rhs(t, u)`` (evoxels/timesteppers.py:32-43)."""
    problem: object
    dt: float
    steps_per_pass: int = 1

    @property
    def order(self) -> int:
        return 1

    def step(self, t, u):
        if isinstance(self.problem, ReactionDiffusion):
            return self.advance(u, 1)
        u = self.problem.vg.check_field(u)
        r = self.problem.rhs(t, u)
        out = torch.empty_like(u)
        _lib.check(_lib.lib().evx_fe_update(u.data_ptr(), r.data_ptr(), float(np.float32(self.dt)),
                                            out.data_ptr(), u.numel(), cuda_stream()), "evx_fe_update")
        return out

    def advance(self, u, nsteps):
        if not isinstance(self.problem, ReactionDiffusion):
            for _ in range(nsteps):
                u = self.step(0.0, u)
            return u
        pr = self.problem
        u = pr.vg.check_field(u)
        out = torch.empty_like(u)
        scratch = torch.empty_like(u[0]) if nsteps > 1 else None
        g = pr.vg.evx_grid()
        L = _lib.lib()
        for ch in range(u.shape[0]):
            _lib.check(L.evx_fd_forward(u[ch].data_ptr(), out[ch].data_ptr(),
                                        scratch.data_ptr() if scratch is not None else None, g, pr._evx_bc,
                                        float(np.float32(pr.D)), float(np.float32(self.dt)), int(nsteps),
                                        int(self.steps_per_pass), cuda_stream()), "evx_fd_forward")
        return out


@dataclass
class RungeKutta4(TimeStepper):
    """Classical explicit Runge-Kutta scheme of order 4 (evoxels/timesteppers.py:46-61)
    for any problem with a GPU ``rhs``: four rhs evaluations, the stage inputs
    ``u + c*k`` and the final ``u + dt/6*(k1 + 2k2 + 2k3 + k4)`` as fused
    elementwise kernels, in the reference's float32 operation order."""
    problem: object
    dt: float

    @property
    def order(self) -> int:
        return 4

    def _stage(self, u, k, c):
        out = torch.empty_like(u)
        _lib.check(_lib.lib().evx_fe_update(u.data_ptr(), k.data_ptr(), float(np.float32(c)), out.data_ptr(),
                                            u.numel(), cuda_stream()), "evx_fe_update")
        return out

    def step(self, t, u):
        u = self.problem.vg.check_field(u)
        dt = self.dt
        k1 = self.problem.rhs(t, u)
        k2 = self.problem.rhs(t + 0.5 * dt, self._stage(u, k1, 0.5 * dt))
        k3 = self.problem.rhs(t + 0.5 * dt, self._stage(u, k2, 0.5 * dt))
        k4 = self.problem.rhs(t + dt, self._stage(u, k3, dt))
        out = torch.empty_like(u)
        _lib.check(_lib.lib().evx_rk4_combine(u.data_ptr(), k1.data_ptr(), k2.data_ptr(), k3.data_ptr(),
                                              k4.data_ptr(), float(np.float32(dt / 6)), out.data_ptr(),
                                              u.numel(), cuda_stream()), "evx_rk4_combine")
        return out

