"""Time steppers backed by the CUDA library.

``PseudoSpectralIMEX`` (evoxels/timesteppers.py:64-89) and ``ForwardEuler``
(evoxels/timesteppers.py:32-43) with the reference's ``(problem, dt)``
constructor, ``order`` and functional ``step(t, u) -> u``.  Both add
``advance(u, nsteps)``, which runs ``nsteps`` steps inside the library (the
IMEX update fused into the next step's rhs pass, forward Euler temporally
blocked), and which ``TimeDependentSolver`` uses between output frames.
``RungeKutta4`` (:46-61), ``ExponentialEuler`` (:136-199), ``RKC1`` (:202-244)
and ``RKC2`` (:246-295) drive any problem whose ``rhs`` runs in the library,
their stage combinations as fused kernels in the reference's float32 order.
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

    def __init__(self, vg, grads=False, cufft3d=False, fused_yz=False, bc=None, cufft_yz=False, z_pass=False):
        self.vg = vg
        self.grid = vg.evx_grid()
        self.grads = grads
        h = C.c_void_p()
        flags = (1 if grads else 0) | (2 if cufft3d else 0) | (4 if fused_yz else 0) | (8 if cufft_yz else 0) | \
            (16 if z_pass else 0)
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


def get_plan(vg, grads=False, cufft3d=False, fused_yz=False, bc=None, cufft_yz=False, z_pass=False):
    """Cached plan per grid; ``cufft3d`` forces cuFFT's 3-D transforms instead of the
    (y, z) transforms plus the fused x-pass used for power-of-two ``Nx``; ``fused_yz``
    replaces cuFFT's (y, z) transforms by the fused cluster kernels (opt-in); for
    nz = 256 the z pass is the library's own by default (y-contiguous spectrum),
    ``z_pass`` uses it for nz in 32/64/128 too, ``cufft_yz`` keeps cuFFT's 2-D (y, z)
    plans for every nz; ``bc`` (normalised BC tuple) selects the mirrored-x step for
    a non-periodic x axis."""
    if bc is not None and all(kind == "periodic" for kind, _ in bc):
        bc = None
    bkey = None if bc is None else tuple((k, tuple(float(x) for x in v) if v is not None else None) for k, v in bc)
    key = (vg.shape, vg.spacing, str(vg.device), bool(grads), bool(cufft3d), bool(fused_yz), bkey, bool(cufft_yz),
           bool(z_pass))
    with _plan_lock:
        p = _plans.get(key)
        if p is None:
            p = ChPlan(vg, grads, cufft3d, fused_yz, bc, cufft_yz, z_pass)
            _plans[key] = p
        return p


def clear_plans():
    with _plan_lock:
        _plans.clear()


def mult_table(plan, table):
    """A real multiplier table over the (extended) rfft grid, shaped like the
    reference's ``phi_1_k_squared`` ([Nx_ext, Ny, Nz//2+1]), as the contiguous
    float32 device table of ``evx_spectral_update`` on ``plan``: the plan's
    spectrum order (``evx_ch_mult_layout``; 1 is [Nx_ext, Nz//2+1, Ny])."""
    t = table.to(torch.float32)
    t = t.reshape(t.shape[-3:])
    layout = int(_lib.lib().evx_ch_mult_layout(plan.handle))
    if layout not in (0, 1):
        raise RuntimeError(f"evx_ch_mult_layout returned {layout}")
    return (t.transpose(1, 2) if layout == 1 else t).contiguous()


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
        return self.problem.vg.check_field(u)

    def step(self, t, u):
        """One step of every channel.  The reference transforms the whole ``(C, Nx, Ny, Nz)`` field, but
        its multiplier does not depend on the channel frequency, so the channel transform and its inverse
        cancel and the step is the single-field step of each channel (up to rounding)."""
        u = self._check(u)
        out = torch.empty_like(u)
        p = self._plan
        for ch in range(u.shape[0]):
            _lib.check(_lib.lib().evx_ch_step(p.handle, u[ch].data_ptr(), out[ch].data_ptr(), self._params,
                                              p.workspace.data_ptr(), cuda_stream()), "evx_ch_step")
        return out

    def advance(self, u, nsteps, traj=None, nonfinite=None, t0=0.0):
        """``nsteps`` steps from ``u`` in one library call; ``traj`` receives u_1..u_n.
        (``t0``: the time of ``u``; the Cahn-Hilliard rhs does not depend on it.)"""
        u = self._check(u)
        out = torch.empty_like(u)
        p = self._plan
        tp = 0
        if traj is not None:
            if u.shape[0] != 1:
                raise NotImplementedError("a kept trajectory is built for one channel (C == 1)")
            if traj.dtype != torch.float32 or not traj.is_contiguous() or traj.numel() < nsteps * p.n:
                raise ValueError("traj must be a contiguous float32 tensor holding nsteps fields")
            tp = traj.data_ptr()
        nf = nonfinite.data_ptr() if nonfinite is not None else None
        for ch in range(u.shape[0]):   # channels step independently (see step)
            _lib.check(_lib.lib().evx_ch_forward(p.handle, u[ch].data_ptr(), out[ch].data_ptr(), int(nsteps),
                                                 tp or None, self._params, nf, p.workspace.data_ptr(),
                                                 cuda_stream()), "evx_ch_forward")
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

    def _fused(self):
        """Forward Euler of a source-free reaction-diffusion problem runs in ``evx_fd_forward``."""
        return isinstance(self.problem, ReactionDiffusion) and self.problem.source_free

    def step(self, t, u):
        if self._fused():
            return self.advance(u, 1, t0=t)
        u = self.problem.vg.check_field(u)
        r = self.problem.rhs(t, u)
        out = torch.empty_like(u)
        _lib.check(_lib.lib().evx_fe_update(u.data_ptr(), r.data_ptr(), float(np.float32(self.dt)),
                                            out.data_ptr(), u.numel(), cuda_stream()), "evx_fe_update")
        return out

    def advance(self, u, nsteps, t0=0.0):
        """``nsteps`` steps from ``u`` at time ``t0``; step k sees the time ``t0 + k*dt``."""
        if not self._fused():
            for k in range(nsteps):
                u = self.step(t0 + k * self.dt, u)
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
        fused = getattr(self.problem, "rhs_stage", None)   # the stage input formed inside the rhs kernel
        if fused is not None:
            k2 = fused(t + 0.5 * dt, u, k1, 0.5 * dt)
            k3 = fused(t + 0.5 * dt, u, k2, 0.5 * dt)
            k4 = fused(t + dt, u, k3, dt)
        else:
            k2 = self.problem.rhs(t + 0.5 * dt, self._stage(u, k1, 0.5 * dt))
            k3 = self.problem.rhs(t + 0.5 * dt, self._stage(u, k2, 0.5 * dt))
            k4 = self.problem.rhs(t + dt, self._stage(u, k3, dt))
        out = torch.empty_like(u)
        _lib.check(_lib.lib().evx_rk4_combine(u.data_ptr(), k1.data_ptr(), k2.data_ptr(), k3.data_ptr(),
                                              k4.data_ptr(), float(np.float32(dt / 6)), out.data_ptr(),
                                              u.numel(), cuda_stream()), "evx_rk4_combine")
        return out


@dataclass
class ExponentialEuler(TimeStepper):
    """Exponential Euler / ETD1 (evoxels/timesteppers.py:136-199; Hochbruck,
    Lubich, Selhofer 1998): ``u + irfftn(dt*phi1(dt*L)*rfftn(pad(rhs(u))))``
    for any problem with a GPU ``rhs`` and a ``fourier_symbol`` L.  The
    multiplier table ``dt*phi1(dt*L)`` is built once on the grid's device with
    the reference's formula (Pade(6,6) for |z| < 0.5); each step is the
    problem's rhs kernel plus ``evx_spectral_update`` (cuFFT over (y, z), the
    x-pass with the table multiply and the x mirror extension fused, or cuFFT
    3-D for other Nx)."""
    problem: object
    dt: float

    def __post_init__(self):
        self.problem.verify_fft_bc_config()
        self.pad = self.problem.pad_fft_bc
        self.phi_1_k_squared = self.phi1(self.dt * self.problem.fourier_symbol)
        self._plan = get_plan(self.problem.vg, bc=self.problem.bc)
        self._mult = mult_table(self._plan, self.dt * self.phi_1_k_squared)

    def phi1(self, z):
        """``(exp(z) - 1)/z`` with the degree-6 Pade form where |z| < 0.5
        (evoxels/timesteppers.py:154-169)."""
        Q = 6
        N = [1, 1 / 26, 5 / 156, 1 / 858, 1 / 5720, 1 / 205920, 1 / 8648640]
        D = [1, -6 / 13, 5 / 52, -5 / 429, 1 / 1144, -1 / 25740, 1 / 1235520]
        phi = (torch.exp(z) - 1) / z
        indx = torch.abs(z) < 0.5
        return self.problem.vg.set(phi, indx, self.phiPade(z[indx], Q, N, D))

    def phiPade(self, z, Q, Ncoeff, Dcoeff):
        """``P_Q(z)/R_Q(z)`` by Horner's rule (evoxels/timesteppers.py:171-189)."""
        numerator = Ncoeff[Q]
        denominator = Dcoeff[Q]
        for k in range(Q - 1, -1, -1):
            numerator = numerator * z + Ncoeff[k]
            denominator = denominator * z + Dcoeff[k]
        return numerator / denominator

    @property
    def order(self) -> int:
        return 1

    def step(self, t, u):
        """One step of every channel (the channel transform of the reference's ``(C, Nx, Ny, Nz)`` FFT
        cancels against its inverse: the table does not depend on the channel frequency)."""
        u = self.problem.vg.check_field(u)
        if isinstance(self.problem, CahnHilliard):
            # the spectral loop's own rhs pass, so that n steps equal advance(u, n) bit for bit
            return self.advance(u, 1, t0=t)
        r = self.problem.rhs(t, u)
        out = torch.empty_like(u)
        p = self._plan
        for ch in range(u.shape[0]):
            _lib.check(_lib.lib().evx_spectral_update(p.handle, u[ch].data_ptr(), r[ch].data_ptr(),
                                                      self._mult.data_ptr(), out[ch].data_ptr(),
                                                      p.workspace.data_ptr(), cuda_stream()), "evx_spectral_update")
        return out

    def advance(self, u, nsteps, nonfinite=None, t0=0.0):
        """``nsteps`` steps from ``u`` at time ``t0``.  For CahnHilliard one library call
        (``evx_ch_forward_mult``: each step's update is fused into the next
        step's rhs pass), bit-identical to ``nsteps`` calls of ``step``; other
        problems step one at a time, step k at the time ``t0 + k*dt``."""
        if not isinstance(self.problem, CahnHilliard):
            for k in range(nsteps):
                u = self.step(t0 + k * self.dt, u)
            return u
        u = self.problem.vg.check_field(u)
        out = torch.empty_like(u)
        p = self._plan
        nf = nonfinite.data_ptr() if nonfinite is not None else None
        prm = self.problem.evx_params(self.dt)
        for ch in range(u.shape[0]):
            _lib.check(_lib.lib().evx_ch_forward_mult(p.handle, u[ch].data_ptr(), out[ch].data_ptr(), int(nsteps),
                                                      self._mult.data_ptr(), prm, nf, p.workspace.data_ptr(),
                                                      cuda_stream()), "evx_ch_forward_mult")
        return out


def _rkc_chebyshev(polygrad, damping):
    """``w0``, ``s`` and the Chebyshev values ``T_s(w0)``, ``T_s'(w0)`` for the
    stage coefficients of evoxels/timesteppers.py:214-217, 258-261, as float32
    CPU tensors (the reference's ``vg.to_backend`` / ``vg.arange`` precision)."""
    w0 = torch.tensor(1 + damping / polygrad ** 2, dtype=torch.float32)
    s = torch.arange(0, polygrad + 1, dtype=torch.float32)
    theta = torch.arccosh(w0)
    T = torch.cosh(s * theta)
    dT = s * torch.sinh(s * theta) / torch.sqrt(w0 ** 2 - 1)
    return w0, s, T, dT


class _RKC(TimeStepper):
    """Shared step of the Runge-Kutta-Chebyshev schemes: ``polygrad`` rhs
    evaluations; the first stage is ``evx_fe_update`` with ``mu11*dt``, every
    later one a fused ``evx_rkc_stage`` over (u, Y_curr, Y_prev, rhs[, rhs_0]).
    The coefficients are float32 tensors, so ``mu1[j]*dt`` and friends round as
    in the reference."""

    _second_order = False

    def _stage_coeffs(self, j):
        dt = self.dt
        c = _lib.EvxRkcCoeffs()
        c.mu0 = float(self.mu0[j])
        c.nu = float(self.nu[j])
        c.one_minus_mu0_nu = float(1 - self.mu0[j] - self.nu[j])
        c.mu1_dt = float(self.mu1[j] * dt)
        c.gamma_dt = float(self.gamma[j] * dt) if self._second_order else 0.0
        return c

    def step(self, t, u):
        u = self.problem.vg.check_field(u)
        L = _lib.lib()
        n = u.numel()
        rhs0 = self.problem.rhs(t, u)
        y_prev, y_curr = u, torch.empty_like(u)
        _lib.check(L.evx_fe_update(u.data_ptr(), rhs0.data_ptr(), float(self.mu11 * self.dt), y_curr.data_ptr(), n,
                                   cuda_stream()), "evx_fe_update")
        r0 = rhs0.data_ptr() if self._second_order else None
        for j in range(self.polygrad - 1):
            rhs = self.problem.rhs(t + float(self.c[j] * self.dt), y_curr)
            y_new = torch.empty_like(u)
            _lib.check(L.evx_rkc_stage(u.data_ptr(), y_curr.data_ptr(), y_prev.data_ptr(), rhs.data_ptr(), r0,
                                       C.byref(self._stage_coeffs(j)), y_new.data_ptr(), n, cuda_stream()),
                       "evx_rkc_stage")
            y_prev, y_curr = y_curr, y_new
        return y_curr


@dataclass
class RKC1(_RKC):
    """Runge-Kutta-Chebyshev scheme of order 1 (evoxels/timesteppers.py:202-244;
    Verwer, Hundsdorfer, Sommeijer 1990) for any problem with a GPU ``rhs``."""
    problem: object
    dt: float
    polygrad: int = 4
    damping: float = 0.05

    def __post_init__(self):
        w0, s, T, dT = _rkc_chebyshev(self.polygrad, self.damping)
        b = 1 / T
        w1 = T[-1] / dT[-1]
        self.mu0 = 2 * w0 * (b[2:] / b[1:-1])
        self.mu1 = 2 * w1 * (b[2:] / b[1:-1])
        self.mu11 = w1 / w0
        self.nu = -(b[2:] / b[:-2])
        self.c = w1 * (dT / T)[1:-1]

    @property
    def order(self) -> int:
        return 1


@dataclass
class RKC2(_RKC):
    """Runge-Kutta-Chebyshev scheme of order 2 (evoxels/timesteppers.py:246-295)
    for any problem with a GPU ``rhs``."""
    problem: object
    dt: float
    polygrad: int = 4
    damping: float = 2 / 13

    _second_order = True

    def __post_init__(self):
        w0, s, T, dT = _rkc_chebyshev(self.polygrad, self.damping)
        d2T = (s * s * T - w0 * dT) / (w0 ** 2 - 1)
        b = d2T / dT ** 2
        b[0] = b[2]
        b[1] = b[2]
        w1 = dT[-1] / d2T[-1]
        self.mu0 = 2 * w0 * (b[2:] / b[1:-1])
        self.mu1 = 2 * w1 * (b[2:] / b[1:-1])
        self.mu11 = b[1] * w1
        self.nu = -(b[2:] / b[:-2])
        self.gamma = -(1 - b[1:-1] * T[1:-1]) * self.mu1
        self.c = w1 * (d2T / dT)[1:-1]
        self.c[0] = self.c[1] / dT[2]

    @property
    def order(self) -> int:
        return 2
