"""Problem definitions whose right-hand sides run in the CUDA library.

Same constructor signatures, attributes and error behaviour as the reference's
``CahnHilliard`` (evoxels/problem_definition.py:290-371) and
``ReactionDiffusion`` (evoxels/problem_definition.py:191-229); ``rhs(t, u)``
calls ``evx_ch_rhs`` / ``evx_rd_rhs`` on the grid's CUDA device.

Scope of the CUDA kernels:
* ``CahnHilliard.mu_hom`` must be ``None`` (the default ``18/eps*c(1-c)(1-2c)``),
  a callable equal to ``w*c*(1-c)*(1-2c)`` for some constant ``w`` (the form
  the reference uses when the bulk energy is pinned independently of ``eps``),
  or a callable equal to the regular-solution potential
  ``log(c) - log(1-c) + w*(1-2c)`` (the logarithmic free energy of the
  reference's solver notebook; forward steps only, the adjoint and the batched
  path take the double well).  The callable is probed once on CPU to find the
  form and ``w``; any other form raises ``NotImplementedError``.
* ``ReactionDiffusion.f`` may be any callable ``f(t, u[, lib])``: like the
  reference it is user code, evaluated with ``lib = torch`` on the grid's
  device and added to the stencil kernel's ``D*laplace(u)``; ``None`` (the
  reference's zero source) lets the forward-Euler steps run fused in one
  library call.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, Callable

import numpy as np
import torch

from . import _lib
from .voxelgrid import VoxelGridGB300, cuda_stream, evx_bc, normalize_bc


def _eval_callable(fn, *args):
    try:
        return fn(*args, torch)
    except TypeError:
        return fn(*args)


def double_well_coefficient(mu_hom, eps):
    """Return ``w`` such that ``mu_hom(c) == w*c*(1-c)*(1-2c)``, or raise.

    ``None`` gives the reference default ``w = 18/eps``
    (evoxels/problem_definition.py:304-305).
    """
    if mu_hom is None:
        return 18 / eps
    c = torch.tensor([0.0, 0.05, 0.1, 0.25, 0.3, 0.5, 0.6, 0.8, 0.9, 1.0], dtype=torch.float64)
    basis = c * (1 - c) * (1 - 2 * c)
    try:
        vals = _eval_callable(mu_hom, c)
        vals = torch.as_tensor(vals, dtype=torch.float64).expand_as(c)
    except Exception as e:  # noqa: BLE001 - any failure means: not a supported form
        raise NotImplementedError(f"mu_hom could not be evaluated on a probe tensor: {e}") from e
    w = float(vals[3] / basis[3])
    if not torch.allclose(vals, w * basis, rtol=1e-12, atol=1e-12 * max(1.0, abs(w))):
        raise NotImplementedError(
            "evoxels_gb300 supports mu_hom of the form w*c*(1-c)*(1-2c) only "
            "(the reference default 18/eps*c*(1-c)*(1-2c) or a pinned coefficient)")
    return w


def bulk_potential(mu_hom, eps):
    """``(form, w)`` of a Cahn-Hilliard bulk term: ``(EVX_BULK_DOUBLE_WELL, w)`` for
    ``w*c*(1-c)*(1-2c)`` (``None``: the reference default ``w = 18/eps``) or
    ``(EVX_BULK_REGULAR_SOLUTION, w)`` for ``log(c) - log(1-c) + w*(1-2c)``; raises
    ``NotImplementedError`` for any other callable."""
    try:
        return _lib.EVX_BULK_DOUBLE_WELL, double_well_coefficient(mu_hom, eps)
    except NotImplementedError as e:
        first = e
    c = torch.tensor([0.05, 0.1, 0.25, 0.3, 0.45, 0.6, 0.8, 0.9], dtype=torch.float64)
    logs = torch.log(c) - torch.log(1 - c)
    try:
        vals = torch.as_tensor(_eval_callable(mu_hom, c), dtype=torch.float64).expand_as(c)
    except Exception:  # noqa: BLE001 - not a supported form
        raise first from None
    w = float((vals[2] - logs[2]) / (1 - 2 * c[2]))
    if not torch.allclose(vals, logs + w * (1 - 2 * c), rtol=1e-12, atol=1e-12 * max(1.0, abs(w))):
        raise NotImplementedError(
            "evoxels_gb300 supports mu_hom of the forms w*c*(1-c)*(1-2c) (the reference default "
            "18/eps*c*(1-c)*(1-2c) or a pinned coefficient) and log(c) - log(1-c) + w*(1-2c)") from None
    return _lib.EVX_BULK_REGULAR_SOLUTION, w


def ch_params(eps, D, A, dt, w=None, bulk=0):
    """``EvxChParams``: float32 roundings of the python-double constants the
    reference evaluates (evoxels/problem_definition.py:303-305,
    evoxels/timesteppers.py:77); ``w`` defaults to ``18/eps``; ``bulk`` the
    form of the bulk term (``EVX_BULK_*``)."""
    f = lambda x: float(np.float32(x))  # noqa: E731
    p = _lib.EvxChParams()
    p.bulk = int(bulk)
    p.D = f(D)
    p.kappa = f(2 * eps)
    p.w = f(18 / eps if w is None else w)
    p.A = f(A)
    p.sym_coef = f(-2 * eps * D * A)
    p.dt = f(dt)
    return p


class _BCMixin:
    def initialize_boundary_conditions(self):
        """(evoxels/problem_definition.py:60-115); ghosts are applied in-kernel."""
        self.bc = normalize_bc(getattr(self, "bc", None), self.vg.convention)
        self._evx_bc = evx_bc(self.bc)

    @property
    def bc_type(self):
        return tuple(axis_bc[0] for axis_bc in self.bc)

    def pad_bc(self, u):
        return self.vg.bc.pad_bc(u, self.bc)

    def verify_fft_bc_config(self):
        """(evoxels/problem_definition.py:138-167)."""
        nonperiodic = tuple(a for a, k in zip(("x", "y", "z"), self.bc_type) if k != "periodic")
        if len(nonperiodic) > 1:
            raise ValueError("FFT-based timesteppers currently support at most one non-periodic axis, "
                             f"got {self.bc_type}.")
        if len(nonperiodic) == 1 and nonperiodic[0] != "x":
            raise NotImplementedError(
                "FFT-based timesteppers currently only implement the single non-periodic axis "
                f"case for x; got {self.bc_type}. Axis permutation is not implemented yet.")
        x_bc = self.bc_type[0]
        if x_bc == "periodic":
            self._pad_fft_bc = self.vg.bc.pad_fft_periodic
        elif x_bc == "dirichlet":
            self._pad_fft_bc = self.vg.bc.pad_fft_dirichlet_periodic
        elif x_bc == "neumann":
            self._pad_fft_bc = self.vg.bc.pad_fft_zero_flux_periodic
        else:
            raise ValueError("FFT-based timesteppers only support periodic, dirichlet, or "
                             f"neumann boundary conditions in x, got {x_bc}.")

    def pad_fft_bc(self, u):
        return self._pad_fft_bc(u)

    def k_squared(self):
        """(evoxels/problem_definition.py:169-177): the mirrored grid's k^2 for a
        Neumann or Dirichlet x axis."""
        if self.bc_type[0] in ("dirichlet", "neumann"):
            return self.vg.rfft_k_squared_nonperiodic()
        return self.vg.rfft_k_squared()


@dataclass
class CahnHilliard(_BCMixin):
    vg: VoxelGridGB300
    eps: float = 3.0
    D: float = 1.0
    mu_hom: Callable | None = None
    A: float = 0.25
    bc: tuple = ("periodic", "periodic", "periodic")
    _fourier_symbol: Any = field(init=False, repr=False, default=None)

    def __post_init__(self):
        self.initialize_boundary_conditions()
        self._bulk, self._w = bulk_potential(self.mu_hom, self.eps)
        if self.mu_hom is None:
            eps = self.eps
            self.mu_hom = lambda c, lib=None: 18 / eps * c * (1 - c) * (1 - 2 * c)

    @property
    def order(self):
        return 2

    @property
    def fourier_symbol(self):
        """``-2*eps*D*A*(k^2)^2`` as a tensor (evoxels/problem_definition.py:303)."""
        if self._fourier_symbol is None:
            self._fourier_symbol = -2 * self.eps * self.D * self.A * self.k_squared() ** 2
        return self._fourier_symbol

    def evx_params(self, dt=0.0):
        """float32 roundings of the python-double constants the reference evaluates."""
        return ch_params(self.eps, self.D, self.A, dt, self._w, self._bulk)

    def rhs(self, t, u):
        """``CahnHilliard.rhs`` on the GPU (evoxels/problem_definition.py:328-371)."""
        u = self.vg.check_field(u)
        out = torch.empty_like(u)
        g = self.vg.evx_grid()
        p = self.evx_params()
        L = _lib.lib()
        for ch in range(u.shape[0]):
            _lib.check(L.evx_ch_rhs(u[ch].data_ptr(), out[ch].data_ptr(), g, self._evx_bc, p, cuda_stream()),
                       "evx_ch_rhs")
        return out


@dataclass
class ReactionDiffusion(_BCMixin):
    vg: VoxelGridGB300
    D: float
    f: Callable | None = None
    A: float = 0.25
    bc: tuple = ("periodic", "periodic", "periodic")
    _fourier_symbol: Any = field(init=False, repr=False, default=None)

    def __post_init__(self):
        # None is the reference's zero source (evoxels/problem_definition.py:201-203); any other
        # callable is evaluated every step, as the reference does, so that a source vanishing at
        # some (t, u) is never mistaken for zero
        self.source_free = self.f is None
        if self.f is None:
            self.f = lambda c=None, t=None, lib=None: 0
        self.initialize_boundary_conditions()

    @property
    def order(self):
        return 2

    @property
    def fourier_symbol(self):
        if self._fourier_symbol is None:
            self._fourier_symbol = -self.D * self.A * self.k_squared()
        return self._fourier_symbol

    def _eval_f(self, t, c):
        """The source term ``f(t, c, lib)`` with ``lib = torch`` (evoxels/problem_definition.py:215-220)."""
        return _eval_callable(self.f, t, c)

    def rhs(self, t, u):
        """``D*laplace(pad_bc(u)) + f(t, u)`` (evoxels/problem_definition.py:226-229): the stencil term
        by ``evx_rd_rhs``, then the user's source added (skipped for the zero source)."""
        u = self.vg.check_field(u)
        out = torch.empty_like(u)
        g = self.vg.evx_grid()
        L = _lib.lib()
        for ch in range(u.shape[0]):
            _lib.check(L.evx_rd_rhs(u[ch].data_ptr(), out[ch].data_ptr(), g, self._evx_bc,
                                    float(np.float32(self.D)), cuda_stream()), "evx_rd_rhs")
        if self.source_free:
            return out
        return out + self._eval_f(t, u)


def ac_params(eps, gab, M, force, curvature, w=None):
    """``EvxAcParams``: float32 roundings of the python-double values the
    reference's TwoPhaseAllenCahn.rhs uses (evoxels/problem_definition.py:420-447)."""
    f = lambda x: float(np.float32(x))  # noqa: E731
    p = _lib.EvxAcParams()
    p.w = f(18 / eps if w is None else w)
    p.eps = f(eps)
    p.gab = f(gab)
    p.M = f(M)
    p.force = f(force)
    p.three_over_eps = f(3 / eps)
    p.curvature = f(curvature)
    p.one_minus_curvature = f(1 - curvature)
    return p


@dataclass
class TwoPhaseAllenCahn(_BCMixin):
    """Two-phase Allen-Cahn (evoxels/problem_definition.py:374-447) on the GPU:
    ``M*(gab*(curvature*L(phi) + (1-curvature)*N(phi) - potential/2/eps)
    + 3/eps*phi*(1-phi)*force)`` with the 19-point normal Laplacian N, every BC
    kind, in one fused kernel.  ``potential`` must be the double-well form
    ``w*u*(1-u)*(1-2u)`` (the default ``w = 18/eps``, or a pinned coefficient)."""
    vg: VoxelGridGB300
    eps: float = 2.0
    gab: float = 1.0
    M: float = 1.0
    force: float = 0.0
    curvature: float = 0.01
    potential: Callable | None = None
    bc: tuple = ("neumann", "neumann", "neumann")
    _fourier_symbol: Any = field(init=False, repr=False, default=None)

    def __post_init__(self):
        self.initialize_boundary_conditions()
        self._w = double_well_coefficient(self.potential, self.eps)
        if self.potential is None:
            eps = self.eps
            self.potential = lambda u, lib=None: 18 / eps * u * (1 - u) * (1 - 2 * u)
        self._params = ac_params(self.eps, self.gab, self.M, self.force, self.curvature, self._w)

    @property
    def order(self):
        return 2

    @property
    def fourier_symbol(self):
        """``-M*gab*k^2`` as a tensor (evoxels/problem_definition.py:389)."""
        if self._fourier_symbol is None:
            self._fourier_symbol = -self.M * self.gab * self.k_squared()
        return self._fourier_symbol

    def rhs(self, t, phi):
        """d phi/dt for every channel (evoxels/problem_definition.py:420-447)."""
        phi = self.vg.check_field(phi)
        out = torch.empty_like(phi)
        g = self.vg.evx_grid()
        L = _lib.lib()
        for ch in range(phi.shape[0]):
            _lib.check(L.evx_ac_rhs(phi[ch].data_ptr(), out[ch].data_ptr(), g, self._evx_bc, self._params,
                                    cuda_stream()), "evx_ac_rhs")
        return out

    def rhs_stage(self, t, phi, k, c):
        """``rhs(t, phi + c*k)`` with the stage input formed inside the kernel, bit for bit as
        ``phi + float32(c)*k`` (the Runge-Kutta stages of evoxels/timesteppers.py:57-59)."""
        phi = self.vg.check_field(phi)
        k = self.vg.check_field(k)
        out = torch.empty_like(phi)
        g = self.vg.evx_grid()
        L = _lib.lib()
        cf = float(np.float32(c))
        for ch in range(phi.shape[0]):
            _lib.check(L.evx_ac_rhs_stage(phi[ch].data_ptr(), k[ch].data_ptr(), cf, out[ch].data_ptr(), g,
                                          self._evx_bc, self._params, cuda_stream()), "evx_ac_rhs_stage")
        return out
