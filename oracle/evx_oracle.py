"""Operation-by-operation CPU restatement of the reference's hot path.

TEST INFRASTRUCTURE ONLY: the oracle the CUDA path is checked against.  Every
function names the reference file:line whose arithmetic it follows (paths are
relative to the evoxels project root).  Floating-point operations are written
in the same order and association as the reference so that, in fp32, the
finite-difference parts reproduce the reference's rounding exactly.

Fields are torch CPU tensors of shape ``(C, Nx, Ny, Nz)`` (z fastest), the
layout ``VoxelGridTorch.init_scalar_field`` produces (evoxels/voxelgrid.py:126-130).

Boundary conditions use the reference's normalised form
``((kind, values), (kind, values), (kind, values))`` for the x, y, z axes,
``kind`` in {'periodic', 'neumann', 'dirichlet'}
(evoxels/problem_definition.py:60-115).
"""

from __future__ import annotations

import numpy as np
import torch

__all__ = [
    "normalize_bc",
    "pad_periodic",
    "pad_bc",
    "grid_factors",
    "laplace",
    "to_face",
    "grad_face",
    "ch_rhs",
    "rd_rhs",
    "rfft_k_squared",
    "imex_prefac",
    "imex_step",
    "rfft_k_squared_nonperiodic",
    "x_bc_kind",
    "pad_fft",
    "grad_center",
    "normal_laplace",
    "ac_rhs",
    "rk4_step",
    "ac_rk4_run",
    "rkc_coeffs",
    "rkc_step",
    "phi1",
    "etd1_multiplier",
    "fe_step",
    "ch_imex_run",
    "rd_fe_run",
    "steady_state_run",
    "ch_imex_vjp",
    "ch_imex_loss_grads",
    "seeded_ch_field",
    "seeded_unit_field",
    "rel_to_max",
]

_SLAB = slice(1, -1)


# ----------------------------------------------------------------------------
# Boundary conditions
# ----------------------------------------------------------------------------

def normalize_bc(bc):
    """Normalise a BC spec the way evoxels/problem_definition.py:60-103 does.

    ``None`` or ``'fully_periodic'`` -> periodic on all axes
    (evoxels/problem_definition.py:62-65).  Raises ``ValueError`` with the
    reference's messages for malformed specs.
    """
    if bc is None or bc == "fully_periodic":
        return (("periodic", None),) * 3
    if len(bc) != 3:
        raise ValueError("bc must contain exactly three axis entries ordered as (x, y, z).")
    out = []
    for axis_bc in bc:
        if isinstance(axis_bc, str):
            if axis_bc == "dirichlet":
                raise ValueError("Dirichlet BCs require explicit values ('dirichlet', (left, right)).")
            if axis_bc not in {"periodic", "neumann"}:
                raise ValueError(f"Unsupported BC type: {axis_bc}")
            out.append((axis_bc, None))
            continue
        if len(axis_bc) != 2:
            raise ValueError(
                "Each axis boundary specification must be either a string or "
                "a tuple like ('dirichlet', (left, right))."
            )
        kind, values = axis_bc
        if kind not in {"periodic", "dirichlet", "neumann"}:
            raise ValueError(f"Unsupported BC type: {kind}")
        if kind == "dirichlet":
            if values is None or len(values) != 2:
                raise ValueError("Dirichlet BCs require two boundary values.")
            out.append((kind, tuple(values)))
        else:
            if values is not None:
                raise ValueError(f"{kind} BCs do not accept boundary values.")
            out.append((kind, None))
    return tuple(out)


def pad_periodic(field):
    """Circular ghost layer of width 1 (evoxels/voxelgrid.py:194-195)."""
    return torch.nn.functional.pad(field, (1, 1, 1, 1, 1, 1), mode="circular")


def pad_bc(field, bc):
    """Generic cell-centred ghost padding (evoxels/boundary_conditions.py:33-59).

    Periodic pad first, then per axis in x, y, z order: Neumann copies the
    first/last interior slab into the ghost slab, Dirichlet writes
    ``2*v - interior``.  The specialised forms
    (evoxels/boundary_conditions.py:16-31) give identical values.
    """
    bc = normalize_bc(bc)
    padded = pad_periodic(field)
    for axis, (kind, values) in enumerate(bc):
        if kind == "periodic":
            continue
        dim = axis + 1

        def sl(i):
            idx = [slice(None)] * 4
            idx[dim] = i
            return tuple(idx)

        if kind == "neumann":
            padded[sl(0)] = padded[sl(1)]
            padded[sl(-1)] = padded[sl(-2)]
        elif kind == "dirichlet":
            padded[sl(0)] = 2.0 * values[0] - padded[sl(1)]
            padded[sl(-1)] = 2.0 * values[1] - padded[sl(-2)]
        else:  # pragma: no cover - normalize_bc rejects it
            raise ValueError(f"Unsupported BC type: {kind}")
    return padded


# ----------------------------------------------------------------------------
# Stencils (evoxels/fd_stencils.py)
# ----------------------------------------------------------------------------

def grid_factors(spacing, dtype):
    """``div_dx``, ``div_dx2`` as the reference builds them (evoxels/voxelgrid.py:29-30)."""
    sp = torch.tensor(np.array(spacing), dtype=dtype)
    return 1 / sp, 1 / sp ** 2


def laplace(padded, div_dx2):
    """Compact 7-point Laplacian on a padded field (evoxels/fd_stencils.py:62-75)."""
    c = padded[:, 1:-1, 1:-1, 1:-1]
    left, right = padded[:, :-2, 1:-1, 1:-1], padded[:, 2:, 1:-1, 1:-1]
    bottom, top = padded[:, 1:-1, :-2, 1:-1], padded[:, 1:-1, 2:, 1:-1]
    back, front = padded[:, 1:-1, 1:-1, :-2], padded[:, 1:-1, 1:-1, 2:]
    return (right + left) * div_dx2[0] + \
           (top + bottom) * div_dx2[1] + \
           (front + back) * div_dx2[2] - \
           2 * c * torch.sum(div_dx2)


def to_face(field, axis):
    """Face average ``0.5*(f[i+1] + f[i])`` along ``axis`` (evoxels/fd_stencils.py:20-30)."""
    d = axis + 1
    n = field.shape[d]
    return 0.5 * (field.narrow(d, 1, n - 1) + field.narrow(d, 0, n - 1))


def grad_face(field, axis, div_dx):
    """Face gradient ``(f[i+1] - f[i]) * 1/h`` along ``axis`` (evoxels/fd_stencils.py:32-42)."""
    d = axis + 1
    n = field.shape[d]
    return (field.narrow(d, 1, n - 1) - field.narrow(d, 0, n - 1)) * div_dx[axis]


# ----------------------------------------------------------------------------
# Right-hand sides (evoxels/problem_definition.py)
# ----------------------------------------------------------------------------

def _default_mu_hom(eps):
    # evoxels/problem_definition.py:304-305
    return lambda c, lib=None: 18 / eps * c * (1 - c) * (1 - 2 * c)


def ch_rhs(u, eps=3.0, D=1.0, bc=None, spacing=(1.0, 1.0, 1.0), mu_hom=None):
    """``CahnHilliard.rhs`` (evoxels/problem_definition.py:328-371).

    ``c = clip(u,0,1)``; ``mu = mu_hom(c) - 2*eps*laplace(pad_bc(c))``;
    ``rhs = D * sum_axes grad_face( to_face(c)*(1-to_face(c)) * grad_face(pad_bc(mu)) )``.
    ``eps`` and ``D`` may be python floats or 0-d tensors (autograd use).
    """
    bc = normalize_bc(bc)
    div_dx, div_dx2 = grid_factors(spacing, u.dtype)
    if mu_hom is None:
        mu_hom = _default_mu_hom(eps)
    c = torch.clip(u, 0, 1)
    c_bc = pad_bc(c, bc)
    lap = laplace(c_bc, div_dx2)
    try:
        mh = mu_hom(c, torch)
    except TypeError:
        mh = mu_hom(c)
    mu = mh - 2 * eps * lap
    mu = pad_bc(mu, bc)

    inner = [(slice(None), slice(None), slice(1, -1), slice(1, -1)),
             (slice(None), slice(1, -1), slice(None), slice(1, -1)),
             (slice(None), slice(1, -1), slice(1, -1), slice(None))]
    divergence = None
    for axis in range(3):
        cf = to_face(c_bc, axis)
        flux = cf * (1 - to_face(c_bc, axis)) * grad_face(mu, axis, div_dx)
        term = grad_face(flux, axis, div_dx)[inner[axis]]
        divergence = term if divergence is None else divergence + term
    return D * divergence


def rd_rhs(u, D=1.0, bc=None, spacing=(1.0, 1.0, 1.0), f=None, t=0.0):
    """``ReactionDiffusion.rhs`` (evoxels/problem_definition.py:226-229).

    ``D*laplace(pad_bc(u)) + f(t, u)``; the default source is the python int 0
    (evoxels/problem_definition.py:202-203).
    """
    bc = normalize_bc(bc)
    _, div_dx2 = grid_factors(spacing, u.dtype)
    lap = laplace(pad_bc(u, bc), div_dx2)
    if f is None:
        src = 0
    else:
        try:
            src = f(t, u, torch)
        except TypeError:
            src = f(t, u)
    return D * lap + src


# ----------------------------------------------------------------------------
# Spectral machinery (evoxels/voxelgrid.py:84-114, evoxels/timesteppers.py:64-89)
# ----------------------------------------------------------------------------

def rfft_k_squared(shape, spacing=(1.0, 1.0, 1.0), dtype=torch.float32):
    """``VoxelGrid.rfft_k_squared`` (evoxels/voxelgrid.py:84-90,110-114).

    ``k_i = 2*pi*fftfreq(n_i, h_i)`` on x and y, ``2*pi*rfftfreq`` on z, summed
    as ``kx**2 + ky**2 + kz**2`` on an ``ij`` mesh, in ``dtype`` (the reference
    uses torch's default dtype here).
    """
    ax = [2 * torch.pi * torch.fft.fftfreq(n, d, dtype=dtype) for n, d in zip(shape, spacing)]
    az = 2 * torch.pi * torch.fft.rfftfreq(shape[2], spacing[2], dtype=dtype)
    kx, ky, kz = torch.meshgrid(ax[0], ax[1], az, indexing="ij")
    return kx ** 2 + ky ** 2 + kz ** 2


def rfft_k_squared_nonperiodic(shape, spacing=(1.0, 1.0, 1.0), dtype=torch.float32):
    """``VoxelGrid.rfft_k_squared_nonperiodic`` for the cell-centred grid
    (evoxels/voxelgrid.py:116-124): the x frequencies of the mirrored grid,
    ``2*pi*fftfreq(2*Nx, h_x)``; y and z as in ``rfft_k_squared``."""
    ax = 2 * torch.pi * torch.fft.fftfreq(2 * shape[0], spacing[0], dtype=dtype)
    ay = 2 * torch.pi * torch.fft.fftfreq(shape[1], spacing[1], dtype=dtype)
    az = 2 * torch.pi * torch.fft.rfftfreq(shape[2], spacing[2], dtype=dtype)
    kx, ky, kz = torch.meshgrid(ax, ay, az, indexing="ij")
    return kx ** 2 + ky ** 2 + kz ** 2


def x_bc_kind(bc):
    """The x-axis kind of a BC spec: 'periodic', 'neumann' or 'dirichlet'."""
    return normalize_bc(bc)[0][0]


def imex_prefac(shape, dt, eps=3.0, D=1.0, A=0.25, spacing=(1.0, 1.0, 1.0), dtype=torch.float32, bc=None):
    """``PseudoSpectralIMEX._fft_prefac`` for ``CahnHilliard``.

    ``symbol = -2*eps*D*A*(k^2)^2`` (evoxels/problem_definition.py:303) and
    ``prefac = dt / (1 - dt*symbol)`` (evoxels/timesteppers.py:77); a Neumann or
    Dirichlet x axis takes the mirrored-grid k^2 (evoxels/problem_definition.py:169-177).
    """
    if x_bc_kind(bc) in ("neumann", "dirichlet"):
        k2 = rfft_k_squared_nonperiodic(shape, spacing, dtype)
    else:
        k2 = rfft_k_squared(shape, spacing, dtype)
    symbol = -2 * eps * D * A * k2 ** 2
    return dt / (1 - dt * symbol)


def pad_fft(dc, bc=None):
    """``CahnHilliard.pad_fft_bc`` on the cell-centred grid
    (evoxels/boundary_conditions.py:60-70): periodic x is the identity, Neumann x
    appends the x-flipped field (even extension), Dirichlet x its negative."""
    kind = x_bc_kind(bc)
    if kind == "neumann":
        return torch.cat((dc, torch.flip(dc, [1])), 1)
    if kind == "dirichlet":
        return torch.cat((dc, -torch.flip(dc, [1])), 1)
    return dc


def imex_step(u, prefac, rhs_fn, bc=None):
    """``PseudoSpectralIMEX.step`` (evoxels/timesteppers.py:85-89).

    ``dc = pad_fft(rhs(u))``; the transform runs over the full 4-D shape of ``dc``
    including the channel axis; the update is trimmed back to ``u``'s x extent.
    """
    dc = pad_fft(rhs_fn(u), bc)
    dc_fft = prefac * torch.fft.rfftn(dc, s=dc.shape)
    update = torch.fft.irfftn(dc_fft, s=dc.shape)[:, :u.shape[1]]
    return u + update


def phi1(z):
    """``ExponentialEuler.phi1`` (evoxels/timesteppers.py:154-189): ``(exp(z)-1)/z``,
    and where |z| < 0.5 the (6,6) Pade form of Hochbruck, Lubich, Selhofer
    (1998) by Horner's rule, in ``z``'s dtype."""
    num = [1, 1 / 26, 5 / 156, 1 / 858, 1 / 5720, 1 / 205920, 1 / 8648640]
    den = [1, -6 / 13, 5 / 52, -5 / 429, 1 / 1144, -1 / 25740, 1 / 1235520]
    phi = (torch.exp(z) - 1) / z
    small = torch.abs(z) < 0.5
    zs = z[small]
    p, q = num[6], den[6]
    for k in range(5, -1, -1):
        p = p * zs + num[k]
        q = q * zs + den[k]
    phi[small] = p / q
    return phi


def etd1_multiplier(symbol, dt):
    """The ETD1 spectral multiplier ``dt * phi1(dt * symbol)``
    (evoxels/timesteppers.py:148,197); one ETD1 step is ``imex_step`` with it."""
    return dt * phi1(dt * symbol)


def fe_step(u, dt, rhs_fn):
    """``ForwardEuler.step`` (evoxels/timesteppers.py:42-43): ``u + dt*rhs``."""
    return u + dt * rhs_fn(u)


def ch_imex_run(u0, nsteps, dt=0.1, eps=3.0, D=1.0, A=0.25, spacing=(1.0, 1.0, 1.0),
                mu_hom=None, k_dtype=None, keep=None, bc=None):
    """``nsteps`` Cahn-Hilliard IMEX steps from ``u0``; returns the final state.

    ``keep`` (optional list) receives every intermediate state, ``u0`` first.
    ``bc``: the problem's BC spec (at most x non-periodic, as the reference allows).
    """
    shape = tuple(u0.shape[1:])
    prefac = imex_prefac(shape, dt, eps, D, A, spacing, k_dtype or u0.dtype, bc)
    u = u0
    if keep is not None:
        keep.append(u)
    for _ in range(nsteps):
        u = imex_step(u, prefac, lambda v: ch_rhs(v, eps, D, bc, spacing, mu_hom), bc)
        if keep is not None:
            keep.append(u)
    return u


def rd_fe_run(u0, nsteps, dt, D=1.0, bc=None, spacing=(1.0, 1.0, 1.0)):
    """``nsteps`` ``ForwardEuler`` steps of ``ReactionDiffusion`` with ``f = 0``."""
    u = u0
    for _ in range(nsteps):
        u = fe_step(u, dt, lambda v: rd_rhs(v, D, bc, spacing))
    return u


# ----------------------------------------------------------------------------
# Adjoint oracle: torch autograd through the restated step
# ----------------------------------------------------------------------------

def ch_imex_vjp(u, lam, dt=0.1, eps=3.0, D=1.0, A=0.25, spacing=(1.0, 1.0, 1.0), mu_hom=None):
    """Vector-Jacobian product of one IMEX step: returns ``(J^T lam, dD, deps)``.

    ``dD``/``deps`` are the contributions of this step to the parameter
    gradients when ``D`` and ``eps`` enter both the rhs and the spectral
    prefactor (``eps`` also sets the default bulk term ``18/eps`` unless
    ``mu_hom`` pins it).
    """
    u = u.detach().clone().requires_grad_(True)
    Dt = torch.tensor(float(D), dtype=u.dtype, requires_grad=True)
    et = torch.tensor(float(eps), dtype=u.dtype, requires_grad=True)
    shape = tuple(u.shape[1:])
    k2 = rfft_k_squared(shape, spacing, u.dtype)
    prefac = dt / (1 - dt * (-2 * et * Dt * A * k2 ** 2))
    mh = mu_hom if mu_hom is not None else (lambda c, lib=None: 18 / et * c * (1 - c) * (1 - 2 * c))
    out = imex_step(u, prefac, lambda v: ch_rhs(v, et, Dt, None, spacing, mh))
    gu, gD, ge = torch.autograd.grad(out, (u, Dt, et), grad_outputs=lam)
    return gu.detach(), float(gD), float(ge)


def ch_imex_loss_grads(c0, target, nsteps, dt=0.1, eps=3.0, D=1.0, A=0.25,
                       spacing=(1.0, 1.0, 1.0), mu_hom=None):
    """Loss ``mean((u_T - target)^2)`` and its gradients w.r.t. ``c0``, ``D``, ``eps``.

    Torch autograd through ``nsteps`` restated IMEX steps (the reference has no
    torch gradient path of its own; this is the autograd-through-the-reference
    construction, evoxels/problem_definition.py:290-371 with tensor ``D``/``eps``).
    """
    c0 = c0.detach().clone().requires_grad_(True)
    Dt = torch.tensor(float(D), dtype=c0.dtype, requires_grad=True)
    et = torch.tensor(float(eps), dtype=c0.dtype, requires_grad=True)
    shape = tuple(c0.shape[1:])
    k2 = rfft_k_squared(shape, spacing, c0.dtype)
    prefac = dt / (1 - dt * (-2 * et * Dt * A * k2 ** 2))
    mh = mu_hom if mu_hom is not None else (lambda c, lib=None: 18 / et * c * (1 - c) * (1 - 2 * c))
    u = c0
    for _ in range(nsteps):
        u = imex_step(u, prefac, lambda v: ch_rhs(v, et, Dt, None, spacing, mh))
    loss = torch.mean((u - target) ** 2)
    g0, gD, ge = torch.autograd.grad(loss, (c0, Dt, et))
    return float(loss.detach()), g0.detach(), float(gD), float(ge)


# ----------------------------------------------------------------------------
# Seeded inputs and error metric
# ----------------------------------------------------------------------------

# ----------------------------------------------------------------------------
# Two-phase Allen-Cahn and the classical Runge-Kutta scheme
# ----------------------------------------------------------------------------

def grad_center(padded, axis, div_dx):
    """``0.5*(f[i+1] - f[i-1]) * div_dx[axis]`` at cell centres (evoxels/fd_stencils.py:44-54)."""
    hi = [slice(None), slice(1, -1), slice(1, -1), slice(1, -1)]
    lo = list(hi)
    hi[axis + 1] = slice(2, None)
    lo[axis + 1] = slice(None, -2)
    return 0.5 * (padded[tuple(hi)] - padded[tuple(lo)]) * div_dx[axis]


def normal_laplace(padded, div_dx, div_dx2):
    """Normal part of the Laplacian, compact 19-point stencil (evoxels/fd_stencils.py:77-103):
    face second differences weighted by the squared centred gradients, plus the
    mixed second differences of each plane weighted by gradient products, over
    ``|grad|^2`` (set to 1 where ``|grad|^2 <= 1e-7``)."""
    f = padded
    C = f[:, 1:-1, 1:-1, 1:-1]
    L, R = f[:, :-2, 1:-1, 1:-1], f[:, 2:, 1:-1, 1:-1]
    B, T = f[:, 1:-1, :-2, 1:-1], f[:, 1:-1, 2:, 1:-1]
    Bk, F = f[:, 1:-1, 1:-1, :-2], f[:, 1:-1, 1:-1, 2:]
    gx, gy, gz = (grad_center(f, a, div_dx) for a in range(3))
    n = gx ** 2 * (R - 2 * C + L) * div_dx2[0] + \
        gy ** 2 * (T - 2 * C + B) * div_dx2[1] + \
        gz ** 2 * (F - 2 * C + Bk) * div_dx2[2] + \
        0.5 * gx * gy * (f[:, 2:, 2:, 1:-1] + f[:, :-2, :-2, 1:-1] -
                         f[:, :-2, 2:, 1:-1] - f[:, 2:, :-2, 1:-1]) * div_dx[0] * div_dx[1] + \
        0.5 * gx * gz * (f[:, 2:, 1:-1, 2:] + f[:, :-2, 1:-1, :-2] -
                         f[:, :-2, 1:-1, 2:] - f[:, 2:, 1:-1, :-2]) * div_dx[0] * div_dx[2] + \
        0.5 * gy * gz * (f[:, 1:-1, 2:, 2:] + f[:, 1:-1, :-2, :-2] -
                         f[:, 1:-1, :-2, 2:] - f[:, 1:-1, 2:, :-2]) * div_dx[1] * div_dx[2]
    norm2 = gx ** 2 + gy ** 2 + gz ** 2
    norm2[norm2 <= 1e-7] = 1.0
    return n / norm2


def ac_rhs(phi, eps=2.0, gab=1.0, M=1.0, force=0.0, curvature=0.01, bc=None, spacing=(1.0, 1.0, 1.0),
           potential=None):
    """``TwoPhaseAllenCahn.rhs`` (evoxels/problem_definition.py:420-447); BCs default to
    Neumann on every axis as the reference's dataclass default."""
    bc = normalize_bc(("neumann", "neumann", "neumann") if bc is None else bc)
    div_dx, div_dx2 = grid_factors(spacing, phi.dtype)
    phi = torch.clip(phi, 0, 1)
    pot = potential(phi) if potential is not None else 18 / eps * phi * (1 - phi) * (1 - 2 * phi)
    phi_pad = pad_bc(phi, bc)
    lap = curvature * laplace(phi_pad, div_dx2)
    n_lap = (1 - curvature) * normal_laplace(phi_pad, div_dx, div_dx2)
    df = gab * (lap + n_lap - pot / 2 / eps) + 3 / eps * phi * (1 - phi) * force
    return M * df


def rk4_step(u, dt, rhs_fn):
    """``RungeKutta4.step`` (evoxels/timesteppers.py:46-61)."""
    k1 = rhs_fn(u)
    k2 = rhs_fn(u + 0.5 * dt * k1)
    k3 = rhs_fn(u + 0.5 * dt * k2)
    k4 = rhs_fn(u + dt * k3)
    return u + (dt / 6) * (k1 + 2 * k2 + 2 * k3 + k4)


def ac_rk4_run(u0, nsteps, dt=0.5, eps=2.0, gab=1.0, M=1.0, force=0.0, curvature=0.01, bc=None,
               spacing=(1.0, 1.0, 1.0)):
    """``nsteps`` RungeKutta4 steps of TwoPhaseAllenCahn (``run_allen_cahn_solver``'s scheme)."""
    u = u0
    for _ in range(nsteps):
        u = rk4_step(u, dt, lambda v: ac_rhs(v, eps, gab, M, force, curvature, bc, spacing))
    return u


def rkc_coeffs(order, polygrad=4, damping=None, dtype=torch.float64):
    """Stage coefficients of RKC1 (evoxels/timesteppers.py:214-229) or RKC2
    (evoxels/timesteppers.py:258-280) from the Chebyshev polynomials T_s at
    w0 = 1 + damping/s^2 (Verwer, Hundsdorfer, Sommeijer 1990), in ``dtype``."""
    if damping is None:
        damping = 0.05 if order == 1 else 2 / 13
    w0 = torch.tensor(1 + damping / polygrad ** 2, dtype=dtype)
    s = torch.arange(0, polygrad + 1, dtype=dtype)
    acw = torch.arccosh(w0)
    T = torch.cosh(s * acw)
    dT = s * torch.sinh(s * acw) / torch.sqrt(w0 ** 2 - 1)
    k = {}
    if order == 1:
        b = 1 / T
        w1 = T[-1] / dT[-1]
        k["mu11"] = w1 / w0
        k["c"] = w1 * (dT / T)[1:-1]
    else:
        d2T = (s * s * T - w0 * dT) / (w0 ** 2 - 1)
        b = d2T / dT ** 2
        b[0] = b[2]
        b[1] = b[2]
        w1 = dT[-1] / d2T[-1]
        k["mu11"] = b[1] * w1
        c = w1 * (d2T / dT)[1:-1]
        c[0] = c[1] / dT[2]
        k["c"] = c
    k["mu0"] = 2 * w0 * (b[2:] / b[1:-1])
    k["mu1"] = 2 * w1 * (b[2:] / b[1:-1])
    k["nu"] = -(b[2:] / b[:-2])
    if order == 2:
        k["gamma"] = -(1 - b[1:-1] * T[1:-1]) * k["mu1"]
    return k


def rkc_step(u, dt, rhs_fn, k):
    """One RKC1 / RKC2 step (evoxels/timesteppers.py:235-244, 284-295) with the
    coefficients ``k`` of :func:`rkc_coeffs`; RKC2 when ``k`` has ``gamma``."""
    r0 = rhs_fn(u)
    y_prev, y = u, u + k["mu11"] * dt * r0
    for j in range(len(k["mu0"])):
        r = rhs_fn(y)
        y_new = k["mu0"][j] * y + k["nu"][j] * y_prev + (1 - k["mu0"][j] - k["nu"][j]) * u + k["mu1"][j] * dt * r
        if "gamma" in k:
            y_new = y_new + k["gamma"][j] * dt * r0
        y_prev, y = y, y_new
    return y


def steady_state_run(u0, step_fn, max_iters, conv_crit=1e-6, check_freq=10):
    """``SteadyStatePseudoTimeSolver._run_loop`` / ``check_convergence``
    (evoxels/solvers.py:218-247): ``diff = u - step(u)``, ``u = step(u)``, and
    at every ``check_freq``-th iteration the per-field measure
    ``torch.linalg.norm(diff[i]) / sqrt(Nx*Ny*Nz)`` in the field's dtype against
    ``conv_crit``.  The iteration counter advances (the reference's loop leaves it
    at 0, which amounts to ``check_freq = 1`` with ``max_iters`` unbounded).

    Returns ``(u, iterations, converged, [(iteration, [rel_change per field]), ...])``.
    """
    u = u0
    it = 0
    converged = False
    checks = []
    nvox = float(np.prod(u0.shape[1:]))
    while not converged and it < max_iters:
        u_next = step_fn(u)
        diff = u - u_next
        if it % check_freq == 0:
            rel = [float(torch.linalg.norm(diff[i]) / np.sqrt(nvox)) for i in range(u.shape[0])]
            checks.append((it, rel))
            converged = all(r <= conv_crit for r in rel)
        u = u_next
        it += 1
    return u, it, converged, checks


def seeded_ch_field(shape, seed):
    """``0.5 + 0.1*U[0,1)`` from ``np.random.default_rng(seed)`` (float64, ``(Nx,Ny,Nz)``)."""
    rng = np.random.default_rng(seed)
    return 0.5 + 0.1 * rng.random(tuple(shape))


def seeded_unit_field(shape, seed):
    """``U[0,1)`` from ``np.random.default_rng(seed)`` (float64, ``(Nx,Ny,Nz)``)."""
    rng = np.random.default_rng(seed)
    return rng.random(tuple(shape))


def rel_to_max(a, ref):
    """``max|a - ref| / max|ref|`` in float64."""
    a = np.asarray(a, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = float(np.max(np.abs(ref)))
    if den == 0.0:
        return float(np.max(np.abs(a - ref)))
    return float(np.max(np.abs(a - ref)) / den)

