"""The pullback rules the CUDA adjoint kernels implement (`csrc/evx_adjoint.cu`, and the tile kernels of
`csrc/evx_ch_fast_adj.cu` with and without x ghosts), restated in float64 torch and checked against autograd
through the oracle's Cahn-Hilliard rhs: periodic, and a Neumann or Dirichlet x axis, where the ghosts'
cotangents fold back into the boundary cell (g = 0 on the ghost side, the boundary plane's outer x face
weighted by 1 - a in mub and by 1 + a in the cbar face sum, mub continued by a*mub into the ghost)."""

import pytest
import torch

import oracle


def _pad_yz(f):
    """Periodic ghost layer in y and z of a (1, nx, ny, nz) field."""
    f = torch.cat([f[:, :, -1:], f, f[:, :, :1]], dim=2)
    return torch.cat([f[:, :, :, -1:], f, f[:, :, :, :1]], dim=3)


def _pad_x(f, kind, ghost_lo, ghost_hi):
    """x ghost layer of a (1, nx, ., .) field: periodic, or the given ghost planes."""
    if kind == "periodic":
        return torch.cat([f[:, -1:], f, f[:, :1]], dim=1)
    return torch.cat([ghost_lo, f, ghost_hi], dim=1)


def pullback_rules(u, g, eps, D, bc):
    """J_r(u)^T g for the rhs r(u) of ``oracle.ch_rhs`` with the default bulk term and unit spacing."""
    kind, vals = oracle.normalize_bc(bc)[0]
    a = -1.0 if kind == "dirichlet" else 1.0
    v_lo, v_hi = (vals if kind == "dirichlet" else (0.0, 0.0))
    kap, w = 2.0 * eps, 18.0 / eps
    c = torch.clip(u, 0, 1)

    def pad_state(f):   # the reference's padding of c and mu: ghost a*cell + b
        lo, hi = f[:, :1], f[:, -1:]
        if kind == "dirichlet":
            lo, hi = 2 * v_lo - lo, 2 * v_hi - hi
        return _pad_yz(_pad_x(f, kind, lo, hi))

    def pad_cot(f, ghost_factor):   # cotangents: ghost = ghost_factor * boundary cell (0 for g)
        return _pad_yz(_pad_x(f, kind, ghost_factor * f[:, :1], ghost_factor * f[:, -1:]))

    def lap(p):
        return oracle.laplace(p, torch.ones(3, dtype=p.dtype))

    cp = pad_state(c)
    mu = w * c * (1 - c) * (1 - 2 * c) - kap * lap(cp)
    mp = pad_state(mu)
    gp = pad_cot(g, 0.0)
    nx = u.shape[1]
    inner = (slice(None), slice(1, -1), slice(1, -1), slice(1, -1))

    def shift(p, axis, s):   # neighbour s (+1 / -1) along axis of the interior cells of a padded field
        idx = [slice(None), slice(1, -1), slice(1, -1), slice(1, -1)]
        idx[axis + 1] = slice(1 + s, p.shape[axis + 1] - 1 + s)
        return p[tuple(idx)]

    mub = torch.zeros_like(u)
    acc = torch.zeros_like(u)
    for axis in range(3):
        c0, g0, m0 = cp[inner], gp[inner], mp[inner]
        faces = {}
        for s in (-1, 1):
            cn, gn, mn = shift(cp, axis, s), shift(gp, axis, s), shift(mp, axis, s)
            cf = 0.5 * (c0 + cn)
            fb = D * (g0 - gn) if s > 0 else D * (gn - g0)     # Fb on the face, lo minus hi
            gm = (mn - m0) if s > 0 else (m0 - mn)             # mu gradient across the face
            faces[s] = (fb * cf * (1 - cf), fb * gm * (1 - 2 * cf))
        wm, wp = torch.ones_like(u), torch.ones_like(u)
        cm, cpw = torch.ones_like(u), torch.ones_like(u)
        if axis == 0 and kind != "periodic":
            wm = wm * torch.where(torch.arange(nx).view(1, nx, 1, 1) == 0, 1 - a, 1.0)
            wp = wp * torch.where(torch.arange(nx).view(1, nx, 1, 1) == nx - 1, 1 - a, 1.0)
            cm = cm * torch.where(torch.arange(nx).view(1, nx, 1, 1) == 0, 1 + a, 1.0)
            cpw = cpw * torch.where(torch.arange(nx).view(1, nx, 1, 1) == nx - 1, 1 + a, 1.0)
        mub = mub + wm * faces[-1][0] - wp * faces[1][0]
        acc = acc + 0.5 * (cm * faces[-1][1] + cpw * faces[1][1])
    lmb = lap(pad_cot(mub, a))
    cbar = w * (1 - 6 * c + 6 * c * c) * mub - kap * lmb + acc
    return torch.where((u >= 0) & (u <= 1), cbar, torch.zeros_like(cbar))


@pytest.mark.parametrize("bc", [None, ("neumann", "periodic", "periodic"),
                                (("dirichlet", (0.0, 0.0)), "periodic", "periodic"),
                                (("dirichlet", (0.3, 0.8)), "periodic", "periodic")])
def test_pullback_rules_equal_autograd(bc):
    shape = (7, 5, 6)
    u = torch.tensor(0.5 + 1.6 * (oracle.seeded_unit_field(shape, 72) - 0.5)).unsqueeze(0)   # some outside [0, 1]
    g = torch.tensor(oracle.seeded_unit_field(shape, 73) - 0.5).unsqueeze(0)
    eps, D = 1.3, 0.9
    x = u.clone().requires_grad_(True)
    r = oracle.ch_rhs(x, eps=eps, D=D, bc=bc)
    (ref,) = torch.autograd.grad(r, x, grad_outputs=g)
    got = pullback_rules(u, g, eps, D, bc)
    assert ((u < 0) | (u > 1)).any()   # the clip mask is exercised
    assert torch.allclose(got, ref, rtol=0, atol=1e-12 * float(ref.abs().max()))
