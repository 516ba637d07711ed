"""Spectral Cahn-Hilliard step with a Neumann or Dirichlet x axis (the reference's
mirrored FFT extension): against the reference's own fp32 runs (golden
fixtures), the FP64 oracle, cuFFT 3-D on the doubled grid, and through the
solver driver."""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc

pytestmark = pytest.mark.gpu
DEV = "cuda"


def vg_for(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).unsqueeze(0)


@pytest.mark.parametrize("i", range(4))
def test_mirror_x_vs_reference_golden(cuda_lib, i):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    g = load_golden(f"ch_imex_nx_{i}")
    shape = tuple(int(x) for x in g["shape"])
    bc = parse_bc(g["bc"])
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape), eps=float(g["eps"]), D=float(g["D"]), bc=bc),
                            float(g["dt"]))
    u = gpu(g["u0"])
    for _ in range(int(g["n"])):
        u = st.step(0.0, u)
    # reference fp32 (pocketfft) vs ours (cuFFT / x-pass): float32 FFT rounding
    assert oracle.rel_to_max(u.cpu().numpy()[0], g["u"][0]) < 2e-6
    ref = oracle.ch_imex_run(torch.tensor(g["u0"]).unsqueeze(0), int(g["n"]), float(g["dt"]), float(g["eps"]),
                             float(g["D"]), bc=bc).numpy()
    assert oracle.rel_to_max(u.cpu().numpy(), ref) <= 1e-5 * int(g["n"])


BCS = [("neumann", "periodic", "periodic"), (("dirichlet", (0.0, 0.0)), "periodic", "periodic"),
       (("dirichlet", (0.3, 0.8)), "periodic", "periodic")]


# power-of-two nx up to 256 use the x-pass with the extension inside; others cuFFT 3-D on 2*nx
@pytest.mark.parametrize("shape", [(32, 20, 36), (8, 12, 16), (64, 16, 24), (24, 16, 20), (256, 8, 8)])
@pytest.mark.parametrize("b", range(3))
def test_mirror_x_paths_agree_and_match_fp64(cuda_lib, shape, b):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.7, D=1.3, bc=BCS[b])
    u0n = oracle.seeded_ch_field(shape, 8 + b)
    u0 = gpu(u0n)
    outs = []
    for cufft3d in (False, True):
        plan = get_plan(vg, cufft3d=cufft3d, bc=prob.bc)
        out = torch.empty_like(u0)
        _lib.check(cuda_lib.evx_ch_forward(plan.handle, u0.data_ptr(), out.data_ptr(), 3, None,
                                           prob.evx_params(0.1), None, plan.workspace.data_ptr(), cuda_stream()))
        outs.append(out.cpu().numpy())
    assert oracle.rel_to_max(outs[0], outs[1]) < 1e-6
    ref = oracle.ch_imex_run(torch.tensor(u0n).unsqueeze(0), 3, 0.1, 1.7, 1.3, bc=prob.bc).numpy()
    assert oracle.rel_to_max(outs[0], ref) <= 3e-5


def test_mirror_x_driver_and_errors(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.solvers import TimeDependentSolver
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX, get_plan
    from evoxels_gb300.voxelfields import VoxelFields
    shape = (16, 12, 8)
    vf = VoxelFields(shape, domain_size=shape)
    c0 = oracle.seeded_ch_field(shape, 31)
    vf.add_field("c", c0.copy())
    bc = ("neumann", "periodic", "periodic")
    solver = TimeDependentSolver(vf, "c", "torch", problem_cls=CahnHilliard, timestepper_cls=PseudoSpectralIMEX)
    solver.solve(time_increment=0.1, frames=2, max_iters=6, problem_kwargs={"bc": bc}, jit=False, verbose=False)
    ref = oracle.ch_imex_run(torch.tensor(c0).unsqueeze(0), 6, 0.1, bc=bc).numpy()[0]
    assert oracle.rel_to_max(vf.fields["c"], ref) <= 6e-5
    # the reference-side pieces of the mirrored step are exposed too
    prob = CahnHilliard(vg_for(shape), bc=(("dirichlet", (0.0, 1.0)), "periodic", "periodic"))
    st = PseudoSpectralIMEX(prob, 0.1)
    u = torch.rand((1,) + shape, device=DEV)
    assert st.pad(u).shape == (1, 2 * shape[0]) + shape[1:]
    assert torch.equal(st.pad(u)[:, shape[0]:], -torch.flip(u, [1]))
    assert tuple(prob.k_squared().shape) == (2 * shape[0], shape[1], shape[2] // 2 + 1)
    # stored increment spectra are a periodic x-pass feature: a clear error on the mirrored step
    plan = get_plan(prob.vg, bc=prob.bc)
    lam = torch.zeros_like(u)
    spec = torch.zeros(4096, dtype=torch.float32, device=DEV)
    with pytest.raises(NotImplementedError, match="periodic x-pass"):
        _lib.check(cuda_lib.evx_ch_adjoint_spectra(plan.handle, torch.cat([u, u]).data_ptr(), spec.data_ptr(), 1,
                                                   lam.data_ptr(), torch.empty_like(lam).data_ptr(),
                                                   prob.evx_params(0.1), None, plan.workspace.data_ptr(), 0),
                   "adjoint")


def _fp64_mirror_vjp(u0, lam, n, eps, D, bc, dt=0.1):
    """dL/du_0, dL/dD and dL/deps of <lam, u_n> through n FP64 oracle steps of the mirrored-x scheme
    (torch autograd; eps also sets the default bulk term 18/eps)."""
    u = torch.tensor(u0).unsqueeze(0).requires_grad_(True)
    Dt = torch.tensor(float(D), dtype=torch.float64, requires_grad=True)
    et = torch.tensor(float(eps), dtype=torch.float64, requires_grad=True)
    k2 = oracle.rfft_k_squared_nonperiodic(tuple(u0.shape), (1.0, 1.0, 1.0), torch.float64)
    prefac = dt / (1 - dt * (-2 * et * Dt * 0.25 * k2 ** 2))
    mh = lambda c, lib=None: 18 / et * c * (1 - c) * (1 - 2 * c)  # noqa: E731
    v = u
    for _ in range(n):
        v = oracle.imex_step(v, prefac, lambda w: oracle.ch_rhs(w, et, Dt, bc, (1.0, 1.0, 1.0), mh), bc)
    g, gD, ge = torch.autograd.grad(v, (u, Dt, et), grad_outputs=torch.tensor(lam).unsqueeze(0))
    return g[0].numpy(), float(gD), float(ge)


# x-pass with the extension inside (power-of-two nx) and cuFFT 3-D on 2*nx; some voxels outside [0, 1]
@pytest.mark.parametrize("shape", [(16, 12, 20), (12, 10, 16), (8, 6, 12)])
@pytest.mark.parametrize("b", range(3))
def test_mirror_x_adjoint_vs_fp64_autograd(cuda_lib, shape, b):
    """The adjoint of the mirrored-x step (Neumann, homogeneous and inhomogeneous Dirichlet x) over three
    steps of the GPU trajectory against torch autograd through the FP64 oracle's mirrored steps from the
    same float64 field: dL/du_0 within 1e-4 relative to max (the periodic adjoint's bar), dL/dD and
    dL/deps within 1e-3 (the real-space sums difference float32 states)."""
    from evoxels_gb300 import _lib
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    bc = BCS[b]
    n, eps, D = 3, 1.5, 1.1
    u0 = oracle.seeded_ch_field(shape, 40 + b) + 0.6 * (oracle.seeded_unit_field(shape, 41 + b) - 0.5)
    lam = oracle.seeded_unit_field(shape, 42 + b) - 0.5
    with pytest.warns(UserWarning) if b else _nowarn():
        r = CahnHilliardAdjoint(vg_for(shape), dt=0.1, bc=bc)
    assert r.mirrored
    traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
    traj[0] = gpu(u0)[0]
    r.forward(traj[0:1], n, D, eps, traj=traj[1:])
    got = r.adjoint(traj, n, gpu(lam), D, eps, None).cpu().numpy()[0]
    ref, rD, re = _fp64_mirror_vjp(u0, lam, n, eps, D, bc)
    assert oracle.rel_to_max(got, ref) < 1e-4, oracle.rel_to_max(got, ref)
    grads = torch.zeros(3, dtype=torch.float64, device=DEV)
    got2 = r.adjoint(traj, n, gpu(lam), D, eps, grads).cpu().numpy()[0]
    # g comes from the g-and-h multiply on this path: the same dL/du up to rounding
    assert oracle.rel_to_max(got2, got) < 1e-6
    gD, ge = r.param_grads(grads, eps)
    assert abs(gD - rD) <= 1e-3 * abs(rD), (gD, rD)
    assert abs(ge - re) <= 1e-3 * abs(re), (ge, re)


class _nowarn:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        return False
