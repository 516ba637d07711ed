"""Exponential Euler (ETD1) on the GPU: the phi1 multiplier table and steps
against the reference's own fp32 runs (golden fixtures), the x-pass and cuFFT
3-D paths against each other and the FP64 oracle for every x BC kind, the
reference's BC rejection, and the solver driver."""

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
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


@pytest.mark.parametrize("i", range(5))
def test_etd1_vs_reference_golden(cuda_lib, i):
    from evoxels_gb300 import problem_definition as PD
    from evoxels_gb300.timesteppers import ExponentialEuler
    g = load_golden(f"etd1_{i}")
    shape = tuple(int(x) for x in g["shape"])
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    if bc is not None:
        kw["bc"] = bc
    st = ExponentialEuler(getattr(PD, str(g["problem"]))(vg_for(shape), **kw), float(g["dt"]))
    assert st.order == 1
    # the table is built by torch on the device: exp rounds within an ulp or two of the CPU's
    phi = st.phi_1_k_squared.cpu().numpy()
    assert phi.shape == g["phi1"].shape
    np.testing.assert_allclose(phi, g["phi1"], rtol=1e-6, atol=0)
    v = gpu(g["u0"])
    for _ in range(3):
        v = st.step(0.0, v)
    # reference fp32 (pocketfft) vs ours (cuFFT / x-pass): float32 FFT rounding
    assert oracle.rel_to_max(v.cpu().numpy(), g["u3"]) < 2e-6


BCS = [("periodic", "periodic", "periodic"), ("neumann", "periodic", "periodic"),
       (("dirichlet", (0.3, 0.8)), "periodic", "periodic")]


# power-of-two nx up to 256 take the x-pass (table multiply, mirror extension inside); others cuFFT 3-D
@pytest.mark.parametrize("shape", [(32, 20, 36), (24, 16, 20), (64, 64, 64), (256, 8, 8), (8, 12, 15)])
@pytest.mark.parametrize("b", range(3))
@pytest.mark.parametrize("pname", ["CahnHilliard", "ReactionDiffusion"])
def test_etd1_paths_agree_and_match_fp64(cuda_lib, shape, b, pname):
    from evoxels_gb300 import _lib
    from evoxels_gb300 import problem_definition as PD
    from evoxels_gb300.timesteppers import ExponentialEuler, get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    vg = vg_for(shape)
    dt = 0.1 if pname == "CahnHilliard" else 0.6
    kw = dict(eps=1.7, D=1.3) if pname == "CahnHilliard" else dict(D=1.1)
    prob = getattr(PD, pname)(vg, bc=BCS[b], **kw)
    st = ExponentialEuler(prob, dt)
    u0n = oracle.seeded_ch_field(shape, 90 + b) if pname == "CahnHilliard" else oracle.seeded_unit_field(shape, 90)
    u0 = gpu(u0n)
    r = prob.rhs(0.0, u0)
    outs = []
    for cufft3d in (False, True):
        plan = get_plan(vg, cufft3d=cufft3d, bc=prob.bc)
        out = torch.empty_like(u0)
        _lib.check(cuda_lib.evx_spectral_update(plan.handle, u0.data_ptr(), r.data_ptr(), st._mult.data_ptr(),
                                                out.data_ptr(), plan.workspace.data_ptr(), cuda_stream()),
                   "evx_spectral_update")
        outs.append(out.cpu().numpy())
    if pname == "CahnHilliard":
        # the Cahn-Hilliard step runs the spectral loop's own rhs pass (fused products), so it differs
        # from the update of the bit-exact rhs by the rhs's rounding only
        assert oracle.rel_to_max(st.step(0.0, u0).cpu().numpy(), outs[0]) < 1e-6
    else:
        torch.testing.assert_close(torch.tensor(outs[0]), st.step(0.0, u0).cpu(), rtol=0, atol=0)
    assert oracle.rel_to_max(outs[0], outs[1]) < 1e-6
    # FP64 oracle: three steps
    mirrored = oracle.x_bc_kind(prob.bc) != "periodic"
    k2 = (oracle.rfft_k_squared_nonperiodic if mirrored else oracle.rfft_k_squared)(shape, dtype=torch.float64)
    if pname == "CahnHilliard":
        sym = -2 * 1.7 * 1.3 * 0.25 * k2 ** 2
        fn = lambda w: oracle.ch_rhs(w, eps=1.7, D=1.3, bc=prob.bc)  # noqa: E731
    else:
        sym = -1.1 * 0.25 * k2
        fn = lambda w: oracle.rd_rhs(w, D=1.1, bc=prob.bc)  # noqa: E731
    m = oracle.etd1_multiplier(sym, dt)
    ref = torch.tensor(u0n).unsqueeze(0)
    v = u0
    for _ in range(3):
        ref = oracle.imex_step(ref, m, fn, prob.bc)
        v = st.step(0.0, v)
    assert oracle.rel_to_max(v.cpu().numpy(), ref.numpy()) < 1e-5


def test_etd1_allen_cahn_driver_and_errors(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard, TwoPhaseAllenCahn
    from evoxels_gb300.solvers import TimeDependentSolver
    from evoxels_gb300.timesteppers import ExponentialEuler, get_plan
    from evoxels_gb300.voxelfields import VoxelFields
    # the reference's own check: Allen-Cahn's default BCs (Neumann on every axis)
    with pytest.raises(ValueError, match="support at most one non-periodic axis"):
        ExponentialEuler(TwoPhaseAllenCahn(vg_for((4, 4, 4))), 0.1)
    shape = (32, 12, 10)
    vf = VoxelFields(shape, domain_size=shape)
    u0 = oracle.seeded_unit_field(shape, 95)
    vf.add_field("phi", u0.copy())
    bc = ("neumann", "periodic", "periodic")
    solver = TimeDependentSolver(vf, "phi", "torch", problem_cls=TwoPhaseAllenCahn, timestepper_cls=ExponentialEuler)
    solver.solve(time_increment=0.3, frames=2, max_iters=6, problem_kwargs={"eps": 2.0, "bc": bc}, jit=False,
                 verbose=False)
    k2 = oracle.rfft_k_squared_nonperiodic(shape, dtype=torch.float64)
    m = oracle.etd1_multiplier(-k2, 0.3)
    ref = torch.tensor(u0).unsqueeze(0)
    for _ in range(6):
        ref = oracle.imex_step(ref, m, lambda w: oracle.ac_rhs(w, eps=2.0, bc=bc), bc)
    assert oracle.rel_to_max(vf.fields["phi"], ref.numpy()[0]) < 3e-5
    # two channels: the reference's 4-D transform (channel axis included) against per-channel steps
    st = ExponentialEuler(CahnHilliard(vg_for((8, 8, 8))), 0.1)
    u2 = oracle.seeded_ch_field((2, 8, 8, 8), 96)
    got = st.step(0.0, torch.tensor(u2, dtype=torch.float32, device=DEV)).cpu().numpy()
    m8 = oracle.etd1_multiplier(-2 * 3.0 * 1.0 * 0.25 * oracle.rfft_k_squared((8, 8, 8), dtype=torch.float64) ** 2, 0.1)
    ref2 = oracle.imex_step(torch.tensor(u2), m8, lambda w: oracle.ch_rhs(w))
    assert oracle.rel_to_max(got, ref2.numpy()) < 1e-5
    plan = get_plan(st.problem.vg)
    x = torch.zeros((1, 8, 8, 8), device=DEV)
    with pytest.raises(_lib.EvxError, match="NULL"):
        _lib.check(cuda_lib.evx_spectral_update(plan.handle, x.data_ptr(), x.data_ptr(), None, x.data_ptr(),
                                                plan.workspace.data_ptr(), None), "evx_spectral_update")


@pytest.mark.parametrize("shape", [(32, 20, 36), (24, 16, 20), (64, 64, 64), (16, 8, 256), (8, 24, 256)])
@pytest.mark.parametrize("b", range(3))
def test_etd1_fused_advance_bitexact(cuda_lib, shape, b):
    """ExponentialEuler.advance for CahnHilliard (one evx_ch_forward_mult call, each update fused into the
    next rhs pass) equals the step-by-step path bit for bit on the x-pass, z-pass and cuFFT 3-D plans."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import ExponentialEuler
    st = ExponentialEuler(CahnHilliard(vg_for(shape), eps=1.7, D=1.3, bc=BCS[b]), 0.1)
    u0 = gpu(oracle.seeded_ch_field(shape, 70 + b))
    v = u0
    for _ in range(4):
        v = st.step(0.0, v)
    if shape[2] == 256:   # the z pass's plan: the table is kept in its [kx][kz][ky] order
        assert torch.equal(st._mult, (st.dt * st.phi_1_k_squared).float().transpose(1, 2).contiguous())
        # against the cuFFT (y, z) plan with the rfftn-ordered table
        from evoxels_gb300 import _lib
        from evoxels_gb300.timesteppers import get_plan, mult_table
        from evoxels_gb300.voxelgrid import cuda_stream
        plan = get_plan(st.problem.vg, bc=st.problem.bc, cufft_yz=True)
        m = mult_table(plan, st.dt * st.phi_1_k_squared)
        r = st.problem.rhs(0.0, u0)
        out = torch.empty_like(u0)
        _lib.check(cuda_lib.evx_spectral_update(plan.handle, u0.data_ptr(), r.data_ptr(), m.data_ptr(),
                                                out.data_ptr(), plan.workspace.data_ptr(), cuda_stream()), "etd1")
        assert oracle.rel_to_max(out.cpu().numpy(), st.step(0.0, u0).cpu().numpy()) < 1e-6
    nf = torch.zeros((1,), dtype=torch.int32, device=DEV)   # OR-ed into by the final update
    w = st.advance(u0, 4, nonfinite=nf)
    assert torch.equal(w, v)
    assert int(nf) == 0
    assert torch.equal(st.advance(u0, 1), st.step(0.0, u0))
    assert torch.equal(st.advance(u0, 0), u0)
    bad = u0.clone()
    bad[0, 1, 2, 3] = float("nan")
    st.advance(bad, 2, nonfinite=nf)
    assert int(nf) == 1
