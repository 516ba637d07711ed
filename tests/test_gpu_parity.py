"""GPU parity of the CUDA path against the oracle and the reference's golden outputs.

Bars (stated per test):
* stencil right-hand sides and forward-Euler steps: bit-exact (same IEEE float32
  operations in the reference's order);
* one IMEX step: max|d|/max|ref| <= 1e-5 against the FP64 oracle; 1000 steps <= 1e-4;
* adjoint: against torch autograd through the FP64 oracle, relative 1e-4 for
  dL/dc0 and 1e-3 for parameter gradients; against central differences 1e-3.
"""

import warnings

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc

pytestmark = pytest.mark.gpu

DEV = "cuda"


def vg_for(shape, spacing=(1.0, 1.0, 1.0)):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    vf = VoxelFields(shape, domain_size=tuple(n * h for n, h in zip(shape, spacing)))
    return VoxelGridGB300(vf.grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).unsqueeze(0)


def cpu32(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32).unsqueeze(0)


def cpu64(a):
    return torch.tensor(np.asarray(a), dtype=torch.float64).unsqueeze(0)


# ---------------------------------------------------------------------------
# stencils: bit-exact
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("i", range(5))
def test_ch_rhs_bitexact_vs_reference_golden(cuda_lib, i):
    from evoxels_gb300.problem_definition import CahnHilliard
    g = load_golden(f"ch_rhs_{i}")
    shape = tuple(int(x) for x in g["shape"])
    spacing = tuple(float(x) for x in g["spacing"])
    bc = parse_bc(g["bc"])
    vg = vg_for(shape, spacing)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = CahnHilliard(vg, eps=3.0, D=1.0, **({"bc": bc} if bc is not None else {}))
    r = prob.rhs(0.0, gpu(g["u0"])).cpu().numpy()
    np.testing.assert_array_equal(r, g["rhs"])


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 1, 2), (33, 17, 9), (40, 36, 70), (64, 64, 64)])
@pytest.mark.parametrize("bc", [None, (("dirichlet", (0.1, 0.9)), "neumann", "periodic"),
                                ("neumann", "neumann", ("dirichlet", (0.0, 1.0)))])
def test_ch_rhs_bitexact_vs_oracle(cuda_lib, shape, bc):
    from evoxels_gb300.problem_definition import CahnHilliard
    u0 = oracle.seeded_ch_field(shape, 7) + 0.6 * (oracle.seeded_unit_field(shape, 8) - 0.5)
    vg = vg_for(shape)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = CahnHilliard(vg, eps=2.5, D=1.3, **({"bc": bc} if bc else {}))
    r = prob.rhs(0.0, gpu(u0)).cpu().numpy()
    ref = oracle.ch_rhs(cpu32(u0), 2.5, 1.3, bc).numpy()
    np.testing.assert_array_equal(r, ref)


@pytest.mark.parametrize("i", range(5))
@pytest.mark.parametrize("spp", [1, 2, 4])
def test_fd_forward_euler_bitexact_vs_reference_golden(cuda_lib, i, spp):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    g = load_golden(f"fd_fe_{i}")
    shape = tuple(int(x) for x in g["shape"])
    bc = parse_bc(g["bc"])
    vg = vg_for(shape)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = ReactionDiffusion(vg, D=1.0, **({"bc": bc} if bc is not None else {}))
    st = ForwardEuler(prob, float(g["dt"]), steps_per_pass=spp)
    u = st.advance(gpu(g["u0"]), int(g["n"])).cpu().numpy()
    np.testing.assert_array_equal(u, g["u"])


@pytest.mark.parametrize("shape", [(2, 3, 5), (17, 9, 33), (48, 40, 64), (70, 33, 35), (5, 3, 4), (33, 17, 68),
                                   (20, 40, 132), (9, 1, 8)])
@pytest.mark.parametrize("bc", [None, (("dirichlet", (0.0, 0.0)), "neumann", "neumann"),
                                ("neumann", ("dirichlet", (1.0, -2.0)), "periodic"),
                                ("periodic", "periodic", ("dirichlet", (0.5, 0.25)))])
def test_fd_steps_bitexact_all_blockings(cuda_lib, shape, bc):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    u0 = oracle.seeded_unit_field(shape, 5)
    dt = 1.0 / 60
    ref = oracle.rd_fe_run(cpu32(u0), 9, dt, 1.0, bc).numpy()
    vg = vg_for(shape)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = ReactionDiffusion(vg, D=1.0, **({"bc": bc} if bc else {}))
    for spp in (1, 2, 4):
        u = ForwardEuler(prob, dt, steps_per_pass=spp).advance(gpu(u0), 9).cpu().numpy()
        np.testing.assert_array_equal(u, ref, err_msg=f"steps_per_pass={spp}")
    r = prob.rhs(0.0, gpu(u0)).cpu().numpy()
    np.testing.assert_array_equal(r, oracle.rd_rhs(cpu32(u0), 1.0, bc).numpy())


# ---------------------------------------------------------------------------
# spectral step: tolerance against the FP64 oracle
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("i", range(4))
def test_ch_imex_vs_reference_golden(cuda_lib, i):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    g = load_golden(f"ch_imex_{i}")
    shape = tuple(int(x) for x in g["shape"])
    prob = CahnHilliard(vg_for(shape), eps=float(g["eps"]), D=float(g["D"]))
    st = PseudoSpectralIMEX(prob, float(g["dt"]))
    u = gpu(g["u0"])
    for _ in range(int(g["n"])):
        u = st.step(0.0, u)
    # reference fp32 (pocketfft) vs ours (cuFFT): agreement to float32 FFT rounding
    assert oracle.rel_to_max(u.cpu().numpy(), g["u"]) < 2e-6


@pytest.mark.parametrize("shape", [(16, 16, 16), (5, 7, 9), (24, 20, 18), (100, 100, 100)])
def test_ch_one_step_error_vs_fp64_oracle(cuda_lib, shape):
    """Per-step error bar: <= 1e-5 relative (to max) against the FP64 oracle."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    u0 = oracle.seeded_ch_field(shape, 1)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    u = st.step(0.0, gpu(u0)).cpu().numpy()
    ref = oracle.ch_imex_run(cpu64(u0), 1, 0.1).numpy()
    err = oracle.rel_to_max(u, ref)
    assert err <= 1e-5, err


def test_ch_forward_fused_equals_stepwise(cuda_lib):
    """The fused multi-step pass performs the same float operations as single steps."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    shape = (24, 20, 36)
    u0 = gpu(oracle.seeded_ch_field(shape, 3))
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape), eps=2.0, D=0.8), 0.1)
    u = u0
    for _ in range(7):
        u = st.step(0.0, u)
    traj = torch.empty((7,) + shape, dtype=torch.float32, device=DEV)
    v = st.advance(u0, 7, traj=traj)
    torch.testing.assert_close(v, u, rtol=0, atol=0)
    torch.testing.assert_close(traj[-1:], u, rtol=0, atol=0)
    w = u0
    for s in range(7):
        w = st.step(0.0, w)
        torch.testing.assert_close(traj[s:s + 1], w, rtol=0, atol=0)


def test_ch_1000_steps_vs_fp64_oracle(cuda_lib):
    """Long-run error bar: <= 1e-4 relative (to max) after 1000 steps (32^3 keeps the FP64 run short)."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    shape = (32, 32, 32)
    u0 = oracle.seeded_ch_field(shape, 1)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    u = st.advance(gpu(u0), 1000).cpu().numpy()
    ref = oracle.ch_imex_run(cpu64(u0), 1000, 0.1).numpy()
    err = oracle.rel_to_max(u, ref)
    assert err <= 1e-4, err


def test_driver_matches_reference_golden(cuda_lib):
    import evoxels_gb300 as evo
    g = load_golden("driver_ch")
    vf = evo.VoxelFields((16, 16, 16), domain_size=(16, 16, 16))
    vf.add_field("c", g["u0"].copy())
    evo.run_cahn_hilliard_solver(vf, "c", "torch", jit=False, time_increment=0.1, frames=2,
                                 max_iters=int(g["n"]), verbose=False)
    assert oracle.rel_to_max(vf.fields["c"], g["c"]) < 2e-6


def test_nonfinite_flag(cuda_lib):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    shape = (8, 8, 8)
    u0 = oracle.seeded_ch_field(shape, 2)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    flag = torch.zeros(1, dtype=torch.int32, device=DEV)
    st.advance(gpu(u0), 3, nonfinite=flag)
    assert int(flag) == 0
    u0[1, 2, 3] = np.nan
    st.advance(gpu(u0), 3, nonfinite=flag)
    assert int(flag) == 1


def test_solver_nan_abort_exits(cuda_lib, capsys):
    import evoxels_gb300 as evo
    vf = evo.VoxelFields((8, 8, 8), domain_size=(8, 8, 8))
    u0 = oracle.seeded_ch_field((8, 8, 8), 2)
    u0[0, 0, 0] = np.nan
    vf.add_field("c", u0)
    with pytest.raises(SystemExit) as e:
        evo.run_cahn_hilliard_solver(vf, "c", "torch", frames=2, max_iters=4, verbose=False)
    assert e.value.code == 1
    assert "NaN detected in frame 0" in capsys.readouterr().out


def test_errors_match_reference(cuda_lib):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    vg = vg_for((4, 4, 4))
    with pytest.raises(ValueError, match="support at most one non-periodic axis"):
        PseudoSpectralIMEX(CahnHilliard(vg, bc=("neumann", "neumann", "periodic")), 0.1)
    with pytest.raises(NotImplementedError, match="Axis permutation"):
        PseudoSpectralIMEX(CahnHilliard(vg, bc=("periodic", "neumann", "periodic")), 0.1)
    with pytest.raises(ValueError):
        CahnHilliard(vg).rhs(0.0, torch.zeros((1, 4, 4, 5), device=DEV))
    with pytest.raises(NotImplementedError):
        CahnHilliard(vg, mu_hom=lambda c: c ** 2)
    # a pinned double-well mu_hom is accepted (the inversion/batched configuration)
    CahnHilliard(vg, eps=1.0, mu_hom=lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c))


# ---------------------------------------------------------------------------
# adjoint
# ---------------------------------------------------------------------------

def _plan_with_grads(vg):
    from evoxels_gb300.timesteppers import get_plan
    return get_plan(vg, grads=True)


def _adjoint(vg, prob, dt, states, lam, grads=False):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    plan = _plan_with_grads(vg)
    n = states.shape[0] - 1
    out = torch.empty_like(lam)
    gbuf = torch.zeros(3, dtype=torch.float64, device=DEV) if grads else None
    _lib.check(_lib.lib().evx_ch_adjoint(plan.handle, states.data_ptr(), n, lam.data_ptr(), out.data_ptr(),
                                         prob.evx_params(dt), gbuf.data_ptr() if grads else None,
                                         plan.workspace.data_ptr(), cuda_stream()), "evx_ch_adjoint")
    return out, gbuf


@pytest.mark.parametrize("shape", [(8, 8, 8), (6, 10, 12), (33, 20, 17)])
def test_ch_adjoint_one_step_vs_autograd(cuda_lib, shape):
    from evoxels_gb300.problem_definition import CahnHilliard
    u0 = oracle.seeded_ch_field(shape, 11) + 0.7 * (oracle.seeded_unit_field(shape, 12) - 0.5)
    lam = oracle.seeded_unit_field(shape, 13) - 0.5
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=2.0, D=1.2)
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    st = PseudoSpectralIMEX(prob, 0.1)
    ug = gpu(u0)
    states = torch.cat([ug, st.step(0.0, ug)], 0).contiguous()
    out, gr = _adjoint(vg, prob, 0.1, states, gpu(lam), grads=True)
    ref, dD, de = oracle.ch_imex_vjp(cpu64(u0), cpu64(lam), 0.1, 2.0, 1.2)
    assert oracle.rel_to_max(out.cpu().numpy(), ref.numpy()) < 1e-4
    gD, gK, gW = gr.cpu().tolist()
    # eps enters as kappa = 2*eps and the default bulk w = 18/eps
    ge = 2 * gK - 18 / 2.0 ** 2 * gW
    assert abs(gD - dD) <= 1e-3 * abs(dD)
    assert abs(ge - de) <= 1e-3 * abs(de)


def test_ch_adjoint_multi_step_vs_reference_autograd_golden(cuda_lib):
    """dL/dc0, dL/dD, dL/deps through 5 steps vs torch autograd through the reference."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    g = load_golden("ch_grad")
    shape = g["u0"].shape
    n, D, eps, dt = int(g["n"]), float(g["D"]), float(g["eps"]), float(g["dt"])
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=eps, D=D)
    st = PseudoSpectralIMEX(prob, dt)
    traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
    traj[0] = gpu(g["u0"])[0]
    st.advance(traj[0:1], n, traj=traj[1:])
    lam = 2 * (traj[n:n + 1] - gpu(g["target"])) / float(np.prod(shape))
    out, gr = _adjoint(vg, prob, dt, traj, lam.contiguous(), grads=True)
    assert oracle.rel_to_max(out.cpu().numpy()[0], g["g_c0"]) < 1e-4
    gD, gK, gW = gr.cpu().tolist()
    ge = 2 * gK - 18 / eps ** 2 * gW
    assert abs(gD - float(g["g_D"])) <= 1e-3 * abs(float(g["g_D"]))
    assert abs(ge - float(g["g_eps"])) <= 1e-3 * abs(float(g["g_eps"]))


def test_fd_adjoint_vs_autograd(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.voxelgrid import cuda_stream
    shape = (12, 9, 14)
    bc = (("dirichlet", (0.3, 0.0)), "neumann", "periodic")
    u0 = oracle.seeded_unit_field(shape, 3)
    lam = oracle.seeded_unit_field(shape, 4) - 0.5
    x = cpu64(u0).requires_grad_(True)
    y = oracle.rd_fe_run(x, 6, 1 / 60, 1.0, bc)
    (ref,) = torch.autograd.grad(y, x, grad_outputs=cpu64(lam))
    vg = vg_for(shape)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = ReactionDiffusion(vg, D=1.0, bc=bc)
    lg = gpu(lam)
    out = torch.empty_like(lg)
    scratch = torch.empty_like(lg)
    _lib.check(_lib.lib().evx_fd_adjoint(lg.data_ptr(), out.data_ptr(), scratch.data_ptr(), vg.evx_grid(),
                                         prob._evx_bc, 1.0, float(np.float32(1 / 60)), 6, cuda_stream()))
    assert oracle.rel_to_max(out.cpu().numpy(), ref.numpy()) < 1e-5


# ---------------------------------------------------------------------------
# fast periodic kernels vs the generic kernels (a misaligned view forces the
# generic path: the fast path needs 16-byte aligned fields and nz % 4 == 0)
# ---------------------------------------------------------------------------

def _misaligned_copy(t):
    flat = torch.empty(t.numel() + 1, dtype=t.dtype, device=t.device)
    v = flat[1:].view(t.shape)
    v.copy_(t)
    assert v.data_ptr() % 16 != 0
    return v


@pytest.mark.parametrize("shape", [(10, 20, 100), (7, 33, 68), (12, 17, 4), (3, 5, 8), (40, 18, 136),
                                   (9, 16, 64), (1, 1, 4)])
def test_ch_rhs_fast_equals_generic_and_oracle(cuda_lib, shape):
    from evoxels_gb300.problem_definition import CahnHilliard
    u0 = oracle.seeded_ch_field(shape, 21) + 0.6 * (oracle.seeded_unit_field(shape, 22) - 0.5)
    prob = CahnHilliard(vg_for(shape), eps=2.0, D=0.9)
    ug = gpu(u0)
    fast = prob.rhs(0.0, ug)
    slow = prob.rhs(0.0, _misaligned_copy(ug))
    torch.testing.assert_close(fast, slow, rtol=0, atol=0)
    np.testing.assert_array_equal(fast.cpu().numpy(), oracle.ch_rhs(cpu32(u0), 2.0, 0.9).numpy())


@pytest.mark.parametrize("spacing", [(0.5, 0.75, 1.25), (0.3, 1.7, 0.9)])
def test_ch_rhs_fast_bitexact_non_unit_spacing(cuda_lib, spacing):
    """The two-lane fast path with spacing factors that are not 1 (no product is exact)."""
    from evoxels_gb300.problem_definition import CahnHilliard
    shape = (12, 20, 64)
    u0 = oracle.seeded_ch_field(shape, 23) + 0.6 * (oracle.seeded_unit_field(shape, 24) - 0.5)
    prob = CahnHilliard(vg_for(shape, spacing), eps=2.3, D=0.7)
    ug = gpu(u0)
    fast = prob.rhs(0.0, ug)
    slow = prob.rhs(0.0, _misaligned_copy(ug))
    torch.testing.assert_close(fast, slow, rtol=0, atol=0)
    np.testing.assert_array_equal(fast.cpu().numpy(), oracle.ch_rhs(cpu32(u0), 2.3, 0.7, None, spacing).numpy())


@pytest.mark.parametrize("shape", [(10, 20, 100), (12, 17, 4), (36, 40, 72)])
def test_ch_forward_fast_matches_fp64(cuda_lib, shape):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    u0 = oracle.seeded_ch_field(shape, 4)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    traj = torch.empty((6,) + shape, dtype=torch.float32, device=DEV)
    st.advance(gpu(u0), 6, traj=traj)
    keep = []
    oracle.ch_imex_run(cpu64(u0), 6, 0.1, keep=keep)
    for s in range(6):
        assert oracle.rel_to_max(traj[s].cpu().numpy(), keep[s + 1].numpy()[0]) <= 1e-5 * (s + 1)


@pytest.mark.parametrize("shape", [(10, 20, 100), (12, 17, 4), (16, 16, 16), (9, 33, 68)])
@pytest.mark.parametrize("grads", [False, True])
def test_ch_adjoint_fast_equals_generic(cuda_lib, shape, grads):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    u0 = oracle.seeded_ch_field(shape, 31) + 0.5 * (oracle.seeded_unit_field(shape, 32) - 0.5)
    lam = oracle.seeded_unit_field(shape, 33) - 0.5
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.5, D=1.1)
    st = PseudoSpectralIMEX(prob, 0.1)
    n = 3
    traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
    traj[0] = gpu(u0)[0]
    st.advance(traj[0:1], n, traj=traj[1:])
    a, ga = _adjoint(vg, prob, 0.1, traj, gpu(lam), grads=grads)
    b, gb = _adjoint(vg, prob, 0.1, _misaligned_copy(traj), gpu(lam), grads=grads)
    assert oracle.rel_to_max(a.cpu().numpy(), b.cpu().numpy()) < 1e-5
    if grads:
        # the real-space gradient sums difference float32 states (u' - u): the two kernels group
        # their partial sums differently, so they agree to the cancellation floor, not to the last bit
        for x, y in zip(ga.cpu().tolist(), gb.cpu().tolist()):
            assert abs(x - y) <= 1e-4 * max(abs(y), 1e-12)
    # and against torch autograd through the FP64 oracle
    v = lam
    ref = cpu64(lam)
    keep = []
    oracle.ch_imex_run(cpu64(u0), n, 0.1, 1.5, 1.1, keep=keep)
    for s in range(n - 1, -1, -1):
        ref, _, _ = oracle.ch_imex_vjp(keep[s], ref, 0.1, 1.5, 1.1)
    del v
    assert oracle.rel_to_max(a.cpu().numpy(), ref.numpy()) < 1e-4


# ---------------------------------------------------------------------------
# fused spectral x-pass (power-of-two Nx) vs cuFFT's 3-D transforms
# ---------------------------------------------------------------------------

def _forward_with(vg, prob, u0, n, cufft3d):
    from evoxels_gb300 import _lib
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    plan = get_plan(vg, grads=True, cufft3d=cufft3d)
    traj = torch.empty((n + 1,) + tuple(vg.shape), dtype=torch.float32, device=DEV)
    traj[0] = u0[0]
    out = torch.empty_like(u0)
    _lib.check(_lib.lib().evx_ch_forward(plan.handle, traj[0:1].data_ptr(), out.data_ptr(), n, traj[1:].data_ptr(),
                                         prob.evx_params(0.1), None, plan.workspace.data_ptr(), cuda_stream()))
    lam = torch.tensor(oracle.seeded_unit_field(vg.shape, 77) - 0.5, dtype=torch.float32, device=DEV).unsqueeze(0)
    lo = torch.empty_like(lam)
    gr = torch.zeros(3, dtype=torch.float64, device=DEV)
    _lib.check(_lib.lib().evx_ch_adjoint(plan.handle, traj.data_ptr(), n, lam.data_ptr(), lo.data_ptr(),
                                         prob.evx_params(0.1), gr.data_ptr(), plan.workspace.data_ptr(), cuda_stream()))
    return out, lo, gr


# ny*(nz/2+1) >= 256 and even takes the pipelined (TMA) kernel, else the per-tile one;
# the TMA shapes cover every (N1, N2) split and partial last tiles
@pytest.mark.parametrize("shape", [(8, 12, 20), (16, 16, 16), (32, 20, 36), (64, 12, 24), (128, 8, 12),
                                   (256, 6, 8), (512, 4, 8), (256, 64, 64),
                                   (8, 32, 30), (16, 24, 40), (64, 18, 30), (128, 16, 34), (256, 10, 50),
                                   (512, 16, 32)])
def test_xpass_matches_cufft3d_and_fp64(cuda_lib, shape):
    from evoxels_gb300.problem_definition import CahnHilliard
    u0n = oracle.seeded_ch_field(shape, 8)
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.7, D=1.3)
    u0 = gpu(u0n)
    a, la, ga = _forward_with(vg, prob, u0, 3, cufft3d=False)
    b, lb, gb = _forward_with(vg, prob, u0, 3, cufft3d=True)
    assert oracle.rel_to_max(a.cpu().numpy(), b.cpu().numpy()) < 1e-6
    assert oracle.rel_to_max(la.cpu().numpy(), lb.cpu().numpy()) < 1e-5
    # the real-space gradient sums difference u_{s+1} - u_s of float32 states, so two
    # FFT implementations that agree to 1e-6 in u give sums that agree to ~1e-4:
    # compared at the bar the gradients meet against FP64 central differences
    for x, y in zip(ga.cpu().tolist(), gb.cpu().tolist()):
        assert abs(x - y) <= 1e-3 * max(abs(y), 1e-9)
    ref = oracle.ch_imex_run(cpu64(u0n), 3, 0.1, 1.7, 1.3).numpy()
    assert oracle.rel_to_max(a.cpu().numpy(), ref) <= 3e-5
    assert cuda_lib.evx_device_status(1) == 0


@pytest.mark.parametrize("bc", [None, ("neumann", "periodic", "periodic")])
def test_multichannel_imex_vs_fp64_4d_transform(cuda_lib, bc):
    """Three fields stepped together: the reference transforms the whole (C, Nx, Ny, Nz) field; its
    multiplier does not depend on the channel frequency, so the steps equal per-channel steps.  Against
    the FP64 oracle's 4-D transform from the same float64 fields: <= 1e-5 per step."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    shape = (16, 12, 10)
    kw = {} if bc is None else {"bc": bc}
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape), eps=2.0, D=0.9, **kw), 0.1)
    u0 = oracle.seeded_ch_field((3,) + shape, 77)
    ug = torch.tensor(u0, dtype=torch.float32, device=DEV)
    one = st.step(0.0, ug).cpu().numpy()
    four = st.advance(ug, 4).cpu().numpy()
    ref1 = oracle.ch_imex_run(torch.tensor(u0), 1, 0.1, 2.0, 0.9, bc=bc).numpy()
    ref4 = oracle.ch_imex_run(torch.tensor(u0), 4, 0.1, 2.0, 0.9, bc=bc).numpy()
    assert oracle.rel_to_max(one, ref1) <= 1e-5
    assert oracle.rel_to_max(four, ref4) <= 4e-5
    with pytest.raises(NotImplementedError, match="one channel"):
        st.advance(ug, 2, traj=torch.empty((2,) + shape, device=DEV))
