"""Stored increment spectra and the spectral-gradient adjoint.

``evx_ch_forward_spectra`` keeps each step's multiplied spectrum; with it
``evx_ch_adjoint_spectra`` forms the mobility gradient sums by Parseval in the
x-pass.  Checked here: the forward result is unchanged by storing, dL/du_0 and
the parameter gradients agree with the real-space adjoint (itself checked
against torch autograd through the FP64 oracle and against the reference's
autograd golden), including odd nz (no Nyquist plane) and grids that take the
generic stencil kernels.
"""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden

pytestmark = pytest.mark.gpu
DEV = "cuda"


def vg_for(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def _gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


def _run(vg, prob, u0, lam, n, spectral, dt=0.1):
    """Forward n steps (trajectory kept) then the adjoint with parameter gradients."""
    from evoxels_gb300 import _lib
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    L = _lib.lib()
    plan = get_plan(vg, grads=True)
    nf = int(L.evx_ch_spectrum_floats(plan.handle))
    traj = torch.empty((n + 1,) + tuple(vg.shape), dtype=torch.float32, device=DEV)
    traj[0] = u0[0]
    out = torch.empty_like(u0)
    spec = torch.empty(max(n * nf, 1), dtype=torch.float32, device=DEV) if spectral else None
    p = prob.evx_params(dt)
    _lib.check(L.evx_ch_forward_spectra(plan.handle, traj[0:1].data_ptr(), out.data_ptr(), n, traj[1:].data_ptr(),
                                        spec.data_ptr() if spectral else None, p, None, plan.workspace.data_ptr(),
                                        cuda_stream()), "evx_ch_forward_spectra")
    lo = torch.empty_like(lam)
    gr = torch.zeros(3, dtype=torch.float64, device=DEV)
    _lib.check(L.evx_ch_adjoint_spectra(plan.handle, traj.data_ptr(), spec.data_ptr() if spectral else None, n,
                                        lam.data_ptr(), lo.data_ptr(), p, gr.data_ptr(), plan.workspace.data_ptr(),
                                        cuda_stream()), "evx_ch_adjoint_spectra")
    return out, lo, gr.cpu().tolist(), nf


@pytest.mark.parametrize("shape", [(8, 12, 20), (16, 10, 18), (32, 6, 15), (32, 20, 36), (64, 12, 24),
                                   (128, 8, 12), (256, 6, 8), (512, 4, 8), (64, 64, 64),
                                   (8, 32, 30), (128, 16, 34), (256, 10, 50), (512, 16, 32)])
def test_spectral_grads_equal_real_space_grads(cuda_lib, shape):
    from evoxels_gb300.problem_definition import CahnHilliard
    u0 = _gpu(oracle.seeded_ch_field(shape, 41) + 0.4 * (oracle.seeded_unit_field(shape, 42) - 0.5))
    lam = _gpu(oracle.seeded_unit_field(shape, 43) - 0.5)
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.6, D=1.2)
    a, la, ga, nf = _run(vg, prob, u0, lam, 4, spectral=True)
    b, lb, gb, _ = _run(vg, prob, u0, lam, 4, spectral=False)
    assert nf > 0
    torch.testing.assert_close(a, b, rtol=0, atol=0)          # storing the spectra changes nothing
    assert oracle.rel_to_max(la.cpu().numpy(), lb.cpu().numpy()) < 1e-6
    # the real-space sums difference float32 states (u_{s+1} - u_s loses digits to
    # rounding); the spectral sums use the exact increments: agreement to 1e-4,
    # accuracy against FP64 in the test below
    for x, y in zip(ga, gb):
        assert abs(x - y) <= 1e-4 * max(abs(y), 1e-9), (ga, gb)
    assert cuda_lib.evx_device_status(1) == 0


def test_spectral_grads_vs_reference_autograd_golden(cuda_lib):
    """dL/dc0, dL/dD, dL/deps through 5 steps vs torch autograd through the reference."""
    from evoxels_gb300.problem_definition import CahnHilliard
    g = load_golden("ch_grad")
    shape = g["u0"].shape
    n, D, eps, dt = int(g["n"]), float(g["D"]), float(g["eps"]), float(g["dt"])
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=eps, D=D)
    u0 = _gpu(g["u0"])
    # lam = dL/du_n of the MSE loss needs u_n: run the forward once without spectra
    out, _, _, _ = _run(vg, prob, u0, torch.zeros_like(u0), n, spectral=False, dt=dt)
    lam = (2 * (out - _gpu(g["target"])) / float(np.prod(shape))).contiguous()
    _, lo, gr, _ = _run(vg, prob, u0, lam, n, spectral=True, dt=dt)
    assert oracle.rel_to_max(lo.cpu().numpy()[0], g["g_c0"]) < 1e-4
    gD, gK, gW = gr
    ge = 2 * gK - 18 / eps ** 2 * gW
    assert abs(gD - float(g["g_D"])) <= 1e-3 * abs(float(g["g_D"]))
    assert abs(ge - float(g["g_eps"])) <= 1e-3 * abs(float(g["g_eps"]))


@pytest.mark.parametrize("shape", [(32, 20, 36), (64, 16, 15)])
def test_spectral_grads_vs_fp64_autograd(cuda_lib, shape):
    """MSE loss gradients through 6 steps (spectral adjoint) vs torch autograd in FP64."""
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    vg = vg_for(shape)
    r = CahnHilliardAdjoint(vg, dt=0.1)
    assert r.spec_floats > 0
    c0n = oracle.seeded_ch_field(shape, 51) + 0.3 * (oracle.seeded_unit_field(shape, 52) - 0.5)
    tgn = oracle.seeded_ch_field(shape, 53)
    loss, g0, gD, ge = r.loss_and_grads(_gpu(c0n), _gpu(tgn), 6, 1.2, 1.5)
    rl, rg0, rgD, rge = oracle.ch_imex_loss_grads(torch.tensor(c0n).unsqueeze(0), torch.tensor(tgn).unsqueeze(0),
                                                  6, 0.1, 1.5, 1.2)
    assert loss == pytest.approx(rl, rel=1e-5)
    assert oracle.rel_to_max(g0.cpu().numpy(), rg0.numpy()) < 1e-4
    assert gD == pytest.approx(rgD, rel=1e-4)
    assert ge == pytest.approx(rge, rel=1e-4)


def test_spectra_rejected_without_xpass_or_misaligned(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    L = _lib.lib()
    shape = (16, 8, 8)
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.6, D=1.2)
    p = prob.evx_params(0.1)
    u = _gpu(oracle.seeded_ch_field(shape, 1))
    out = torch.empty_like(u)
    plan3d = get_plan(vg, grads=True, cufft3d=True)
    assert int(L.evx_ch_spectrum_floats(plan3d.handle)) == 0
    spec = torch.empty(1 << 16, dtype=torch.float32, device=DEV)
    with pytest.raises(NotImplementedError):
        _lib.check(L.evx_ch_forward_spectra(plan3d.handle, u.data_ptr(), out.data_ptr(), 1, None, spec.data_ptr(), p,
                                            None, plan3d.workspace.data_ptr(), cuda_stream()), "fwd")
    plan = get_plan(vg, grads=True)
    assert int(L.evx_ch_spectrum_floats(plan.handle)) > 0
    with pytest.raises(_lib.EvxError, match="16-byte aligned"):
        _lib.check(L.evx_ch_forward_spectra(plan.handle, u.data_ptr(), out.data_ptr(), 1, None, spec[1:].data_ptr(),
                                            p, None, plan.workspace.data_ptr(), cuda_stream()), "fwd")
    states = torch.cat([u, u], 0).contiguous()
    gr = torch.zeros(3, dtype=torch.float64, device=DEV)
    with pytest.raises(NotImplementedError):
        _lib.check(L.evx_ch_adjoint_spectra(plan3d.handle, states.data_ptr(), spec.data_ptr(), 1, u.data_ptr(),
                                            out.data_ptr(), p, gr.data_ptr(), plan3d.workspace.data_ptr(),
                                            cuda_stream()), "adj")


def test_runner_checkpointed_equals_stored_with_spectra(cuda_lib):
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    shape = (32, 20, 28)
    vg = vg_for(shape)
    r = CahnHilliardAdjoint(vg, dt=0.1)
    rr = CahnHilliardAdjoint(vg, dt=0.1, spectral=False)
    assert r.spec_floats > 0 and rr.spec_floats == 0
    c0 = _gpu(oracle.seeded_ch_field(shape, 3))
    tg = _gpu(oracle.seeded_ch_field(shape, 4))
    res = {}
    for name, runner, K in (("stored", r, None), ("ckpt", r, 6), ("real", rr, None)):
        res[name] = runner.loss_and_grads(c0, tg, 15, 1.2, 1.5, checkpoint_every=K)
    torch.testing.assert_close(res["ckpt"][1], res["stored"][1], rtol=0, atol=0)
    assert res["ckpt"][2] == pytest.approx(res["stored"][2], rel=1e-12)
    assert res["ckpt"][3] == pytest.approx(res["stored"][3], rel=1e-12)
    assert oracle.rel_to_max(res["real"][1].cpu().numpy(), res["stored"][1].cpu().numpy()) < 1e-6
    assert res["real"][2] == pytest.approx(res["stored"][2], rel=1e-5)
    assert res["real"][3] == pytest.approx(res["stored"][3], rel=1e-5)
