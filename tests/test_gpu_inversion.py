"""Differentiated inversion: autograd Function with checkpointing, gradients
against central finite differences of the FP64 oracle (bar: 1e-3 relative),
and a parameter fit in the configuration of the inversion workload (pinned
bulk, gradient coefficient free)."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

PIN = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)  # noqa: E731


def runner_for(shape, pinned=None, spectral=True):
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    vg = VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device="cuda")
    return CahnHilliardAdjoint(vg, dt=0.1, pinned_w=pinned, spectral=spectral)


def test_autograd_function_checkpointed_equals_stored(cuda_lib):
    from evoxels_gb300.adjoint import ch_imex_trajectory
    shape = (24, 20, 28)
    r = runner_for(shape)
    c0 = torch.tensor(oracle.seeded_ch_field(shape, 3), dtype=torch.float32, device="cuda").unsqueeze(0)
    tgt = torch.tensor(oracle.seeded_ch_field(shape, 4), dtype=torch.float32, device="cuda").unsqueeze(0)
    out = {}
    for K in (None, 5, 7):
        x = c0.clone().requires_grad_(True)
        D = torch.tensor(1.2, requires_grad=True)
        e = torch.tensor(1.5, requires_grad=True)
        u = ch_imex_trajectory(x, D, e, 20, r, checkpoint_every=K)
        loss = torch.mean((u - tgt) ** 2)
        loss.backward()
        out[K] = (float(loss.detach()), x.grad.clone(), float(D.grad), float(e.grad))
    for K in (5, 7):
        assert out[K][0] == pytest.approx(out[None][0], rel=1e-6)
        torch.testing.assert_close(out[K][1], out[None][1], rtol=0, atol=0)   # recompute is bit-identical
        assert out[K][2] == pytest.approx(out[None][2], rel=1e-12)
        assert out[K][3] == pytest.approx(out[None][3], rel=1e-12)


@pytest.mark.parametrize("pinned,spectral", [(None, True), (6.0, True), (None, False)])
def test_parameter_gradients_vs_central_differences(cuda_lib, pinned, spectral):
    shape = (16, 16, 16)
    n, D, eps, h = 10, 1.1, 1.4, 1e-3
    r = runner_for(shape, pinned, spectral)
    c0n = oracle.seeded_ch_field(shape, 5)
    tgn = oracle.seeded_ch_field(shape, 6)
    c0 = torch.tensor(c0n, dtype=torch.float32, device="cuda").unsqueeze(0)
    tg = torch.tensor(tgn, dtype=torch.float32, device="cuda").unsqueeze(0)
    loss, g0, gD, ge = r.loss_and_grads(c0, tg, n, D, eps, checkpoint_every=4)
    mu = None if pinned is None else PIN
    c064 = torch.tensor(c0n).unsqueeze(0)
    tg64 = torch.tensor(tgn).unsqueeze(0)

    def L(d, e):
        u = oracle.ch_imex_run(c064, n, 0.1, e, d, mu_hom=mu)
        return float(torch.mean((u - tg64) ** 2))
    fD = (L(D + h, eps) - L(D - h, eps)) / (2 * h)
    fe = (L(D, eps + h) - L(D, eps - h)) / (2 * h)
    assert abs(gD - fD) <= 1e-3 * abs(fD), (gD, fD)
    assert abs(ge - fe) <= 1e-3 * abs(fe), (ge, fe)
    # dL/dc0 against autograd through the FP64 oracle
    _, ref0, _, _ = oracle.ch_imex_loss_grads(c064, tg64, n, 0.1, eps, D, mu_hom=mu)
    assert oracle.rel_to_max(g0.cpu().numpy(), ref0.numpy()) < 1e-4


def test_parameter_fit_moves_toward_the_truth(cuda_lib):
    """Inversion workload in miniature: target from M=1, kappa=2 (eps=1), bulk pinned;
    fit from M=0.7, kappa=1.5 using the adjoint's gradients."""
    from evoxels_gb300.adjoint import fit_parameters
    shape = (32, 32, 32)
    r = runner_for(shape, pinned=6.0)
    c0 = torch.tensor(oracle.seeded_ch_field(shape, 3), dtype=torch.float32, device="cuda").unsqueeze(0)
    target = r.forward(c0, 40, 1.0, 1.0)
    D, e, hist = fit_parameters(r, c0, target, 40, 0.7, 0.75, iters=25, lr=0.05, checkpoint_every=10)
    assert hist[-1][0] < 0.1 * hist[0][0]
    assert abs(D - 1.0) < abs(0.7 - 1.0) and abs(e - 1.0) < abs(0.75 - 1.0)
