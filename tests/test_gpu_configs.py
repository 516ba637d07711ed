"""The differentiated configurations at their full sizes.

* Inversion: Cahn-Hilliard 128^3, 200 steps of dt = 0.1, c0 = 0.5 + 0.1 U[0,1) (seed 3); the target
  comes from mobility M = 1.0 and gradient coefficient kappa = 2.0, the forward run from M = 0.7 and
  kappa = 1.5 (bulk term pinned to the eps = 3 default, w = 6); MSE of the final fields; checkpoint
  every 20 steps.  dL/dM and dL/dkappa against central differences with step 1e-3, dL/dc0 (along its
  own direction, unit maximum) against the Richardson combination of central differences with steps
  1e-3 and 5e-4: <= 1e-3 relative.
* Large grid: Cahn-Hilliard 512^3 from seed 5 with the reference defaults.  The first step against the
  FP64 oracle (<= 1e-5 relative to max); 900 forward steps, then the adjoint through the last 100 with
  checkpoint-and-recompute (K = 10) equal to the adjoint over the stored trajectory, and dL/dM against
  central differences (<= 1e-3).
"""

import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _vg(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def test_inversion_config_gradients_vs_central_differences(cuda_lib):
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    shape, n, h = (128, 128, 128), 200, 1e-3
    r = CahnHilliardAdjoint(_vg(shape), dt=0.1, pinned_w=6.0)
    c0 = torch.tensor(oracle.seeded_ch_field(shape, 3), dtype=torch.float32, device=DEV).unsqueeze(0)
    target = r.forward(c0, n, 1.0, 1.0)                 # kappa = 2*eps = 2.0
    M, eps = 0.7, 0.75                                  # kappa = 1.5
    loss, g0, gM, geps = r.loss_and_grads(c0, target, n, M, eps, checkpoint_every=20)
    gK = geps / 2.0                                     # dL/dkappa

    def L(m, e, c=c0):
        return float(r.mse(r.forward(c, n, m, e), target))
    assert loss == pytest.approx(L(M, eps), rel=1e-12)
    fM = (L(M + h, eps) - L(M - h, eps)) / (2 * h)
    fK = (L(M, eps + h / 2) - L(M, eps - h / 2)) / (2 * h)
    assert abs(gM - fM) <= 1e-3 * abs(fM), (gM, fM)
    assert abs(gK - fK) <= 1e-3 * abs(fK), (gK, fK)
    # dL/dc0 along its own direction scaled to a unit maximum (a step h moves every voxel by at most
    # h).  Along a smooth direction the loss moves by ~1e-4 of itself and the difference quotient is
    # at the float32 rounding floor of the forward run (~1e-3); along the gradient it moves by ~20%,
    # but there the spinodal growth makes the central difference's O(h^2) term ~2e-3 at h = 1e-3 (in
    # float64 with exact gradients at 48^3: 4.3e-2, 1.1e-2, 2.9e-3, 7.3e-4 at h = 4, 2, 1, 0.5 e-3).
    # Richardson's combination of the central differences with steps h and h/2 removes that term.
    v = g0 / g0.abs().max()
    gc = float((g0.double() * v.double()).sum())

    def fd_c(step):
        return (L(M, eps, c0 + step * v) - L(M, eps, c0 - step * v)) / (2 * step)
    fc = fd_c(h)
    fr = (4 * fd_c(h / 2) - fc) / 3
    assert abs(gc - fr) <= 1e-3 * abs(fr), (gc, fr, fc)


def test_large_grid_config_fp64_step_and_adjoint_of_last_100(cuda_lib):
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    torch.cuda.empty_cache()
    shape = (512, 512, 512)
    vg = _vg(shape)
    st = PseudoSpectralIMEX(CahnHilliard(vg), 0.1)
    c0n = oracle.seeded_ch_field(shape, 5)
    c0 = torch.tensor(c0n, dtype=torch.float32, device=DEV).unsqueeze(0)
    # first step against the FP64 oracle on the host (same float64 input)
    u1 = st.step(0.0, c0).cpu().numpy()
    ref = oracle.ch_imex_run(torch.from_numpy(c0n).unsqueeze(0), 1, 0.1).numpy()
    err = oracle.rel_to_max(u1, ref)
    assert err <= 1e-5, err
    del u1, ref, c0n
    # 900 steps forward, then the last 100 differentiated
    u900 = st.advance(c0, 900)
    del c0
    assert torch.isfinite(u900).all()
    r = CahnHilliardAdjoint(vg, dt=0.1)
    target = r.forward(u900, 100, 1.1, 3.0)
    res = {K: r.loss_and_grads(u900, target, 100, 1.0, 3.0, checkpoint_every=K) for K in (10, 100)}
    (l10, g10, m10, e10), (l100, g100, m100, e100) = res[10], res[100]
    assert l10 == pytest.approx(l100, rel=1e-12)
    assert torch.equal(g10, g100)                       # recompute is bit-identical
    assert m10 == pytest.approx(m100, rel=1e-9) and e10 == pytest.approx(e100, rel=1e-9)
    assert torch.isfinite(g10).all()
    h = 1e-3
    fM = (float(r.mse(r.forward(u900, 100, 1.0 + h, 3.0), target))
          - float(r.mse(r.forward(u900, 100, 1.0 - h, 3.0), target))) / (2 * h)
    assert abs(m10 - fM) <= 1e-3 * abs(fM), (m10, fM)
    del res, g10, g100, u900, target
    torch.cuda.empty_cache()
