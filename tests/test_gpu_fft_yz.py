"""Fused (y, z) transforms (thread-block clusters, distributed shared memory)
against cuFFT (torch.fft) and FP64 numpy, and the spectral step with them
against the same step on cuFFT's (y, z) plans."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"

SHAPES = [(3, 64, 64), (5, 128, 256), (2, 256, 256), (7, 256, 128), (4, 64, 256), (300, 64, 128), (1, 128, 64),
          (9, 256, 64)]


def _r2c(L, x):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    nx, ny, nz = x.shape
    out = torch.empty((nx, ny, nz // 2 + 1), dtype=torch.complex64, device=DEV)
    _lib.check(L.evx_fft_yz_r2c(x.data_ptr(), out.data_ptr(), nx, ny, nz, cuda_stream()), "evx_fft_yz_r2c")
    return out


def _c2r(L, spec, nz):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    nx, ny, _ = spec.shape
    out = torch.empty((nx, ny, nz), dtype=torch.float32, device=DEV)
    _lib.check(L.evx_fft_yz_c2r(spec.data_ptr(), out.data_ptr(), nx, ny, nz, cuda_stream()), "evx_fft_yz_c2r")
    return out


@pytest.mark.parametrize("shape", SHAPES)
def test_yz_r2c_c2r_vs_cufft_and_fp64(cuda_lib, shape):
    nx, ny, nz = shape
    xn = np.random.default_rng(sum(shape)).standard_normal(shape)
    x = torch.tensor(xn, dtype=torch.float32, device=DEV)
    spec = _r2c(cuda_lib, x)
    ref32 = torch.fft.rfft2(x, dim=(1, 2))
    ref64 = np.fft.rfft2(xn, axes=(1, 2))
    got = torch.view_as_real(spec).cpu().numpy()
    assert oracle.rel_to_max(got, torch.view_as_real(ref32).cpu().numpy()) < 1e-6
    assert oracle.rel_to_max(got, np.stack([ref64.real, ref64.imag], -1)) < 1e-6
    # inverse of a Hermitian-consistent spectrum, unnormalised like cuFFT's C2R
    back = _c2r(cuda_lib, ref32.contiguous(), nz)
    want = torch.fft.irfft2(ref32, s=(ny, nz), dim=(1, 2)) * (ny * nz)
    assert oracle.rel_to_max(back.cpu().numpy(), want.cpu().numpy()) < 1e-6
    assert oracle.rel_to_max(back.cpu().numpy() / (ny * nz), xn) < 1e-6
    assert cuda_lib.evx_device_status(1) == 0


def test_yz_rejects_unsupported(cuda_lib):
    x = torch.zeros((2, 32, 64), dtype=torch.float32, device=DEV)
    with pytest.raises(NotImplementedError):
        _r2c(cuda_lib, x)
    x = torch.zeros((2, 64, 96), dtype=torch.float32, device=DEV)
    with pytest.raises(NotImplementedError):
        _r2c(cuda_lib, x)


@pytest.mark.parametrize("shape", [(32, 64, 128), (64, 256, 256), (16, 128, 64)])
def test_ch_step_with_fused_yz_equals_cufft_yz(cuda_lib, shape):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300, cuda_stream
    vg = VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)
    prob = CahnHilliard(vg, eps=1.7, D=1.3)
    u0 = torch.tensor(oracle.seeded_ch_field(shape, 8), dtype=torch.float32, device=DEV).unsqueeze(0)
    lam = torch.tensor(oracle.seeded_unit_field(shape, 9) - 0.5, dtype=torch.float32, device=DEV).unsqueeze(0)
    res = []
    for fused_yz in (True, False):
        plan = get_plan(vg, grads=True, fused_yz=fused_yz)
        n = 4
        traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
        traj[0] = u0[0]
        out = torch.empty_like(u0)
        p = prob.evx_params(0.1)
        _lib.check(cuda_lib.evx_ch_forward(plan.handle, traj[0:1].data_ptr(), out.data_ptr(), n, traj[1:].data_ptr(),
                                           p, None, plan.workspace.data_ptr(), cuda_stream()))
        lo = torch.empty_like(lam)
        gr = torch.zeros(3, dtype=torch.float64, device=DEV)
        _lib.check(cuda_lib.evx_ch_adjoint(plan.handle, traj.data_ptr(), n, lam.data_ptr(), lo.data_ptr(), p,
                                           gr.data_ptr(), plan.workspace.data_ptr(), cuda_stream()))
        res.append((out, lo, gr.cpu().tolist()))
    (a, la, ga), (b, lb, gb) = res
    assert oracle.rel_to_max(a.cpu().numpy(), b.cpu().numpy()) < 1e-6
    assert oracle.rel_to_max(la.cpu().numpy(), lb.cpu().numpy()) < 1e-5
    for x, y in zip(ga, gb):
        assert abs(x - y) <= 1e-3 * max(abs(y), 1e-9)
    ref = oracle.ch_imex_run(torch.tensor(oracle.seeded_ch_field(shape, 8)).unsqueeze(0), 4, 0.1, 1.7, 1.3).numpy()
    assert oracle.rel_to_max(a.cpu().numpy(), ref) <= 3e-5
