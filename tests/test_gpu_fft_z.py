"""The library's own z pass (y-contiguous half spectrum) used by the x-pass
plans: the standalone transforms against torch.fft, and every spectral path
(IMEX forward, mirrored x, spectral and real-space adjoint gradients, ETD1)
against the same plans on cuFFT's 2-D (y, z) transforms."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def vg_for(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


# (160, 70, 256): more row groups than resident blocks (the C2R's next-item copies) and a last group of
# 6 rows (its copies beyond the grid zero-filled)
@pytest.mark.parametrize("shape", [(3, 32, 256), (2, 96, 256), (4, 70, 128), (2, 33, 64), (1, 7, 256), (2, 1, 64),
                                   (3, 40, 32), (2, 300, 32), (160, 70, 256)])
def test_z_transforms_vs_torch(cuda_lib, shape):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    nx, ny, nz = shape
    u = torch.rand(shape, device=DEV)
    spec = torch.empty((nx, nz // 2 + 1, ny), dtype=torch.complex64, device=DEV)
    _lib.check(cuda_lib.evx_fft_z_r2c(u.data_ptr(), spec.data_ptr(), nx, ny, nz, cuda_stream()), "r2c")
    ref = torch.fft.rfft(u.double(), dim=2).transpose(1, 2)
    err = (spec.to(torch.complex128) - ref).abs().max() / ref.abs().max()
    assert err < 2e-7 * np.log2(nz), err
    back = torch.empty_like(u)
    s2 = spec.clone()
    _lib.check(cuda_lib.evx_fft_z_c2r(s2.data_ptr(), back.data_ptr(), nx, ny, nz, cuda_stream()), "c2r")
    assert torch.equal(s2, spec)                      # the input is not modified
    torch.testing.assert_close(back / nz, u, rtol=0, atol=2e-6)
    # imaginary parts of kz = 0 and nz/2 are ignored, as by a C2R transform
    s3 = spec.clone()
    s3[:, 0, :] += 1j * 0.5
    s3[:, nz // 2, :] -= 1j * 0.25
    back2 = torch.empty_like(u)
    _lib.check(cuda_lib.evx_fft_z_c2r(s3.data_ptr(), back2.data_ptr(), nx, ny, nz, cuda_stream()), "c2r")
    torch.testing.assert_close(back2, back, rtol=0, atol=1e-5)
    with pytest.raises(NotImplementedError):
        _lib.check(cuda_lib.evx_fft_z_r2c(u.data_ptr(), spec.data_ptr(), nx, ny, 96, cuda_stream()), "r2c")


SHAPES = [(32, 64, 64), (64, 40, 128), (16, 48, 256), (128, 8, 64), (8, 20, 128), (32, 24, 32)]


@pytest.mark.parametrize("shape", SHAPES)
def test_forward_matches_cufft_yz_plan(cuda_lib, shape):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    vg = vg_for(shape)
    u0 = gpu(oracle.seeded_ch_field(shape, 5))
    outs = []
    for cufft_yz in (False, True):
        for bc in (None, ("neumann", "periodic", "periodic"), (("dirichlet", (0.2, 0.9)), "periodic", "periodic")):
            prob = CahnHilliard(vg, eps=1.8, D=1.1, bc=bc if bc else ("periodic",) * 3)
            plan = get_plan(vg, bc=prob.bc, cufft_yz=cufft_yz, z_pass=not cufft_yz)
            out = torch.empty_like(u0)
            _lib.check(cuda_lib.evx_ch_forward(plan.handle, u0.data_ptr(), out.data_ptr(), 4, None,
                                               prob.evx_params(0.1), None, plan.workspace.data_ptr(), cuda_stream()),
                       "forward")
            outs.append(out.cpu().numpy())
    for a, b in zip(outs[:3], outs[3:]):
        assert oracle.rel_to_max(a, b) < 1e-6
    ref = oracle.ch_imex_run(torch.tensor(oracle.seeded_ch_field(shape, 5)).unsqueeze(0), 4, 0.1, 1.8, 1.1).numpy()
    assert oracle.rel_to_max(outs[0], ref) < 1e-5


@pytest.mark.parametrize("shape", SHAPES[:4])
@pytest.mark.parametrize("spectral", [True, False])
def test_adjoint_matches_cufft_yz_plan(cuda_lib, shape, spectral):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    L = _lib.lib()
    vg = vg_for(shape)
    prob = CahnHilliard(vg, eps=1.6, D=1.2)
    p = prob.evx_params(0.1)
    n = 3
    u0 = gpu(oracle.seeded_ch_field(shape, 7) + 0.3 * (oracle.seeded_unit_field(shape, 8) - 0.5))
    lam = gpu(oracle.seeded_unit_field(shape, 9) - 0.5)
    res = []
    for cufft_yz in (False, True):
        plan = get_plan(vg, grads=True, cufft_yz=cufft_yz, z_pass=not cufft_yz)
        nf = int(L.evx_ch_spectrum_floats(plan.handle))
        traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
        traj[0] = u0[0]
        out = torch.empty_like(u0)
        spec = torch.empty(max(n * nf, 1), dtype=torch.float32, device=DEV) if spectral else None
        _lib.check(L.evx_ch_forward_spectra(plan.handle, traj[0:1].data_ptr(), out.data_ptr(), n, traj[1:].data_ptr(),
                                            spec.data_ptr() if spectral else None, p, None,
                                            plan.workspace.data_ptr(), cuda_stream()), "fwd")
        lo = torch.empty_like(lam)
        gr = torch.zeros(3, dtype=torch.float64, device=DEV)
        _lib.check(L.evx_ch_adjoint_spectra(plan.handle, traj.data_ptr(), spec.data_ptr() if spectral else None, n,
                                            lam.data_ptr(), lo.data_ptr(), p, gr.data_ptr(), plan.workspace.data_ptr(),
                                            cuda_stream()), "adj")
        res.append((out.cpu().numpy(), lo.cpu().numpy(), gr.cpu().tolist()))
    (a, la, ga), (b, lb, gb) = res
    assert oracle.rel_to_max(a, b) < 1e-6
    assert oracle.rel_to_max(la, lb) < 1e-5
    for x, y in zip(ga, gb):
        assert abs(x - y) <= 1e-3 * max(abs(y), 1e-9), (ga, gb)


def test_etd1_matches_cufft_yz_plan(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import ExponentialEuler, get_plan, mult_table
    from evoxels_gb300.voxelgrid import cuda_stream
    shape = (32, 24, 64)
    for bc in (("periodic",) * 3, ("neumann", "periodic", "periodic")):
        vg = vg_for(shape)
        prob = CahnHilliard(vg, eps=2.0, D=1.0, bc=bc)
        st = ExponentialEuler(prob, 0.1)
        u0 = gpu(oracle.seeded_ch_field(shape, 11))
        r = prob.rhs(0.0, u0)
        outs = []
        for cufft_yz in (False, True):
            plan = get_plan(vg, bc=prob.bc, cufft_yz=cufft_yz, z_pass=not cufft_yz)
            assert cuda_lib.evx_ch_mult_layout(plan.handle) == (0 if cufft_yz else 1)
            m = mult_table(plan, st.dt * st.phi_1_k_squared)   # the z pass's table is [kx][kz][ky]
            out = torch.empty_like(u0)
            _lib.check(cuda_lib.evx_spectral_update(plan.handle, u0.data_ptr(), r.data_ptr(), m.data_ptr(),
                                                    out.data_ptr(), plan.workspace.data_ptr(), cuda_stream()), "etd1")
            outs.append(out.cpu().numpy())
        assert oracle.rel_to_max(outs[0], outs[1]) < 1e-6
