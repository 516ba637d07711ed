"""Full-size checks through properties that do not depend on the grid size:
the benchmark grids (256^3 and 512^3 Cahn-Hilliard, 512^3 finite differences)
conserve the mean where the scheme does, stay finite and bounded, agree across
the FFT paths of the same step, and match the oracle bit for bit on blocks whose
dependence cone the oracle can evaluate on its own."""

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


def test_ch_256_mean_conserved_and_paths_agree(cuda_lib):
    """The spectral step's k = 0 mode is untouched (the rhs is a divergence): the mean of c stays
    put up to float32 rounding; the y-contiguous z pass and cuFFT's 2-D plans agree."""
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    shape = (256, 256, 256)
    vg = vg_for(shape)
    prob = CahnHilliard(vg)
    g = torch.Generator(device=DEV).manual_seed(5)
    u0 = 0.5 + 0.1 * torch.rand((1,) + shape, device=DEV, generator=g)
    outs = []
    for cufft_yz in (False, True):
        plan = get_plan(vg, cufft_yz=cufft_yz)
        out = torch.empty_like(u0)
        _lib.check(cuda_lib.evx_ch_forward(plan.handle, u0.data_ptr(), out.data_ptr(), 10, None, prob.evx_params(0.1),
                                           None, plan.workspace.data_ptr(), cuda_stream()), "forward")
        outs.append(out)
    a, b = outs
    assert torch.isfinite(a).all()
    m0, m1 = u0.double().mean().item(), a.double().mean().item()
    assert abs(m1 - m0) <= 1e-6 * abs(m0), (m0, m1)
    assert (a.max() - a.min()).item() < (u0.max() - u0.min()).item() * 10
    assert ((a - b).abs().max() / b.abs().max()).item() < 1e-6


def test_fd_512_blocks_bitexact_and_bounded(cuda_lib):
    """Two forward-Euler steps of the 512^3 config (Dirichlet 0 on x, Neumann y and z): blocks at the
    domain corners and in the interior equal the oracle's run on the block (cells within two of a cut
    face excluded), and the maximum principle holds (dt <= h^2/6)."""
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    shape = (512, 512, 512)
    bc = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
    with pytest.warns(UserWarning):
        prob = ReactionDiffusion(vg_for(shape), D=1.0, bc=bc)
    g = torch.Generator(device=DEV).manual_seed(2)
    u0 = torch.rand((1,) + shape, device=DEV, generator=g)
    n, dt = 2, 0.1 / 6
    u = ForwardEuler(prob, dt).advance(u0, n)
    assert u.min().item() >= 0.0 and u.max().item() <= 1.0
    s = 24
    for (x0, y0, z0) in [(0, 0, 0), (512 - s, 512 - s, 512 - s), (250, 100, 300), (0, 300, 512 - s)]:
        blk = u0[:, x0:x0 + s, y0:y0 + s, z0:z0 + s].cpu()
        # the block's own BC on domain faces; a cut face gets a wrong ghost, so cells within n
        # of it are excluded
        ref = blk
        for _ in range(n):
            ref = oracle.fe_step(ref, dt, lambda w: oracle.rd_rhs(w, 1.0, bc))
        lo = [0 if c == 0 else n for c in (x0, y0, z0)]
        hi = [s if c + s == 512 else s - n for c in (x0, y0, z0)]
        got = u[:, x0:x0 + s, y0:y0 + s, z0:z0 + s].cpu()
        sl = (slice(None), slice(lo[0], hi[0]), slice(lo[1], hi[1]), slice(lo[2], hi[2]))
        assert torch.equal(got[sl], ref[sl]), (x0, y0, z0)


def test_ch_512_mean_conserved(cuda_lib):
    """512^3 (the large single-grid config): two IMEX steps conserve the mean and stay finite."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    shape = (512, 512, 512)
    g = torch.Generator(device=DEV).manual_seed(3)
    u0 = 0.5 + 0.1 * torch.rand((1,) + shape, device=DEV, generator=g)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    u = st.advance(u0, 2)
    assert torch.isfinite(u).all()
    m0, m1 = u0.double().mean().item(), u.double().mean().item()
    assert abs(m1 - m0) <= 1e-6 * abs(m0), (m0, m1)
