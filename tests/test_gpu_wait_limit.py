"""Bounded device waits and the status word that reports them.

The pipelined x-pass waits on its tile loads with a poll limit.  With the limit set to zero polls every
such wait gives up at once (no fault: all loads still land before the kernel leaves), so the give-up path
runs as it would after a real timeout.  Checked: the status bit is set, the kernel stores nothing more,
the synchronous check and the product's own checks raise (the frame pipeline of the drop-in driver, the
adjoint's gradients), and with the default limit restored the next calls give the same bits as before.
"""

import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"
SHAPE = (64, 64, 64)     # power-of-two x with an even, >= 256 pencil count: the TMA-pipelined x-pass


def _vg(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def test_xpass_wait_give_up_is_reported_and_recovers(cuda_lib):
    import evoxels_gb300 as evo
    from evoxels_gb300 import _lib
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    vg = _vg(SHAPE)
    st = PseudoSpectralIMEX(CahnHilliard(vg), 0.1)
    c0 = oracle.seeded_ch_field(SHAPE, 1)
    u0 = torch.tensor(c0, dtype=torch.float32, device=DEV).unsqueeze(0)
    good = st.advance(u0, 3)
    torch.cuda.synchronize()
    assert cuda_lib.evx_device_status(1) == 0
    runner = CahnHilliardAdjoint(vg, dt=0.1)
    target = runner.forward(u0, 4, 1.2, 3.0)
    ref_grads = runner.loss_and_grads(u0, target, 4, 1.0, 3.0)
    try:
        _lib.check(cuda_lib.evx_set_wait_polls(0), "evx_set_wait_polls")
        st.advance(u0, 3)
        torch.cuda.synchronize()
        assert cuda_lib.evx_device_status(0) & 1
        with pytest.raises(_lib.DeviceWaitError, match="bounded wait"):
            _lib.check_device_status("after advance")
        assert cuda_lib.evx_device_status(0) == 0          # the raise clears the word
        # the drop-in driver reads the word with each frame
        vf = evo.VoxelFields(SHAPE, domain_size=SHAPE)
        vf.add_field("c", c0.copy())
        with pytest.raises(_lib.DeviceWaitError, match="frame 1"):
            evo.run_cahn_hilliard_solver(vf, "c", "torch", frames=2, max_iters=4, verbose=False)
        assert cuda_lib.evx_device_status(0) == 0
        with pytest.raises(_lib.DeviceWaitError):
            runner.loss_and_grads(u0, target, 4, 1.0, 3.0)
    finally:
        cuda_lib.evx_set_wait_polls(-1)
        torch.cuda.synchronize()
        cuda_lib.evx_device_status(1)
    again = st.advance(u0, 3)
    assert torch.equal(again, good)
    l1, g1, d1, e1 = runner.loss_and_grads(u0, target, 4, 1.0, 3.0)
    assert l1 == ref_grads[0] and torch.equal(g1, ref_grads[1]) and (d1, e1) == ref_grads[2:]
    torch.cuda.synchronize()
    assert cuda_lib.evx_device_status(0) == 0


def test_time_dependent_source_bitexact_with_times(cuda_lib):
    """``ReactionDiffusion`` with a source ``f(t, u)``: the user's callable runs as torch operations on
    the device after the stencil kernel, as the reference adds it, and ``advance`` hands each step its
    own time ``t0 + k*dt``: bit-identical to the oracle's loop."""
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    shape = (20, 18, 24)
    bc = ("neumann", "periodic", ("dirichlet", (0.5, 0.0)))
    f = lambda t, c, lib=None: 0.25 * c * (1 - c) + 0.1 * t  # noqa: E731
    with pytest.warns(UserWarning):
        prob = ReactionDiffusion(_vg(shape), D=0.8, f=f, bc=bc)
    assert not prob.source_free
    u0 = torch.tensor(oracle.seeded_unit_field(shape, 12), dtype=torch.float32).unsqueeze(0)
    dt, n, t0 = 0.05, 7, 0.3
    st = ForwardEuler(prob, dt)
    got = st.advance(u0.to(DEV), n, t0=t0).cpu()
    ref = u0
    for k in range(n):
        ref = oracle.fe_step(ref, dt, lambda w, t=t0 + k * dt: oracle.rd_rhs(w, 0.8, bc, f=f, t=t))
    assert torch.equal(got, ref)
    # rhs alone, and a source that vanishes at t = 0 is not dropped
    g = lambda t, c: t * c  # noqa: E731
    with pytest.warns(UserWarning):
        p2 = ReactionDiffusion(_vg(shape), D=0.8, f=g, bc=bc)
    r = p2.rhs(0.7, u0.to(DEV)).cpu()
    assert torch.equal(r, oracle.rd_rhs(u0, 0.8, bc, f=g, t=0.7))
