"""CUDA graph replay of repeated multi-step calls: a plan runs the first call
with a key eagerly, captures the second and replays the graph after that.
Every replayed call must equal the eager path bit for bit, count the same
kernel launches, and a change of any pointer or parameter must not reuse a
graph made for another key."""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture
def graphs(cuda_lib):
    from evoxels_gb300 import _lib
    L = _lib.lib()
    was = L.evx_graphs_enabled()
    yield L
    L.evx_set_graphs(was)


def vg_for(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


def counted(L, fn):
    torch.cuda.synchronize()
    c0 = L.evx_launch_count()
    out = fn()
    torch.cuda.synchronize()
    return out, L.evx_launch_count() - c0


@pytest.mark.parametrize("shape", [(32, 24, 20), (64, 32, 256), (24, 16, 20)])
def test_forward_adjoint_replay_bitexact(graphs, shape):
    """x-pass (z pass for nz = 256) and cuFFT 3-D plans: forward with trajectory and stored spectra, then
    the spectral adjoint with parameter gradients, four identical calls each."""
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    L = graphs
    n = 5
    run = CahnHilliardAdjoint(vg_for(shape), dt=0.1)
    traj = torch.empty((n + 1,) + shape, dtype=torch.float32, device=DEV)
    traj[0] = gpu(oracle.seeded_ch_field(shape, 3))[0]
    spec = run.new_spectra(n)
    lam = gpu(oracle.seeded_unit_field(shape, 4) - 0.5)
    grads = torch.zeros(3, dtype=torch.float64, device=DEV)

    def fwd():
        return run.forward(traj[0:1], n, 1.1, 2.5, traj=traj[1:], spectra=spec).clone()

    def adj():
        grads.zero_()
        out = run.adjoint(traj, n, lam, 1.1, 2.5, grads, spec).clone()
        return out, grads.clone()

    L.evx_set_graphs(0)
    (ref_u, nf_e) = counted(L, fwd)
    ref_traj = traj.clone()
    ((ref_l, ref_g), na_e) = counted(L, adj)
    L.evx_set_graphs(1)
    for _ in range(4):
        traj[1:].fill_(-1.0)
        u, nf = counted(L, fwd)
        assert torch.equal(u, ref_u) and torch.equal(traj, ref_traj)
        assert nf == nf_e
        (lo, g), na = counted(L, adj)
        assert torch.equal(lo, ref_l) and torch.equal(g, ref_g)
        assert na == na_e
    # another parameter set on the same pointers: its own key, not the graph of the first
    L.evx_set_graphs(0)
    ref2 = run.forward(traj[0:1], n, 0.7, 2.5, traj=traj[1:], spectra=spec).clone()
    L.evx_set_graphs(1)
    for _ in range(3):
        assert torch.equal(run.forward(traj[0:1], n, 0.7, 2.5, traj=traj[1:], spectra=spec), ref2)
    assert not torch.equal(ref2, ref_u)


def test_stepper_pointer_change_and_etd1(graphs):
    """PseudoSpectralIMEX.advance and ExponentialEuler.advance on new inputs every call and on repeated
    inputs (alternating buffers, as a solver loop allocates them) equal the eager path."""
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import ExponentialEuler, PseudoSpectralIMEX
    L = graphs
    shape = (32, 16, 24)
    prob = CahnHilliard(vg_for(shape), eps=1.5, D=0.9)
    for st in (PseudoSpectralIMEX(prob, 0.1), ExponentialEuler(prob, 0.1)):
        u0 = gpu(oracle.seeded_ch_field(shape, 8))
        L.evx_set_graphs(0)
        ref, u = [], u0
        for _ in range(6):
            u = st.advance(u, 3)
            ref.append(u.clone())
        L.evx_set_graphs(1)
        u = u0
        for k in range(6):
            u = st.advance(u, 3)
            assert torch.equal(u, ref[k]), k
        for k in range(4):   # the same input again and again
            assert torch.equal(st.advance(u0, 3), ref[0])


def test_batch_replay_bitexact(graphs):
    from evoxels_gb300.batched import BatchedCahnHilliard, BatchTuning
    L = graphs
    shapes = [(32, 32, 32), (16, 24, 64), (24, 20, 36), (32, 32, 32)]
    b = BatchedCahnHilliard(shapes, [1.0, 0.8, 1.2, 0.9], [1.5, 1.0, 0.8, 1.2], 0.1,
                            tuning=BatchTuning(graph_steps=4))
    u0 = b.pack([oracle.seeded_ch_field(s, 20 + i) for i, s in enumerate(shapes)])
    n = 9
    traj = torch.empty((n,) + tuple(u0.shape), dtype=torch.float32, device=DEV)
    states = torch.empty((n + 1,) + tuple(u0.shape), dtype=torch.float32, device=DEV)
    lam = torch.rand_like(u0) - 0.5
    grads = torch.zeros((len(shapes), 3), dtype=torch.float64, device=DEV)

    def run():
        out = b.forward(u0, n).clone()            # chunk graphs inside when eager
        outt = b.forward(u0, n, traj=traj).clone()
        states[0] = u0
        states[1:] = traj
        grads.zero_()
        lo = b.adjoint(states, n, lam, grads).clone()
        return out, outt, lo, grads.clone()

    L.evx_set_graphs(0)
    ref, n_e = counted(L, run)
    L.evx_set_graphs(1)
    for _ in range(4):
        got, n_g = counted(L, run)
        for x, y in zip(got, ref):
            assert torch.equal(x, y)
        assert n_g == n_e


def test_caller_capture_and_profiling_stay_eager(graphs):
    """A call made while the caller captures its own graph runs eagerly into that capture; with kernel
    timing on no graph is used (every launch is timed)."""
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    L = graphs
    shape = (32, 16, 16)
    st = PseudoSpectralIMEX(CahnHilliard(vg_for(shape)), 0.1)
    u0 = gpu(oracle.seeded_ch_field(shape, 9))
    L.evx_set_graphs(0)
    ref = st.advance(u0, 4).clone()
    L.evx_set_graphs(1)
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(3):
            st.advance(u0, 4)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        out = st.advance(u0, 4)
    for _ in range(2):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert torch.equal(out, ref)
    L.evx_prof_reset()
    L.evx_prof_enable(1)
    try:
        for _ in range(3):
            assert torch.equal(st.advance(u0, 4), ref)
        _lib.check(L.evx_prof_collect(), "collect")
        cnt = C_count(L, "ch_axpy")
        assert cnt == 3
    finally:
        L.evx_prof_enable(0)
        L.evx_prof_reset()


def C_count(L, slot):
    import ctypes
    name = ctypes.create_string_buffer(64)
    ms, cnt = ctypes.c_double(), ctypes.c_longlong()
    i = 0
    while L.evx_prof_query(i, name, 64, ctypes.byref(ms), ctypes.byref(cnt)) == 0:
        if name.value.decode() == slot:
            return cnt.value
        i += 1
    return 0
