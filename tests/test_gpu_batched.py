"""Batched uneven instances against the single-grid path and the FP64 oracle.

Bars: each instance of the batch within 1e-6 (relative to max) of the same
instance stepped alone (the stencils are bit-identical; cuFFT's batched plans
may round differently), within 1e-5 per step of the FP64 oracle; tunings that
do not change the FFT grouping give identical bits; adjoint within 1e-5 and
parameter gradients within 1e-4 of the single-grid adjoint.
"""

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu

SHAPES = [(32, 32, 32), (48, 48, 48), (16, 24, 64), (32, 32, 32), (24, 20, 36), (8, 12, 100)]
D = [1.0, 0.7, 1.6, 1.2, 0.9, 1.1]
EPS = [1.5, 0.5, 1.2, 0.8, 1.0, 1.4]
PIN = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)  # noqa: E731


def fields(seed=4):
    return [oracle.seeded_ch_field(s, (seed * 100 + i)) for i, s in enumerate(SHAPES)]


def single(shape, d, e, mu=None):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    vf = VoxelFields(shape, domain_size=shape)
    vg = VoxelGridGB300(vf.grid_info(), device="cuda")
    prob = CahnHilliard(vg, eps=e, D=d, mu_hom=mu)
    return vg, prob, PseudoSpectralIMEX(prob, 0.1)


@pytest.mark.parametrize("mu", [None, PIN])
def test_batched_forward_matches_single_grids_and_fp64(cuda_lib, mu):
    from evoxels_gb300.batched import BatchedCahnHilliard
    b = BatchedCahnHilliard(SHAPES, D, EPS, 0.1, mu_hom=mu)
    f = fields()
    n = 6
    traj = torch.empty(n * b.total, dtype=torch.float32, device="cuda")
    out = b.forward(b.pack(f), n, traj=traj)
    outs = b.unpack(out)
    for i, s in enumerate(SHAPES):
        _, _, st = single(s, D[i], EPS[i], mu)
        ref = st.advance(torch.tensor(f[i], dtype=torch.float32, device="cuda").unsqueeze(0), n)
        assert oracle.rel_to_max(outs[i].cpu().numpy(), ref.cpu().numpy()) < 1e-6
        keep = []
        oracle.ch_imex_run(torch.tensor(f[i], dtype=torch.float64).unsqueeze(0), n, 0.1, EPS[i], D[i],
                           mu_hom=mu, keep=keep)
        assert oracle.rel_to_max(outs[i].cpu().numpy(), keep[-1].numpy()) < 1e-5 * n
        # the trajectory's last slot is the output; an intermediate one matches its step
        last = traj[(n - 1) * b.total:n * b.total]
        assert torch.equal(b.unpack(last)[i], outs[i])
        mid = b.unpack(traj[2 * b.total:3 * b.total])[i]
        assert oracle.rel_to_max(mid.cpu().numpy(), keep[3].numpy()) < 1e-5 * 3


def test_batched_tunings_and_graphs_agree(cuda_lib):
    from evoxels_gb300.batched import BatchedCahnHilliard, BatchTuning
    f = fields(5)
    n = 25
    base = BatchedCahnHilliard(SHAPES, D, EPS, 0.1, tuning=BatchTuning(graph_steps=0))
    ref = base.forward(base.pack(f), n)
    ref_list = [t.clone() for t in base.unpack(ref)]
    for tune in [BatchTuning(graph_steps=20), BatchTuning(graph_steps=4, tile_variant=0),
                 BatchTuning(tile_variant=1, x_chunk=8), BatchTuning(x_chunk=64, blocks_per_sm=1),
                 BatchTuning(fft_group_max=1)]:
        b = BatchedCahnHilliard(SHAPES, D, EPS, 0.1, tuning=tune)
        u0 = b.pack(f)
        out = b.forward(u0, n)
        out2 = b.forward(u0, n)   # the cached graph is replayed
        assert torch.equal(out, out2)
        for i, t in enumerate(b.unpack(out)):
            if tune.fft_group_max:
                assert oracle.rel_to_max(t.cpu().numpy(), ref_list[i].cpu().numpy()) < 1e-6, tune
            else:
                assert torch.equal(t, ref_list[i]), tune


def test_batched_adjoint_matches_single_grids(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.batched import BatchedCahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    b = BatchedCahnHilliard(SHAPES, D, EPS, 0.1)
    f = fields(6)
    n = 3
    states = torch.empty((n + 1) * b.total, dtype=torch.float32, device="cuda")
    states[:b.total].copy_(b.pack(f))
    b.forward(states[:b.total], n, traj=states[b.total:])
    rng = np.random.default_rng(9)
    lams = [rng.random(s) - 0.5 for s in SHAPES]
    lam = b.pack(lams)
    grads = torch.zeros((b.n, 3), dtype=torch.float64, device="cuda")
    out = b.adjoint(states, n, lam, grads)
    outs = b.unpack(out)
    for i, s in enumerate(SHAPES):
        vg, prob, st = single(s, D[i], EPS[i])
        tr = torch.stack([b.unpack(states[k * b.total:(k + 1) * b.total])[i][0] for k in range(n + 1)]).contiguous()
        plan = get_plan(vg, grads=True)
        lg = torch.tensor(lams[i], dtype=torch.float32, device="cuda").unsqueeze(0)
        ref = torch.empty_like(lg)
        g1 = torch.zeros(3, dtype=torch.float64, device="cuda")
        _lib.check(_lib.lib().evx_ch_adjoint(plan.handle, tr.data_ptr(), n, lg.data_ptr(), ref.data_ptr(),
                                             prob.evx_params(0.1), g1.data_ptr(), plan.workspace.data_ptr(),
                                             cuda_stream()))
        assert oracle.rel_to_max(outs[i].cpu().numpy(), ref.cpu().numpy()) < 1e-5
        for x, y in zip(grads[i].cpu().tolist(), g1.cpu().tolist()):
            # float32 per-thread partial sums are grouped differently (work items vs blocks)
            assert abs(x - y) <= 1e-4 * max(abs(y), 1e-9), (i, x, y)


@pytest.mark.parametrize("flags", [{}, {"cufft3d": True}])
def test_batched_spectral_grads_match_real_space(cuda_lib, flags):
    """Stored increment spectra (x-pass layout for the power-of-two groups, rfftn layout for the others,
    or every group on cuFFT 3-D): the forward is unchanged by storing, dL/du_0 agrees with the
    real-space adjoint to 1e-6 and the parameter gradients to 1e-4 (the real-space sums difference
    float32 states, the spectral ones use the exact increments)."""
    from evoxels_gb300.batched import BatchedCahnHilliard
    b = BatchedCahnHilliard(SHAPES, D, EPS, 0.1, **flags)
    n = 3
    u0 = b.pack(fields(8))
    res = []
    for spectral in (True, False):
        states = torch.empty((n + 1) * b.total, dtype=torch.float32, device="cuda")
        states[:b.total].copy_(u0)
        spec = b.new_spectra(n) if spectral else None
        out = b.forward(states[:b.total], n, traj=states[b.total:], spectra=spec)
        lam = b.pack([np.random.default_rng([11, i]).random(s) - 0.5 for i, s in enumerate(SHAPES)])
        grads = torch.zeros((b.n, 3), dtype=torch.float64, device="cuda")
        lo = b.adjoint(states, n, lam, grads, spectra=spec)
        res.append((out, states, lo, grads.cpu().numpy()))
    (oa, sa, la, ga), (ob, sb, lb, gb) = res
    assert torch.equal(oa, ob) and torch.equal(sa, sb)
    for x, y in zip(b.unpack(la), b.unpack(lb)):
        assert oracle.rel_to_max(x.cpu().numpy(), y.cpu().numpy()) < 1e-6
    for i in range(b.n):
        for x, y in zip(ga[i], gb[i]):
            assert abs(x - y) <= 1e-4 * max(abs(y), 1e-9), (i, ga[i], gb[i])
    with pytest.raises(Exception, match="trajectory"):
        b.forward(u0, n, spectra=b.new_spectra(n))


def test_autotuner_returns_a_valid_tuning(cuda_lib, tmp_path, monkeypatch):
    from evoxels_gb300 import autotune
    from evoxels_gb300.batched import BatchTuning
    monkeypatch.setenv("EVX_AUTOTUNE_CACHE", str(tmp_path / "cache.json"))
    space = {"tile_variant": [-1, 1], "graph_steps": [20, 0]}
    t = autotune.tune_batched(SHAPES[:3], 1.0, 1.0, steps=4, space=space)
    assert isinstance(t, BatchTuning)
    again = autotune.tune_batched(SHAPES[:3], 1.0, 1.0, steps=4, space=space)   # from the cache
    assert again == t
    assert (tmp_path / "cache.json").exists()


@pytest.mark.parametrize("variant", ["cufft3d", "cufft_yz"])
def test_batched_xpass_groups_match_cufft3d(cuda_lib, variant):
    """Power-of-two groups (batched x-pass; with the library's z pass in the second case)
    against cuFFT 3-D or cuFFT's 2-D (y, z) plans for every group."""
    from evoxels_gb300.batched import BatchedCahnHilliard
    f = fields(7)
    res = []
    for other in (False, True):
        kw = {variant: other} if variant == "cufft3d" else ({"cufft_yz": True} if other else {"z_pass": True})
        b = BatchedCahnHilliard(SHAPES, D, EPS, 0.1, **kw)
        n = 4
        states = torch.empty((n + 1) * b.total, dtype=torch.float32, device="cuda")
        states[:b.total].copy_(b.pack(f))
        b.forward(states[:b.total], n, traj=states[b.total:])
        lam = b.pack([np.random.default_rng(11 + i).random(s) - 0.5 for i, s in enumerate(SHAPES)])
        grads = torch.zeros((b.n, 3), dtype=torch.float64, device="cuda")
        out = b.adjoint(states, n, lam, grads)
        res.append((b.unpack(states[n * b.total:]), b.unpack(out), grads.cpu().numpy()))
    (ua, la, ga), (ub, lb, gb) = res
    for i in range(len(SHAPES)):
        assert oracle.rel_to_max(ua[i].cpu().numpy(), ub[i].cpu().numpy()) < 1e-6, i
        assert oracle.rel_to_max(la[i].cpu().numpy(), lb[i].cpu().numpy()) < 1e-5, i
        # real-space gradient sums difference float32 states: the cross-FFT bar
        np.testing.assert_allclose(ga[i], gb[i], rtol=1e-3, atol=1e-9)


ODD = [(8, 12, 100), (24, 20, 36), (16, 24, 64), (8, 12, 100), (48, 8, 4), (12, 16, 8), (32, 32, 32), (64, 8, 12),
       (6, 5, 28), (8, 12, 100)]


@pytest.mark.parametrize("tune", [{}, {"x_chunk": 3}, {"tile_variant": 1, "x_chunk": 5}, {"fft_group_max": 1},
                                  {"tile_variant": 0, "blocks_per_sm": 1}])
def test_batched_odd_group_layouts_match_single_grids(cuda_lib, tune):
    """Ten instances in eight shape groups (padding between groups, nz down to 4, ny below the tile
    height, x chunks that do not divide nx), every tile shape and chunking: the layout passes the
    batch's own descriptor check at creation, and every instance (forward with trajectory, then the
    adjoint) equals the instance run alone within 1e-6 / 1e-5."""
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    from evoxels_gb300.batched import BatchedCahnHilliard, BatchTuning
    d = [1.0 + 0.1 * i for i in range(len(ODD))]
    e = [0.5 + 0.2 * i for i in range(len(ODD))]
    b = BatchedCahnHilliard(ODD, d, e, 0.1, tuning=BatchTuning(**tune))
    f = [oracle.seeded_ch_field(s, 300 + i) for i, s in enumerate(ODD)]
    n = 3
    states = torch.empty((n + 1) * b.total, dtype=torch.float32, device="cuda")
    states[:b.total].copy_(b.pack(f))
    out = b.forward(states[:b.total], n, traj=states[b.total:])
    lam = b.pack([np.random.default_rng([13, i]).random(s) - 0.5 for i, s in enumerate(ODD)])
    grads = torch.zeros((b.n, 3), dtype=torch.float64, device="cuda")
    lo = b.unpack(b.adjoint(states, n, lam, grads))
    outs = b.unpack(out)
    lams = b.unpack(lam)
    for i, s in enumerate(ODD):
        vg, prob, st = single(s, d[i], e[i])
        ref = st.advance(torch.tensor(f[i], dtype=torch.float32, device="cuda").unsqueeze(0), n)
        assert oracle.rel_to_max(outs[i].cpu().numpy(), ref.cpu().numpy()) < 1e-6, (i, tune)
        r = CahnHilliardAdjoint(vg, 0.1)
        tr = torch.stack([b.unpack(states[k * b.total:(k + 1) * b.total])[i][0] for k in range(n + 1)]).contiguous()
        lr = r.adjoint(tr, n, lams[i].contiguous(), d[i], e[i], None)
        assert oracle.rel_to_max(lo[i].cpu().numpy(), lr.cpu().numpy()) < 1e-5, (i, tune)
