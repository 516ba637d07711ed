"""The benchmark configurations at their stated sizes, against the oracle.

* Plain Cahn-Hilliard through the drop-in driver ``run_cahn_hilliard_solver``: 100^3,
  c0 = 0.5 + 0.1 U[0,1) from seed 1, dt 0.1, 1000 steps, 10 frames, the reference defaults
  (eps 3, D 1, A 0.25, default bulk term).  Every exported frame against the FP64 oracle run from
  the same float64 field: <= 1e-5 relative to max per step for the first frames and <= 1e-4 at
  every frame up to step 1000 (the reference's own float32 run is 2.2e-5 from FP64 after 1000
  steps at this size).
* Explicit finite differences with the stencil configuration's boundaries (Dirichlet 0 on x,
  Neumann on y and z, dt = 1/60, U[0,1) from seed 2): all 2000 steps at 64^3 bit-identical to the
  float32 oracle for 1, 2 and 4 steps per HBM pass; at 512^3, 12 steps on corner, edge and
  interior blocks (cells whose dependence cone crosses a cut face excluded).
* Batched uneven instances: the 64-instance layout itself (sides from {32, 48, 64, 96, 128} drawn
  with seed 4, M ~ U[0.5, 2], kappa ~ U[0.5, 3], bulk pinned to 18/3, c0 from seeds (4, i)), with
  the autotuned tuning the benchmark uses.  Every instance within 1e-6 of the same instance
  stepped alone, a sample of instances within 1e-5 per step of the FP64 oracle; the adjoint of
  every instance within 1e-5 of the single-grid adjoint, and one instance of each side against the
  FP64 oracle's autograd (parameter gradients within 1e-3).
"""

import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _vg(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def test_driver_100cubed_1000_steps_every_frame_vs_fp64(cuda_lib):
    import evoxels_gb300 as evo
    torch.set_num_threads(os.cpu_count() or 1)
    shape = (100, 100, 100)
    c0 = oracle.seeded_ch_field(shape, 1)
    vf = evo.VoxelFields(shape, domain_size=shape)
    vf.add_field("c", c0.copy())
    frames = []
    orig = vf.set_field

    def record(name, arr):
        frames.append(np.array(arr, dtype=np.float32, copy=True))
        orig(name, arr)
    vf.set_field = record
    evo.run_cahn_hilliard_solver(vf, "c", "torch", jit=True, time_increment=0.1, frames=10, max_iters=1000,
                                 verbose=False)
    assert len(frames) == 11                     # steps 0, 100, ..., 900 and the final state
    u = torch.from_numpy(c0).unsqueeze(0)        # FP64 oracle from the same float64 field
    errs = []
    for f, fr in enumerate(frames):
        if f:
            u = oracle.ch_imex_run(u, 100, 0.1)
        errs.append(oracle.rel_to_max(fr, u[0].numpy()))
    print("config 1 frame errors vs FP64:", ["%.2e" % e for e in errs])
    assert errs[0] <= 6e-8                        # the float32 cast of the input
    assert max(errs) <= 1e-4, errs
    assert errs[1] <= 1e-5 * 100, errs


@pytest.mark.parametrize("spp", [1, 2, 4])
def test_fd_config_bcs_2000_steps_bitexact_64cubed(cuda_lib, spp):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    shape = (64, 64, 64)
    bc = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
    with pytest.warns(UserWarning):
        prob = ReactionDiffusion(_vg(shape), D=1.0, bc=bc)
    u0 = torch.tensor(oracle.seeded_unit_field(shape, 2), dtype=torch.float32).unsqueeze(0)
    dt, n = 0.1 / 6, 2000
    got = ForwardEuler(prob, dt, steps_per_pass=spp).advance(u0.to(DEV), n).cpu()
    ref = oracle.rd_fe_run(u0, n, dt, 1.0, bc)
    assert torch.equal(got, ref)
    # the float32 run stays within the reference's own float32-vs-FP64 floor scale
    ref64 = oracle.rd_fe_run(u0.double(), n, dt, 1.0, bc)
    assert oracle.rel_to_max(got.numpy(), ref64.numpy()) <= 2e-5


def test_fd_512_blocks_12_steps_bitexact(cuda_lib):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    shape = (512, 512, 512)
    bc = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
    with pytest.warns(UserWarning):
        prob = ReactionDiffusion(_vg(shape), D=1.0, bc=bc)
    u0 = torch.tensor(oracle.seeded_unit_field(shape, 2), dtype=torch.float32, device=DEV).unsqueeze(0)
    n, dt, s = 12, 0.1 / 6, 40
    u = ForwardEuler(prob, dt).advance(u0, n)
    assert u.min().item() >= 0.0 and u.max().item() <= 1.0
    for (x0, y0, z0) in [(0, 0, 0), (512 - s, 512 - s, 512 - s), (236, 100, 300), (0, 300, 512 - s),
                         (512 - s, 0, 200)]:
        blk = u0[:, x0:x0 + s, y0:y0 + s, z0:z0 + s].cpu()
        ref = oracle.rd_fe_run(blk, n, dt, 1.0, bc)
        lo = [0 if c == 0 else n for c in (x0, y0, z0)]
        hi = [s if c + s == 512 else s - n for c in (x0, y0, z0)]
        got = u[:, x0:x0 + s, y0:y0 + s, z0:z0 + s].cpu()
        sl = (slice(None), slice(lo[0], hi[0]), slice(lo[1], hi[1]), slice(lo[2], hi[2]))
        assert torch.equal(got[sl], ref[sl]), (x0, y0, z0)


def _config4():
    rng = np.random.default_rng(4)
    sides = rng.choice([32, 48, 64, 96, 128], 64)
    M = rng.uniform(0.5, 2.0, 64)
    kappa = rng.uniform(0.5, 3.0, 64)
    shapes = [(int(a),) * 3 for a in sides]
    fields = [0.5 + 0.1 * np.random.default_rng([4, i]).random(s) for i, s in enumerate(shapes)]
    return shapes, M, kappa / 2, fields


PIN = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)  # noqa: E731


@pytest.fixture(scope="module")
def config4_batch():
    from evoxels_gb300 import autotune
    from evoxels_gb300.batched import BatchedCahnHilliard
    shapes, M, eps, fields = _config4()
    tuning = autotune.tune_batched(shapes, M, eps, 0.1, mu_hom=PIN, steps=10, use_cache=False)
    b = BatchedCahnHilliard(shapes, M, eps, 0.1, mu_hom=PIN, tuning=tuning)
    return b, shapes, M, eps, fields


def test_batched_config4_forward_every_instance(cuda_lib, config4_batch):
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    b, shapes, M, eps, fields = config4_batch
    n = 5
    outs = b.unpack(b.forward(b.pack(fields), n))
    sample = {int(np.argmax([s[0] for s in shapes])), 0, 17, 40}
    for i, s in enumerate(shapes):
        st = PseudoSpectralIMEX(CahnHilliard(_vg(s), eps=float(eps[i]), D=float(M[i]), mu_hom=PIN), 0.1)
        ref = st.advance(torch.tensor(fields[i], dtype=torch.float32, device=DEV).unsqueeze(0), n)
        assert oracle.rel_to_max(outs[i].cpu().numpy(), ref.cpu().numpy()) < 1e-6, i
        if i in sample:
            r64 = oracle.ch_imex_run(torch.tensor(fields[i]).unsqueeze(0), n, 0.1, float(eps[i]), float(M[i]),
                                     mu_hom=PIN)
            assert oracle.rel_to_max(outs[i].cpu().numpy(), r64.numpy()) < 1e-5 * n, i


def _fp64_adjoint(f0, lam, n, eps, M):
    """dL/du_0 and the parameter gradients of <lam, u_n> through n FP64 oracle steps (torch autograd
    step by step, the bulk term pinned)."""
    keep = []
    oracle.ch_imex_run(torch.tensor(f0).unsqueeze(0), n, 0.1, eps, M, mu_hom=PIN, keep=keep)
    lt, dD, de = torch.tensor(lam).unsqueeze(0), 0.0, 0.0
    for s in range(n - 1, -1, -1):
        lt, a, b = oracle.ch_imex_vjp(keep[s], lt, 0.1, eps, M, mu_hom=PIN)
        dD, de = dD + a, de + b
    return lt, dD, de


def test_batched_config4_adjoint_every_instance(cuda_lib, config4_batch):
    """The batched forward + adjoint (increment spectra kept, spectral parameter gradients) against
    each instance's single-grid forward + adjoint: dL/du_0 within 1e-5, the parameter gradients within
    1e-4 where the single grid also keeps increment spectra (power-of-two sides); one instance of each
    side against the FP64 oracle's autograd: dL/du_0 within 1e-5, dL/dM and dL/deps within 1e-3."""
    from evoxels_gb300.adjoint import CahnHilliardAdjoint
    b, shapes, M, eps, fields = config4_batch
    n = 3
    states = torch.empty((n + 1) * b.total, dtype=torch.float32, device=DEV)
    states[:b.total].copy_(b.pack(fields))
    spec = b.new_spectra(n)
    b.forward(states[:b.total], n, traj=states[b.total:], spectra=spec)
    lams = [np.random.default_rng([9, i]).random(s) - 0.5 for i, s in enumerate(shapes)]
    grads = torch.zeros((b.n, 3), dtype=torch.float64, device=DEV)
    outs = b.unpack(b.adjoint(states, n, b.pack(lams), grads, spectra=spec))
    gD, geps = b.param_grads(grads)
    runners, sampled = {}, set()
    for i, s in enumerate(shapes):
        r = runners.get(s)
        if r is None:
            r = runners[s] = CahnHilliardAdjoint(_vg(s), 0.1, pinned_w=18 / 3.0)
        tr = torch.empty((n + 1,) + s, dtype=torch.float32, device=DEV)
        tr[0] = torch.tensor(fields[i], dtype=torch.float32, device=DEV)
        sp = r.new_spectra(n)
        r.forward(tr[0:1], n, float(M[i]), float(eps[i]), traj=tr[1:], spectra=sp)
        g1 = torch.zeros(3, dtype=torch.float64, device=DEV)
        lg = torch.tensor(lams[i], dtype=torch.float32, device=DEV).unsqueeze(0)
        ref = r.adjoint(tr, n, lg, float(M[i]), float(eps[i]), g1, sp)
        assert oracle.rel_to_max(outs[i].cpu().numpy(), ref.cpu().numpy()) < 1e-5, i
        if sp is not None:
            d1, e1 = r.param_grads(g1, float(eps[i]))
            assert abs(gD[i] - d1) <= 1e-4 * abs(d1) and abs(geps[i] - e1) <= 1e-4 * abs(e1), (i, gD[i], d1)
        if s[0] not in sampled:
            sampled.add(s[0])
            l64, d64, e64 = _fp64_adjoint(fields[i], lams[i], n, float(eps[i]), float(M[i]))
            assert oracle.rel_to_max(outs[i].cpu().numpy(), l64.numpy()) < 1e-5, i
            assert abs(gD[i] - d64) <= 1e-3 * abs(d64), (i, gD[i], d64)
            assert abs(geps[i] - e64) <= 1e-3 * abs(e64), (i, geps[i], e64)
