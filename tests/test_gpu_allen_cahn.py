"""Two-phase Allen-Cahn (19-point normal Laplacian) and RungeKutta4 on the GPU:
bit-exact against the reference's own outputs (golden fixtures) and the oracle
on odd shapes, every BC kind and non-unit spacing; the drop-in driver."""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc

pytestmark = pytest.mark.gpu
DEV = "cuda"


def vg_for(shape, spacing=(1.0, 1.0, 1.0)):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    domain = tuple(n * h for n, h in zip(shape, spacing))
    return VoxelGridGB300(VoxelFields(shape, domain_size=domain).grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


@pytest.mark.parametrize("i", range(5))
def test_ac_rhs_and_rk4_bitexact_vs_reference_golden(cuda_lib, i):
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    from evoxels_gb300.timesteppers import RungeKutta4
    g = load_golden(f"ac_{i}")
    shape = tuple(int(x) for x in g["shape"])
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    if bc is not None:
        kw["bc"] = bc
    prob = TwoPhaseAllenCahn(vg_for(shape), **kw)
    u0 = gpu(g["u0"])
    r = prob.rhs(0.0, u0)
    torch.testing.assert_close(r.cpu(), torch.tensor(g["rhs"]), rtol=0, atol=0)
    st = RungeKutta4(prob, 0.1)
    v = u0
    for _ in range(3):
        v = st.step(0.0, v)
    torch.testing.assert_close(v.cpu(), torch.tensor(g["u3"]), rtol=0, atol=0)


BCS = [None, ("periodic", "periodic", "periodic"), (("dirichlet", (0.1, 0.9)), "neumann", "periodic"),
       ("neumann", ("dirichlet", (1.0, 0.0)), ("dirichlet", (0.3, 0.6))),
       (("dirichlet", (0.0, 1.0)), ("dirichlet", (0.2, 0.4)), "neumann")]


@pytest.mark.parametrize("shape,spacing", [((33, 17, 9), (1.0, 1.0, 1.0)), ((5, 40, 66), (0.5, 0.75, 1.25)),
                                           ((64, 64, 64), (1.0, 1.0, 1.0)), ((3, 2, 70), (2.0, 1.0, 0.5))])
@pytest.mark.parametrize("b", range(len(BCS)))
def test_ac_rhs_bitexact_vs_oracle(cuda_lib, shape, spacing, b):
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    kw = dict(eps=1.7, gab=0.8, M=1.2, force=0.3, curvature=0.1)
    if BCS[b] is not None:
        kw["bc"] = BCS[b]
    prob = TwoPhaseAllenCahn(vg_for(shape, spacing), **kw)
    u0 = 1.4 * oracle.seeded_unit_field(shape, 60 + b) - 0.2
    r = prob.rhs(0.0, gpu(u0)).cpu()
    kw.pop("bc", None)
    ref = oracle.ac_rhs(torch.tensor(u0, dtype=torch.float32).unsqueeze(0), bc=BCS[b], spacing=spacing, **kw)
    torch.testing.assert_close(r, ref, rtol=0, atol=0)


def test_run_allen_cahn_solver_matches_oracle(cuda_lib, capsys):
    import evoxels_gb300 as evo
    shape = (20, 16, 12)
    vf = evo.VoxelFields(shape, domain_size=shape)
    c0 = oracle.seeded_unit_field(shape, 71)
    vf.add_field("phi", c0.copy())
    evo.run_allen_cahn_solver(vf, "phi", "torch", time_increment=0.5, frames=2, max_iters=6, verbose=False)
    ref = oracle.ac_rk4_run(torch.tensor(c0, dtype=torch.float32).unsqueeze(0), 6, dt=0.5).numpy()[0]
    np.testing.assert_array_equal(vf.fields["phi"], ref)   # bit-exact through the whole driver
    # fp64 oracle: fp32 RK4 stays within the per-step bar
    ref64 = oracle.ac_rk4_run(torch.tensor(c0).unsqueeze(0), 6, dt=0.5).numpy()[0]
    assert oracle.rel_to_max(vf.fields["phi"], ref64) <= 1e-5 * 6


def test_ac_potential_forms(cuda_lib):
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    vg = vg_for((8, 8, 8))
    TwoPhaseAllenCahn(vg, potential=lambda u, lib=None: 5.0 * u * (1 - u) * (1 - 2 * u))   # pinned well: fine
    with pytest.raises(NotImplementedError):
        TwoPhaseAllenCahn(vg, potential=lambda u, lib=None: u ** 2)
    # default Neumann BCs: the symbol lives on the x-mirrored grid, as the reference's k_squared
    assert tuple(TwoPhaseAllenCahn(vg).fourier_symbol.shape) == (16, 8, 5)
    assert tuple(TwoPhaseAllenCahn(vg, bc=("periodic",) * 3).fourier_symbol.shape) == (8, 8, 5)


@pytest.mark.parametrize("bc", [None, ("periodic", "periodic", "periodic"),
                                (("dirichlet", (0.2, 0.9)), "neumann", "periodic")])
def test_ac_rhs_stage_equals_rhs_of_stage_field(cuda_lib, bc):
    """rhs(u + c*k) with the stage input formed inside the kernel equals rhs(evx_fe_update(u, k, c))
    bit for bit (RungeKutta4 takes the fused form)."""
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    from evoxels_gb300.voxelgrid import cuda_stream
    shape = (20, 18, 70)
    kw = {} if bc is None else {"bc": bc}
    prob = TwoPhaseAllenCahn(vg_for(shape), eps=2.5, curvature=0.1, **kw)
    u = gpu(1.4 * oracle.seeded_unit_field(shape, 81) - 0.2)
    k = gpu(oracle.seeded_unit_field(shape, 82) - 0.5)
    for c in (0.25, 0.5 * 0.37, 0.37):
        stage = torch.empty_like(u)
        _lib.check(cuda_lib.evx_fe_update(u.data_ptr(), k.data_ptr(), float(np.float32(c)), stage.data_ptr(),
                                          u.numel(), cuda_stream()), "fe")
        torch.testing.assert_close(prob.rhs_stage(0.0, u, k, c), prob.rhs(0.0, stage), rtol=0, atol=0)
