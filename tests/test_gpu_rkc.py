"""Runge-Kutta-Chebyshev schemes (RKC1, RKC2) on the GPU over the Allen-Cahn,
reaction-diffusion and Cahn-Hilliard right-hand sides: bit-exact against the
reference's own runs (golden fixtures) given the same float32 stage
coefficients, within float32 rounding of them with this host's coefficients,
against the FP64 oracle on larger odd grids, and through the solver driver."""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc

pytestmark = pytest.mark.gpu
DEV = "cuda"


def vg_for(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


def gpu(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device=DEV).reshape((1,) + np.asarray(a).shape[-3:])


def stepper_for(g):
    from evoxels_gb300 import problem_definition as PD
    from evoxels_gb300 import timesteppers as TS
    shape = tuple(int(x) for x in g["shape"])
    bc = parse_bc(g["bc"])
    kw = eval(str(g["kw"]))   # the fixture's own repr of the keyword dict
    kw.pop("bc", None)
    if bc is not None:
        kw["bc"] = bc
    prob = getattr(PD, str(g["problem"]))(vg_for(shape), **kw)
    return getattr(TS, str(g["scheme"]))(prob, float(g["dt"]), **eval(str(g["skw"])))


@pytest.mark.parametrize("i", range(5))
def test_rkc_bitexact_vs_reference_golden(cuda_lib, i):
    g = load_golden(f"rkc_{i}")
    st = stepper_for(g)
    names = [k for k in ("mu0", "mu1", "mu11", "nu", "c", "gamma") if k in g]
    for k in names:   # this host's libm may round cosh/arccosh an ulp apart from the fixture's
        np.testing.assert_allclose(getattr(st, k).numpy(), g[k], rtol=3e-7, atol=0)
    u = gpu(g["u0"])
    v = u
    for _ in range(3):
        v = st.step(0.0, v)
    assert oracle.rel_to_max(v.cpu().numpy()[0], g["u3"][0]) < 1e-5
    for k in names:
        setattr(st, k, torch.tensor(g[k]))
    v = u
    for _ in range(3):
        v = st.step(0.0, v)
    assert np.array_equal(v.cpu().numpy(), g["u3"])


@pytest.mark.parametrize("order,shape,polygrad", [(1, (33, 20, 17), 4), (2, (40, 24, 30), 5), (2, (64, 64, 64), 8),
                                                  (1, (17, 9, 70), 10)])
def test_rkc_allen_cahn_vs_fp64_oracle(cuda_lib, order, shape, polygrad):
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    from evoxels_gb300.timesteppers import RKC1, RKC2
    bc = (("dirichlet", (0.0, 1.0)), "periodic", "neumann")
    prob = TwoPhaseAllenCahn(vg_for(shape), eps=2.5, curvature=0.1, bc=bc)
    st = (RKC1 if order == 1 else RKC2)(prob, 0.2, polygrad=polygrad)
    assert st.order == order
    u0n = 1.4 * oracle.seeded_unit_field(shape, 70 + polygrad) - 0.2
    v = gpu(u0n)
    for _ in range(4):
        v = st.step(0.0, v)
    out = {}
    for dtype in (torch.float32, torch.float64):
        k = oracle.rkc_coeffs(order, polygrad, dtype=dtype)
        ref = torch.tensor(u0n, dtype=dtype).unsqueeze(0)
        for _ in range(4):
            ref = oracle.rkc_step(ref, 0.2, lambda w: oracle.ac_rhs(w, eps=2.5, curvature=0.1, bc=bc), k)
        out[dtype] = ref.numpy()
    # the float32 oracle runs the reference's operations on this host: bit for bit
    assert np.array_equal(v.cpu().numpy(), out[torch.float32])
    # the Chebyshev recursion (mu0 ~ 2, nu ~ -1) amplifies float32 rounding with the stage count
    assert oracle.rel_to_max(v.cpu().numpy(), out[torch.float64]) < 4e-4


def test_rkc2_driver_and_stage_errors(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
    from evoxels_gb300.solvers import TimeDependentSolver
    from evoxels_gb300.timesteppers import RKC2
    from evoxels_gb300.voxelfields import VoxelFields
    shape = (16, 12, 10)
    vf = VoxelFields(shape, domain_size=shape)
    u0 = oracle.seeded_unit_field(shape, 80)
    vf.add_field("phi", u0.copy())
    solver = TimeDependentSolver(vf, "phi", "torch", problem_cls=TwoPhaseAllenCahn, timestepper_cls=RKC2)
    solver.solve(time_increment=0.2, frames=2, max_iters=6, problem_kwargs={"eps": 2.0}, jit=False, verbose=False)
    k = oracle.rkc_coeffs(2, dtype=torch.float32)
    ref = torch.tensor(u0, dtype=torch.float32).unsqueeze(0)
    for _ in range(6):
        ref = oracle.rkc_step(ref, 0.2, lambda w: oracle.ac_rhs(w, eps=2.0), k)
    assert np.array_equal(vf.fields["phi"], ref.numpy()[0])
    c = _lib.EvxRkcCoeffs()
    x = torch.zeros(8, device=DEV)
    with pytest.raises(_lib.EvxError, match="NULL"):
        _lib.check(cuda_lib.evx_rkc_stage(x.data_ptr(), None, x.data_ptr(), x.data_ptr(), None, c, x.data_ptr(), 8,
                                          None), "evx_rkc_stage")
