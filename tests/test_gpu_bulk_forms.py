"""The regular-solution bulk term ``log(c) - log(1-c) + w*(1-2c)`` (the logarithmic free energy the
reference's solver notebook passes to ``run_cahn_hilliard_solver``) against fixtures the reference
produced: ``CahnHilliard.rhs`` on the periodic fast path and the generic (Neumann x) kernel within
1e-5 relative to max (CUDA's ``logf`` and torch's ``log`` may differ in the last bit), the drop-in
driver over 20 steps within 1e-5 per step; the bulk form reaches the kernels through the parameter
struct, the adjoint and the batched path refuse it, and unsupported callables raise."""

import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, parse_bc

pytestmark = pytest.mark.gpu
DEV = "cuda"


def regular_solution_mu(c, lib):
    return lib.log(c) - lib.log(1 - c) + 3.0 * (1 - 2 * c)


def _vg(shape):
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    return VoxelGridGB300(VoxelFields(shape, domain_size=shape).grid_info(), device=DEV)


@pytest.mark.parametrize("i", range(2))
def test_rhs_regular_solution_vs_reference(cuda_lib, i):
    from evoxels_gb300 import _lib
    from evoxels_gb300.problem_definition import CahnHilliard
    g = load_golden(f"ch_log_rhs_{i}")
    shape = tuple(g["shape"].tolist())
    bc = parse_bc(g["bc"])
    kw = {"bc": bc} if bc is not None else {}
    prob = CahnHilliard(_vg(shape), eps=3.0, D=1.0, mu_hom=regular_solution_mu, **kw)
    assert prob.evx_params().bulk == _lib.EVX_BULK_REGULAR_SOLUTION and prob.evx_params().w == 3.0
    u = torch.tensor(g["u0"], dtype=torch.float32, device=DEV).unsqueeze(0)
    r = prob.rhs(0.0, u).cpu().numpy()
    assert oracle.rel_to_max(r, g["rhs"]) < 1e-5


def test_driver_regular_solution_vs_reference(cuda_lib):
    import evoxels_gb300 as evo
    g = load_golden("driver_ch_log")
    vf = evo.VoxelFields((16, 16, 16), domain_size=(16, 16, 16))
    vf.add_field("c", np.array(g["u0"]))
    evo.run_cahn_hilliard_solver(vf, "c", "torch", time_increment=0.1, frames=2, max_iters=int(g["n"]),
                                 eps=3.0, diffusivity=1.0, mu_hom=regular_solution_mu, verbose=False)
    err = oracle.rel_to_max(vf.fields["c"], g["c"])
    assert err < 1e-5 * int(g["n"]), err
    # and against the FP64 oracle run from the same float64 field
    ref = oracle.ch_imex_run(torch.tensor(g["u0"]).unsqueeze(0), int(g["n"]), 0.1, mu_hom=regular_solution_mu)
    assert oracle.rel_to_max(vf.fields["c"], ref[0].numpy()) < 1e-5 * int(g["n"])


def test_regular_solution_forward_only_and_unsupported_forms(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.batched import BatchedCahnHilliard
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.timesteppers import get_plan
    from evoxels_gb300.voxelgrid import cuda_stream
    shape = (16, 16, 16)
    vg = _vg(shape)
    prob = CahnHilliard(vg, mu_hom=regular_solution_mu)
    plan = get_plan(vg, grads=True)
    states = torch.full((2,) + shape, 0.5, dtype=torch.float32, device=DEV)
    lam = torch.zeros((1,) + shape, dtype=torch.float32, device=DEV)
    out = torch.empty_like(lam)
    rc = cuda_lib.evx_ch_adjoint(plan.handle, states.data_ptr(), 1, lam.data_ptr(), out.data_ptr(),
                                 prob.evx_params(0.1), None, plan.workspace.data_ptr(), cuda_stream())
    with pytest.raises(NotImplementedError, match="double-well"):
        _lib.check(rc, "evx_ch_adjoint")
    with pytest.raises(NotImplementedError):
        BatchedCahnHilliard([shape], 1.0, 3.0, 0.1, mu_hom=regular_solution_mu)
    with pytest.raises(NotImplementedError, match="log"):
        CahnHilliard(vg, mu_hom=lambda c, lib: lib.sin(c))
