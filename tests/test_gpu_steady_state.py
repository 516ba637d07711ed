"""Pseudo-time steady-state solver (evoxels/solvers.py:210-247) on the CUDA
path: the iterates, the stopping iteration, the per-field relative changes and
the exported field against the oracle's restatement of the loop; one step
evaluation per iteration; ``max_iters`` bounds a run that does not converge."""

import warnings

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SHAPE = (16, 12, 10)
BC = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
DT = 0.15
CRIT = 9.97e-6   # between two checks' relative changes (>= 0.27% from each)


def _solver(step_fn=None, conv_crit=CRIT, check_freq=10):
    import evoxels_gb300 as evo
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.solvers import SteadyStatePseudoTimeSolver
    from evoxels_gb300.timesteppers import ForwardEuler
    vf = evo.VoxelFields(SHAPE, domain_size=SHAPE)
    vf.add_field("c", oracle.seeded_unit_field(SHAPE, 7))
    kw = dict(step_fn=step_fn) if step_fn else dict(problem_cls=ReactionDiffusion, timestepper_cls=ForwardEuler)
    return vf, SteadyStatePseudoTimeSolver(vf, "c", "torch", conv_crit=conv_crit, check_freq=check_freq, **kw)


def _oracle_run(conv_crit, check_freq, max_iters):
    import torch
    u0 = torch.from_numpy(oracle.seeded_unit_field(SHAPE, 7)).to(torch.float32)[None]
    step = lambda v: oracle.fe_step(v, DT, lambda w: oracle.rd_rhs(w, 1.0, BC))  # noqa: E731
    return oracle.steady_state_run(u0, step, max_iters, conv_crit, check_freq)


def _solve(solver, max_iters=5000, verbose=False):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")   # Dirichlet on a cell-centred grid
        solver.solve(time_increment=DT, max_iters=max_iters, problem_kwargs={"D": 1.0, "bc": BC}, verbose=verbose)


@pytest.mark.parametrize("check_freq", [1, 7])
def test_steady_state_matches_oracle(cuda_lib, check_freq):
    vf, solver = _solver(check_freq=check_freq)
    _solve(solver)
    u_ref, it_ref, conv_ref, checks = _oracle_run(CRIT, check_freq, 5000)
    assert conv_ref and solver.converged
    assert solver.iter == it_ref
    # forward Euler steps are bit-exact, so the converged field is too
    np.testing.assert_array_equal(vf.fields["c"], u_ref[0].numpy())


def test_steady_state_rel_changes_match_oracle(cuda_lib):
    import torch
    vf, solver = _solver()
    _solve(solver, max_iters=1)   # builds the stepper; one check at iteration 0
    u = torch.from_numpy(oracle.seeded_unit_field(SHAPE, 7)).to(torch.float32)[None]
    u_next = oracle.fe_step(u, DT, lambda w: oracle.rd_rhs(w, 1.0, BC))
    ours = solver.rel_changes(u.cuda(), u_next.cuda())
    _, _, _, checks = _oracle_run(CRIT, 10, 1)
    # device reduction in double against the reference's float32 norm
    assert abs(ours[0] - checks[0][1][0]) <= 1e-6 * checks[0][1][0]


def test_steady_state_one_step_per_iteration(cuda_lib):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.timesteppers import ForwardEuler
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    vg = VoxelGridGB300(VoxelFields(SHAPE, domain_size=SHAPE).grid_info(), device="cuda")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        stepper = ForwardEuler(ReactionDiffusion(vg, D=1.0, bc=BC), DT)
    calls = []

    def step_fn(t, u):
        calls.append(t)
        return stepper.step(t, u)
    vf, solver = _solver(step_fn=step_fn, check_freq=7)
    _solve(solver)
    u_ref, it_ref, _, _ = _oracle_run(CRIT, 7, 5000)
    assert solver.converged and solver.iter == it_ref
    assert len(calls) == it_ref   # the reference evaluates the step twice per iteration
    assert calls[:3] == [0.0, DT, 2 * DT]
    np.testing.assert_array_equal(vf.fields["c"], u_ref[0].numpy())


def test_steady_state_stops_at_max_iters(cuda_lib, capsys):
    vf, solver = _solver(conv_crit=0.0, check_freq=5)
    _solve(solver, max_iters=23, verbose=True)
    assert not solver.converged and solver.iter == 23
    u_ref, _, _, checks = _oracle_run(0.0, 5, 23)
    np.testing.assert_array_equal(vf.fields["c"], u_ref[0].numpy())
    out = capsys.readouterr().out
    lines = [ln for ln in out.splitlines() if ln.startswith("Iter ")]
    assert [int(ln.split()[1].rstrip(":")) for ln in lines] == [c[0] for c in checks] == [0, 5, 10, 15, 20]
    assert lines[0].startswith("Iter 0: Field 'c' relative change: ")
    assert "Converged" not in out


def test_steady_state_rejects_bad_check_freq(cuda_lib):
    vf, solver = _solver(check_freq=0)
    with pytest.raises(ValueError):
        _solve(solver, max_iters=3)
