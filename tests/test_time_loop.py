"""Host logic of ``TimeDependentSolver._run_loop`` on CPU (synchronous export): the frames, their
numbers and times, the states exported and the final state equal a direct restatement of the
reference loop (evoxels/solvers.py:193-208), with a user ``step_fn`` called step by step and a
stepper's ``advance`` handed whole frame intervals."""

import pytest
import torch

import oracle

SHAPE = (6, 5, 4)
DT = 0.1


def _step(v):
    return oracle.fe_step(v, 0.05, lambda w: oracle.rd_rhs(w, 1.0, None))


def _reference_loop(u, max_iters, frames):
    """The reference's loop: export at i % (max_iters // frames) == 0, step, final export."""
    n_out = max_iters // frames
    out, frame = [], 0
    for i in range(max_iters):
        if i % n_out == 0:
            out.append((frame, i * DT, u))
            frame += 1
        u = _step(u)
    out.append((frame, max_iters * DT, u))
    return u, out


def _solver(use_advance, calls, outputs):
    from evoxels_gb300.solvers import TimeDependentSolver
    s = object.__new__(TimeDependentSolver)      # no grid: the loop alone
    s.async_output = False

    class Stepper:
        def advance(self, u, n, t0=0.0):
            calls.append(("advance", n, t0))
            for _ in range(n):
                u = _step(u)
            return u
    s._stepper = Stepper() if use_advance else None
    s._handle_outputs = lambda u, frame, time, *rest: outputs.append((frame, time, u))
    return s


@pytest.mark.parametrize("max_iters,frames", [(20, 4), (23, 4), (10, 10), (7, 3), (5, 1)])
@pytest.mark.parametrize("use_advance", [True, False])
def test_frames_match_reference_loop(max_iters, frames, use_advance):
    u0 = torch.tensor(oracle.seeded_unit_field(SHAPE, 3), dtype=torch.float32).unsqueeze(0)
    calls, outputs = [], []

    def step_fn(t, u):
        calls.append(("step", t))
        return _step(u)
    u = _solver(use_advance, calls, outputs)._run_loop(u0, step_fn, DT, frames, max_iters, False, False, None,
                                                        "viridis")
    ref, ref_out = _reference_loop(u0, max_iters, frames)
    assert torch.equal(u, ref)
    assert [(f, t) for f, t, _ in outputs] == [(f, t) for f, t, _ in ref_out]
    assert all(torch.equal(a, b) for (_, _, a), (_, _, b) in zip(outputs, ref_out))
    n_out = max_iters // frames
    if use_advance:   # one library call per frame interval, the last one cut at max_iters
        assert [n for _, n, _ in calls] == [min(n_out, max_iters - i) for i in range(0, max_iters, n_out)]
        assert [t0 for _, _, t0 in calls] == [i * DT for i in range(0, max_iters, n_out)]
    else:
        assert [t for _, t in calls] == [i * DT for i in range(max_iters)]


def test_more_frames_than_iterations_fails_like_the_reference():
    u0 = torch.zeros((1,) + SHAPE)
    with pytest.raises(ZeroDivisionError):
        _reference_loop(u0, 3, 5)
    with pytest.raises(ZeroDivisionError):
        _solver(True, [], [])._run_loop(u0, lambda t, u: u, DT, 5, 3, False, False, None, "viridis")
