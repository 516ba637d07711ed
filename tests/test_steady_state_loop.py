"""Host logic of ``SteadyStatePseudoTimeSolver._run_loop`` on CPU: the solver is built without a
grid, its stepper and difference norm replaced by CPU stand-ins computed with the oracle, and the
loop's iterates, stopping iteration, ``advance`` chunks and step times compared with the oracle's
restatement of the reference loop (evoxels/solvers.py:218-247)."""

import numpy as np
import pytest
import torch

import oracle

SHAPE = (8, 6, 5)
BC = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
DT = 0.15


def _step(v):
    return oracle.fe_step(v, DT, lambda w: oracle.rd_rhs(w, 1.0, BC))


def _solver(check_freq, use_advance, calls, outputs):
    from evoxels_gb300.solvers import SteadyStatePseudoTimeSolver
    s = object.__new__(SteadyStatePseudoTimeSolver)   # no grid: the loop alone
    s.conv_crit, s.check_freq, s.fieldnames = 1e-4, check_freq, ["c"]

    class Stepper:
        def advance(self, u, n, t0=0.0):
            calls.append(("advance", n))
            for _ in range(n):
                u = _step(u)
            return u
    s._stepper = Stepper() if use_advance else None
    s.rel_changes = lambda u, v: [float(torch.linalg.norm(u[0] - v[0]) / np.sqrt(np.prod(SHAPE)))]
    s._handle_outputs = lambda u, frame, time, *rest: outputs.append((frame, time))
    return s


def _step_fn(calls):
    def f(t, u):
        calls.append(("step", t))
        return _step(u)
    return f


@pytest.mark.parametrize("check_freq", [1, 7])
@pytest.mark.parametrize("use_advance", [True, False])
def test_loop_matches_oracle(check_freq, use_advance):
    u0 = torch.tensor(oracle.seeded_unit_field(SHAPE, 7), dtype=torch.float32).unsqueeze(0)
    calls, outputs = [], []
    s = _solver(check_freq, use_advance, calls, outputs)
    u = s._run_loop(u0, _step_fn(calls), DT, 10, 5000, False, False, None, "viridis")
    ref, it, conv, _ = oracle.steady_state_run(u0, _step, 5000, 1e-4, check_freq)
    assert s.converged == conv and s.iter == it
    assert torch.equal(u, ref)
    assert outputs == [(0, (it - 1) * DT)]
    steps = [c for c in calls if c[0] == "step"]
    adv = [c[1] for c in calls if c[0] == "advance"]
    # one step evaluation per checked iteration; the rest in advance chunks of check_freq - 1
    assert len(steps) + sum(adv) == it
    if use_advance:
        assert len(steps) == (it - 1) // check_freq + 1
        assert all(n == check_freq - 1 for n in adv)
    else:
        assert not adv and [t for _, t in steps] == [i * DT for i in range(it)]


def test_loop_stops_at_max_iters_and_rejects_bad_check_freq():
    u0 = torch.tensor(oracle.seeded_unit_field(SHAPE, 7), dtype=torch.float32).unsqueeze(0)
    calls, outputs = [], []
    s = _solver(5, True, calls, outputs)
    s.conv_crit = 0.0
    u = s._run_loop(u0, _step_fn(calls), DT, 10, 23, False, False, None, "viridis")
    ref, it, conv, _ = oracle.steady_state_run(u0, _step, 23, 0.0, 5)
    assert not s.converged and s.iter == it == 23 and torch.equal(u, ref)
    for bad in (0, -3, 2.5):
        s = _solver(bad, True, [], [])
        with pytest.raises(ValueError):
            s._run_loop(u0, _step_fn([]), DT, 10, 5, False, False, None, "viridis")
