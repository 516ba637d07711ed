"""Frame output of the solver loop (evoxels/solvers.py:152-208): the asynchronous
path (device NaN flag, pinned host copy on a side stream, overlapped with the
next interval) exports the same fields, writes the same VTK files and aborts
at the same frame as the reference's synchronous export; the NaN flag kernel."""

import os

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _solve(async_output, shape=(32, 24, 20), frames=4, iters=12, vtk_dir=None, step_fn=None):
    import evoxels_gb300 as evo
    from evoxels_gb300.problem_definition import CahnHilliard
    from evoxels_gb300.solvers import TimeDependentSolver
    from evoxels_gb300.timesteppers import PseudoSpectralIMEX
    vf = evo.VoxelFields(shape, domain_size=shape)
    vf.add_field("c", oracle.seeded_ch_field(shape, 5))
    seen = []
    orig = vf.set_field

    def record(name, arr):
        seen.append(arr.copy())
        orig(name, arr)
    vf.set_field = record
    kw = dict(step_fn=step_fn) if step_fn else dict(problem_cls=CahnHilliard, timestepper_cls=PseudoSpectralIMEX)
    solver = TimeDependentSolver(vf, "c", "torch", async_output=async_output, **kw)
    cwd = os.getcwd()
    if vtk_dir:
        os.chdir(vtk_dir)
    try:
        solver.solve(time_increment=0.1, frames=frames, max_iters=iters, vtk_out=bool(vtk_dir), verbose=False)
    finally:
        os.chdir(cwd)
    return seen, vf


def test_async_frames_equal_sync_frames(cuda_lib, tmp_path):
    a_dir, s_dir = tmp_path / "a", tmp_path / "s"
    a_dir.mkdir()
    s_dir.mkdir()
    fa, vfa = _solve(True, vtk_dir=str(a_dir))
    fs, vfs = _solve(False, vtk_dir=str(s_dir))
    assert len(fa) == len(fs) == 5   # frames 0..3 and the final state
    for x, y in zip(fa, fs):
        assert x.dtype == y.dtype == np.float32
        np.testing.assert_array_equal(x, y)
    np.testing.assert_array_equal(vfa.fields["c"], vfs.fields["c"])
    names = sorted(os.listdir(a_dir))
    assert names == sorted(os.listdir(s_dir)) and len(names) == 5
    for n in names:
        assert (a_dir / n).read_bytes() == (s_dir / n).read_bytes()
    # the final state is the same as the stepper's own run
    ref = oracle.ch_imex_run(torch.tensor(oracle.seeded_ch_field((32, 24, 20), 5)).unsqueeze(0), 12, 0.1).numpy()[0]
    assert oracle.rel_to_max(vfa.fields["c"], ref) < 2e-5


@pytest.mark.parametrize("async_output", [True, False])
def test_nan_abort_frame_and_time_match(cuda_lib, capsys, async_output):
    """A NaN that appears mid-run aborts at the first frame that holds it, in both paths."""
    def step_fn(t, u):   # the state turns NaN from the step taken at t = 0.5 on
        return u + (float("nan") if t >= 0.45 else 0.0)
    with pytest.raises(SystemExit) as e:
        _solve(async_output, frames=4, iters=12, step_fn=step_fn)
    assert e.value.code == 1
    out = capsys.readouterr().out
    assert "NaN detected in frame 2 at time 0.6000000000000001. Aborting simulation." in out


def test_nan_flag_kernel(cuda_lib):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    flag = torch.full((1,), 7, dtype=torch.int32, device=DEV)
    for n, pos, val, expect in [(1 << 20, None, None, 0), (1 << 20 | 3, (1 << 20) + 2, float("nan"), 1),
                                (4097, 5, float("inf"), 0), (4097, 0, float("-nan"), 1), (0, None, None, 0)]:
        x = torch.rand(n + 1, device=DEV)
        if pos is not None:
            x[pos + 1] = val
        # offset by one float: the unaligned (scalar) path; the aligned one below
        _lib.check(cuda_lib.evx_nan_flag(x[1:].data_ptr(), n, flag.data_ptr(), cuda_stream()), "evx_nan_flag")
        assert int(flag) == expect, (n, pos, val)
        y = x[1:].clone()
        _lib.check(cuda_lib.evx_nan_flag(y.data_ptr(), n, flag.data_ptr(), cuda_stream()), "evx_nan_flag")
        assert int(flag) == expect, (n, pos, val)
