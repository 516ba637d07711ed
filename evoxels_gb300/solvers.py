"""Solver loop: the reference's ``TimeDependentSolver`` on the CUDA backend.

Same dataclass fields, ``solve`` keywords, frame schedule, NaN abort and
printed timing line as evoxels/solvers.py:12-208.  Between output frames the
loop hands whole runs of steps to the stepper's ``advance`` (one library call
per frame interval) when the stepper has one; a user ``step_fn`` is called
step by step exactly as in the reference.

Frame output (evoxels/solvers.py:152-187) is asynchronous by default: at a
frame the state's NaN flag is computed on the device and the state is copied
to pinned host memory on a side stream, while the next interval's steps are
already queued on the compute stream; the host then waits for the copy only,
exports the fields, applies the NaN abort with the frame's own number and
time, and writes the VTK file, all overlapped with the GPU's next interval.
``async_output=False`` restores the reference's synchronous export.
"""

from __future__ import annotations

import sys
from dataclasses import dataclass
from timeit import default_timer as timer
from typing import Any, Callable

import numpy as np
import torch

from .voxelgrid import VoxelGridGB300


class TorchMemoryProfiler:
    """Wall-time and device-memory report (evoxels/profiler.py:44-81, GPU branch)."""

    def __init__(self, device):
        self.device = device
        torch.cuda.reset_peak_memory_stats(device=device)

    def update_memory_stats(self):
        pass

    def print_memory_stats(self, start, end, iters):
        print(f"Wall time: {np.around(end - start, 4)} s after {iters} iterations "
              f"({np.around((end - start) / iters, 4)} s/iter)")
        print(f"GPU-RAM (torch)       current: "
              f"{torch.cuda.memory_allocated(self.device) / 1024**2:.2f} MB "
              f"({torch.cuda.max_memory_allocated(self.device) / 1024**2:.2f} MB max, "
              f"{torch.cuda.max_memory_reserved(self.device) / 1024**2:.2f} MB reserved)")


@dataclass
class BaseSolver:
    """Generic wrapper for solving one or more fields with a time stepper (evoxels/solvers.py:12-114)."""
    vf: Any
    fieldnames: Any
    backend: str
    problem_cls: Any = None
    timestepper_cls: Any = None
    step_fn: Callable | None = None
    device: str = "cuda"
    async_output: bool = True

    def __post_init__(self):
        if self.backend not in ("torch", "gb300"):
            raise ValueError(f"Unsupported backend: {self.backend}")
        self.vg = VoxelGridGB300(self.vf.grid_info(), precision=self.vf.precision, device=self.device)
        self.profiler = TorchMemoryProfiler(self.vg.device)
        if isinstance(self.fieldnames, str):
            self.fieldnames = [self.fieldnames]
        else:
            self.fieldnames = list(self.fieldnames)

    def _init_fields(self):
        u_list = [self.vg.init_scalar_field(self.vf.fields[name]) for name in self.fieldnames]
        u = self.vg.concatenate(u_list, 0)
        return self.vg.bc.trim_boundary_nodes(u)

    def _init_stepper(self, time_increment, problem_kwargs, jit):
        """``jit`` is accepted for signature parity; the step is compiled CUDA already."""
        problem_kwargs = problem_kwargs or {}
        self._stepper = None
        if self.step_fn is not None:
            self.problem = None
            return self.step_fn
        if self.problem_cls is None or self.timestepper_cls is None:
            raise ValueError("Either provide step_fn or both problem_cls and timestepper_cls")
        self.problem = self.problem_cls(self.vg, **problem_kwargs)
        self._stepper = self.timestepper_cls(self.problem, time_increment)
        return self._stepper.step

    def solve(self, time_increment=0.1, frames=10, max_iters=100, problem_kwargs=None, jit=True,
              verbose=True, vtk_out=False, plot_bounds=None, colormap="viridis"):
        u = self._init_fields()
        step = self._init_stepper(time_increment, problem_kwargs, jit)
        torch.cuda.synchronize(self.vg.device)
        start = timer()
        u = self._run_loop(u, step, time_increment, frames, max_iters, vtk_out, verbose, plot_bounds, colormap)
        torch.cuda.synchronize(self.vg.device)
        end = timer()
        self.computation_time = end - start
        if verbose:
            self.profiler.print_memory_stats(start, end, max_iters)

    def _export_fields(self, u_out):
        for i, name in enumerate(self.fieldnames):
            self.vf.set_field(name, self.vg.export_scalar_field_to_numpy(u_out[i:i + 1]))

    def _handle_outputs(self, u, frame, time, vtk_out, verbose, plot_bounds, colormap):
        """Export, NaN abort, optional VTK (evoxels/solvers.py:152-187; no plotting)."""
        from . import _lib
        u_out = u  # trim_ghost_nodes(pad_bc(u)) == u for cell-centred grids
        self._export_fields(u_out)
        _lib.check_device_status(f"frame {frame}")
        has_nan = any(np.isnan(self.vf.fields[name]).any() for name in self.fieldnames)
        self._frame_tail(has_nan, frame, time, vtk_out)

    def _frame_tail(self, has_nan, frame, time, vtk_out):
        if has_nan:
            print(f"NaN detected in frame {frame} at time {time}. Aborting simulation.")
            sys.exit(1)
        if vtk_out:
            cls = self.problem_cls.__name__ if self.problem_cls is not None else "step_fn"
            filename = cls + "_" + self.fieldnames[0] + f"_{frame:03d}.vtk"
            self.vf.export_to_vtk(filename=filename, field_names=self.fieldnames)

    # ---- asynchronous frames --------------------------------------------------
    def _begin_output(self, u, frame, time):
        """Queue the frame's NaN flag and host copy on the side stream; returns the pending frame."""
        from . import _lib
        dev = self.vg.device
        pipe = getattr(self, "_pipe", None)
        if pipe is None or pipe["host"].shape != u.shape:
            pipe = {"stream": torch.cuda.Stream(dev),
                    "host": torch.empty(u.shape, dtype=u.dtype).pin_memory(),
                    "flag_dev": torch.zeros(1, dtype=torch.int32, device=dev),
                    "flag_host": torch.zeros(1, dtype=torch.int32).pin_memory(),
                    "status_host": torch.zeros(1, dtype=torch.int32).pin_memory()}
            self._pipe = pipe
        st = pipe["stream"]
        st.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(st):
            _lib.check(_lib.lib().evx_nan_flag(u.data_ptr(), u.numel(), pipe["flag_dev"].data_ptr(), st.cuda_stream),
                       "evx_nan_flag")
            pipe["host"].copy_(u, non_blocking=True)
            pipe["flag_host"].copy_(pipe["flag_dev"], non_blocking=True)
            # the kernels' status word (a bounded wait that gave up) travels with the frame
            _lib.check(_lib.lib().evx_device_status_async(pipe["status_host"].data_ptr(), st.cuda_stream),
                       "evx_device_status_async")
            done = torch.cuda.Event()
            done.record(st)
        u.record_stream(st)   # the caching allocator keeps u until the copy has read it
        return (done, frame, time)

    def _finish_output(self, pending, vtk_out):
        done, frame, time = pending
        done.synchronize()
        from . import _lib
        _lib.raise_device_status(int(self._pipe["status_host"][0]), f"frame {frame}")
        host = self._pipe["host"]
        for i, name in enumerate(self.fieldnames):
            self.vf.set_field(name, host[i].numpy().copy())
        self._frame_tail(bool(self._pipe["flag_host"][0]), frame, time, vtk_out)


@dataclass
class TimeDependentSolver(BaseSolver):
    """Fixed-step time loop with ``frames`` evenly spaced exports (evoxels/solvers.py:189-208)."""

    def _run_loop(self, u, step, time_increment, frames, max_iters, vtk_out, verbose, plot_bounds, colormap):
        n_out = max_iters // frames
        frame = 0
        advance = getattr(self._stepper, "advance", None)
        pending = None
        i = 0
        while i < max_iters:
            time = i * time_increment
            if i % n_out == 0:
                if self.async_output:
                    pending = self._begin_output(u, frame, time)
                else:
                    self._handle_outputs(u, frame, time, vtk_out, verbose, plot_bounds, colormap)
                frame += 1
            if advance is not None:
                n = min(n_out - i % n_out, max_iters - i)
                u = advance(u, n, t0=time)
                i += n
            else:
                u = step(time, u)
                i += 1
            if pending is not None:   # the next steps are queued: wait for the frame's copy only
                self._finish_output(pending, vtk_out)
                pending = None
        time = max_iters * time_increment
        if self.async_output:
            self._finish_output(self._begin_output(u, frame, time), vtk_out)
        else:
            self._handle_outputs(u, frame, time, vtk_out, verbose, plot_bounds, colormap)
        return u


@dataclass
class SteadyStatePseudoTimeSolver(BaseSolver):
    """Pseudo-time iteration to a steady state (evoxels/solvers.py:210-247).

    Same fields (``conv_crit``, ``check_freq``), convergence measure
    ``||u - step(u)||_F / sqrt(Nx*Ny*Nz)`` per field, printed lines and single
    output frame as the reference.  The reference evaluates ``step(time, u)``
    twice per iteration (once for the difference, once for the update); the
    steps here are deterministic and functional, so one evaluation gives both.
    Iterations between checks run as one ``advance`` call when the stepper has
    one, and the difference norm is a device reduction (``evx_mse_grad``
    without a gradient: ``sqrt(mean(d^2))`` equals the reference's measure).

    Two deliberate differences.  The reference never advances its iteration
    counter (``self.iter`` stays 0), so it checks every iteration, passes time
    0 to every step and ignores ``max_iters``.  Here the counter advances, so
    convergence is checked every ``check_freq`` iterations and ``max_iters``
    bounds the loop; with ``check_freq=1`` and an autonomous problem the
    iterates, the stopping iteration and the output are those of the
    reference's loop.  And on the reference's torch backend the first check
    raises ``TypeError`` (``torch.sqrt`` of the Python int ``Nx*Ny*Nz``,
    evoxels/solvers.py:238-239); here the measure is computed as written.
    """
    conv_crit: float = 1e-6
    check_freq: int = 10

    def _run_loop(self, u, step, time_increment, frames, max_iters, vtk_out, verbose, plot_bounds, colormap):
        cf = int(self.check_freq)
        if cf != self.check_freq or cf < 1:
            raise ValueError("check_freq must be a positive integer")
        self.converged = False
        self.iter = 0
        advance = getattr(self._stepper, "advance", None)
        time = 0.0
        while not self.converged and self.iter < max_iters:
            time = self.iter * time_increment
            if self.iter % cf == 0:
                u_next = step(time, u)
                self.converged = self.check_convergence(u, u_next, verbose)
                u = u_next
                self.iter += 1
                continue
            n = min(cf - self.iter % cf, max_iters - self.iter)
            if advance is not None:
                u = advance(u, n, t0=self.iter * time_increment)
            else:
                for s in range(n):
                    u = step((self.iter + s) * time_increment, u)
            self.iter += n
            time = (self.iter - 1) * time_increment
        self._handle_outputs(u, 0, time, vtk_out, verbose, plot_bounds, colormap)
        return u

    def rel_changes(self, u, u_next):
        """``||u[i] - u_next[i]||_F / sqrt(Nx*Ny*Nz)`` per field, as host floats."""
        from . import _lib
        from .voxelgrid import cuda_stream
        n = u[0].numel()
        L = _lib.lib()
        need = int(L.evx_mse_scratch_bytes(n))
        sc = getattr(self, "_conv_scratch", None)
        if sc is None or sc.numel() < need or sc.device != u.device:
            sc = torch.empty(need, dtype=torch.uint8, device=u.device)
            self._conv_scratch = sc
        ms = torch.empty(u.shape[0], dtype=torch.float64, device=u.device)
        for i in range(u.shape[0]):
            _lib.check(L.evx_mse_grad(u[i].data_ptr(), u_next[i].data_ptr(), n, None, ms[i:i + 1].data_ptr(),
                                      sc.data_ptr(), sc.numel(), cuda_stream()), "evx_mse_grad")
        return [float(np.sqrt(m)) for m in ms.cpu().tolist()]

    def check_convergence(self, u, u_next, verbose):
        """Relative change of every field below ``conv_crit`` (evoxels/solvers.py:231-247)."""
        converged = True
        for name, rel_change in zip(self.fieldnames, self.rel_changes(u, u_next)):
            if rel_change > self.conv_crit:
                converged = False
            if verbose:
                print(f"Iter {self.iter}: Field '{name}' relative change: {rel_change:.2e}")
        if converged and verbose:
            print(f"Converged after {self.iter} iterations.")
        return converged
