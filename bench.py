"""Benchmark of the evoxels time-stepping hot path on GB300.

Default workload (the headline metric): Cahn-Hilliard 256^3, fp32, periodic,
seeded c0 = 0.5 + 0.1*U[0,1) (seed 6), reference defaults eps=3, D=1, dt=0.1.
One bench step = one gradient evaluation of an inversion: 10 IMEX steps
forward (trajectory kept in HBM), the MSE loss against a seeded target and its
gradient, then 10 adjoint steps giving dL/dc0, dL/dD and dL/deps.  A
voxel-step counts one forward plus one adjoint step of one voxel.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload ch256_fwd_adj|ch100_fwd|fd512|ch512_fwd|ch512_fwd_adj|ch128_inversion|ac256_rk4|ac256_rkc2|ch256_etd1|driver256|batched64_fwd|batched64_fwd_adj]

``--impl reference`` times the CPU oracle (the operation-by-operation torch
restatement of the reference's own torch path; the reference itself is pure
Python/torch) on the host cores with all threads, on the same workload; each
step is a bounded sample (one forward + one adjoint step at the same size).

Multi-GPU (torchrun): single-grid workloads run as independent replicas, one
per rank (weak scaling, no collective on the data path); the batched workloads
shard the 64 instances over the ranks (balanced by voxel count, strong scaling,
no collective on the data path).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "voxel-steps/s fwd+adjoint CH 256³: batched/fused vs plain, same GPU, ≤1e-5 err"
FALLBACK_HBM_GBS = 6800.0

# DRAM bytes (read + write) per voxel of one launch, from the single-launch ncu
# captures summarised under profiles/ (rhs and pullback at 256^3, forward Euler
# at 512^3) of the kernels as they are now built; traffic grows in proportion to
# the voxels a launch processes.  A kernel change needs a new capture here.
NCU_DRAM_BYTES_PER_VOXEL = {
    "ch_rhs_fused": (153.186048e6 + 92.427520e6) / 256 ** 3,
    "ch_pullback_grads": (344.547840e6 + 54.629120e6) / 256 ** 3,
    "fd_step": (561.215488e6 + 497.061376e6) / 512 ** 3,
    "fd_tblock2": (554.379264e6 + 495.615488e6) / 512 ** 3,
    "ch_xpass_adj_spec": (135.312128e6 + 9.059584e6) / 256 ** 3,
    "ch_xpass_fwd_store": (67.669760e6 + 74.952704e6) / 256 ** 3,
    "ch_xpass_fwd": (135.399168e6 + 74.517248e6) / (512 * 256 * 256),
    "ch_pullback_grads_spec": (309.864192e6 + 57.453056e6) / 256 ** 3,
    "ac_rhs": (68.689152e6 + 24.427008e6) / 256 ** 3,
}


def algorithmic_bytes(slot, n, nspec):
    """Compulsory HBM bytes of one launch of each kernel slot (fp32 fields, complex64 spectra)."""
    table = {
        "ch_rhs_fused": 16 * n,     # read u_{n-1}, update; write u_n, r
        "ch_rhs": 8 * n,            # read u; write r
        "ch_axpy": 16 * n,          # read u, update; write u_out and the trajectory slot
        "ch_kspace_fwd": 16 * nspec,  # read + write the half spectrum
        "ch_kspace_adj": 24 * nspec,  # read lam_hat; write g_hat, h_hat
        "ch_xpass_fwd": 16 * nspec,   # read + write the (y,z)-transformed spectrum
        "ch_xpass_adj": 24 * nspec,   # read lam_hat; write g_hat and h_hat
        "ch_xpass_fwd_store": 24 * nspec,  # read + write the spectrum; write the stored increment spectrum
        "ch_xpass_adj_spec": 24 * nspec,   # read lam_hat and the stored spectrum; write g_hat
        "ch_pullback_grads": 24 * n,  # read u_s, g, lam, h, u_{s+1}; write lam_s
        "ch_pullback_grads_spec": 16 * n,  # read u_s, g, lam; write lam_s
        "ch_pullback": 16 * n,
        "mse_grad": 12 * n,
        "cufft_r2c": 4 * n + 8 * nspec,
        "cufft_c2r": 8 * nspec + 4 * n,
        "cufft_c2r_x2": 16 * nspec + 8 * n,
        "fft_yz_r2c": 4 * n + 8 * nspec,   # read the field, write the (y,z) half spectrum
        "fft_yz_c2r": 8 * nspec + 4 * n,
        "fft_z_r2c": 4 * n + 8 * nspec,    # read the field, write the z-transformed half spectrum
        "fft_z_c2r": 8 * nspec + 4 * n,    # read the half spectrum, write the field
        "cufft_c2c_y": 16 * nspec,         # read + write the half spectrum (library)
        "batch_cufft_c2c_y": 16 * nspec,
        "batch_rhs_fused": 16 * n,
        "batch_rhs": 8 * n,
        "batch_kspace_fwd": 16 * nspec,
        "batch_kspace_adj": 24 * nspec,
        "batch_pullback_grads": 24 * n,
        "batch_pullback": 16 * n,
        "batch_axpy": 12 * n,
        "batch_cufft_r2c": 4 * n + 8 * nspec,
        "batch_cufft_c2r": 8 * nspec + 4 * n,
        "fd_step": 8 * n,
        "fd_tblock2": 8 * n,
        "fd_tblock4": 8 * n,
        "ac_rhs": 8 * n,            # read phi, write the rhs (19-point stencil, halos from L2)
        "rk4_combine": 24 * n,      # read u, k1..k4; write u'
        "fe_update": 12 * n,        # read u, r; write u + c*r
        "rkc_stage": 20 * n,        # read u, Y_curr, Y_prev, rhs; write Y_new
        "rkc2_stage": 24 * n,       # ... and rhs_0
        "xpass_mult": 20 * nspec,   # read + write the (y,z)-transformed spectrum, read the multiplier table
        "spec_mult": 20 * nspec,
        "mirror_copy_x": 12 * n,    # read r; write its 2*nx-plane extension
        "rd_rhs": 8 * n,
    }
    return table.get(slot)


def read_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", FALLBACK_HBM_GBS)), "measured"
    return FALLBACK_HBM_GBS, "fallback"


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------

class ClockSampler:
    """Samples nvidia-smi SM clocks and throttle reasons during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_id):
        self.device_id = device_id
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device_id}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads (our arm)
# ---------------------------------------------------------------------------

class ChFwdAdj:
    """CH 256^3 (or other size) forward + adjoint gradient evaluation."""

    def __init__(self, torch, device, n=256, steps_per=10, seed=6, grads=True, shape=None):
        from evoxels_gb300.adjoint import CahnHilliardAdjoint
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        self.torch = torch
        self.shape = tuple(shape) if shape else (n, n, n)
        self.n = int(np.prod(self.shape))
        self.nspec = self.shape[0] * self.shape[1] * (self.shape[2] // 2 + 1)
        self.T = steps_per
        self.grads = grads
        vf = VoxelFields(self.shape, domain_size=self.shape)
        self.vg = VoxelGridGB300(vf.grid_info(), device=device)
        self.runner = CahnHilliardAdjoint(self.vg, dt=0.1)
        rng_c0 = 0.5 + 0.1 * np.random.default_rng(seed).random(self.shape)
        rng_t = 0.5 + 0.1 * np.random.default_rng(seed + 100).random(self.shape)
        self.c0_host = torch.tensor(rng_c0, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.t_host = torch.tensor(rng_t, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.traj = torch.empty((self.T + 1,) + self.shape, dtype=torch.float32, device=device)
        self.c0 = self.traj[0:1]          # the initial state lives in trajectory slot 0
        self.c0.copy_(self.c0_host)
        self.target = self.t_host.to(device)
        self.lam = torch.empty((1,) + self.shape, dtype=torch.float32, device=device)
        self.spectra = self.runner.new_spectra(self.T) if grads else None
        self.g_host = torch.empty((1,) + self.shape, dtype=torch.float32).pin_memory()
        self.units_per_step = self.n * self.T
        self.config = {"workload": f"ch{n}_fwd_adj", "grid": list(self.shape), "fwd_adj_steps_per_bench_step": self.T,
                       "dt": 0.1, "eps": 3.0, "D": 1.0, "A": 0.25, "bc": "periodic", "seed_c0": seed,
                       "seed_target": seed + 100, "param_grads": grads,
                       "stored_spectra": self.spectra is not None,
                       "l2": "inputs larger than L2: the kept trajectory is %.2f GB" % ((self.T + 1) * 4 * self.n / 1e9)}

    def step(self, before_loss=None):
        """Device-resident step: forward (trajectory kept), loss gradient, adjoint."""
        r = self.runner
        r.forward(self.traj[0:1], self.T, 1.0, 3.0, traj=self.traj[1:], spectra=self.spectra)
        if before_loss is not None:
            before_loss()
        loss = r.mse(self.traj[self.T:self.T + 1], self.target, self.lam)
        grads = self.torch.zeros(3, dtype=self.torch.float64, device=self.c0.device) if self.grads else None
        g0 = r.adjoint(self.traj, self.T, self.lam, 1.0, 3.0, grads, self.spectra)
        return loss, g0, grads

    def step_e2e(self):
        """Same step from host buffers: H2D of c0 and target, D2H of dL/dc0, loss and grads.  The
        target's copy runs on a side stream during the forward steps (the loss is its first use)."""
        torch = self.torch
        cur = torch.cuda.current_stream()
        if not hasattr(self, "side"):
            self.side = torch.cuda.Stream()
        self.c0.copy_(self.c0_host, non_blocking=True)
        self.side.wait_stream(cur)             # the previous step's loss has read the target
        with torch.cuda.stream(self.side):
            self.target.copy_(self.t_host, non_blocking=True)
        loss, g0, grads = self.step(before_loss=lambda: cur.wait_stream(self.side))
        self.g_host.copy_(g0, non_blocking=True)
        out = torch.cat([loss, grads]).cpu()
        return out

    def e2e_bytes(self):
        return 2 * 4 * self.n, 4 * self.n + 8 * 4

    def fp64_errors(self):
        """Error of this workload's GPU results against the FP64 oracle on the host, from the same
        float64 inputs: the state after the bench step's forward steps, and one adjoint step
        (dL/du and the step's dL/dD, dL/deps) against torch autograd through the FP64 oracle.
        ``max|gpu - fp64| / max|fp64|`` for fields, relative error for the scalars."""
        import oracle
        torch = self.torch
        torch.set_num_threads(os.cpu_count() or 1)
        dev = self.c0.device
        c0_64 = torch.tensor(0.5 + 0.1 * np.random.default_rng(self.config["seed_c0"]).random(self.shape)).unsqueeze(0)
        traj = torch.empty((self.T + 1,) + self.shape, dtype=torch.float32, device=dev)
        traj[0:1].copy_(c0_64)
        self.runner.forward(traj[0:1], self.T, 1.0, 3.0, traj=traj[1:])
        t0 = time.perf_counter()
        u64 = oracle.ch_imex_run(c0_64, self.T, 0.1)
        fwd = oracle.rel_to_max(traj[self.T].cpu().numpy(), u64[0].numpy())
        one = oracle.rel_to_max(traj[1].cpu().numpy(), oracle.ch_imex_run(c0_64, 1, 0.1)[0].numpy())
        lam64 = torch.tensor(np.random.default_rng(7).random(self.shape) - 0.5).unsqueeze(0)
        g64, dD, deps = oracle.ch_imex_vjp(c0_64, lam64, 0.1, 3.0, 1.0)
        lam = lam64.float().to(dev)
        grads = torch.zeros(3, dtype=torch.float64, device=dev)
        g = self.runner.adjoint(traj[0:2], 1, lam, 1.0, 3.0, grads)
        adj = oracle.rel_to_max(g.cpu().numpy(), g64.numpy())
        gD, geps = self.runner.param_grads(grads, 3.0)
        host_s = time.perf_counter() - t0
        del traj
        return {"forward_1_step": float("%.3g" % one), "forward_%d_steps" % self.T: float("%.3g" % fwd),
                "adjoint_1_step_dL_du": float("%.3g" % adj),
                "adjoint_1_step_dL_dD": float("%.3g" % (abs(gD - dD) / abs(dD))),
                "adjoint_1_step_dL_deps": float("%.3g" % (abs(geps - deps) / abs(deps))),
                "bar": "1e-5 per step (fields, max|err|/max|ref|)",
                "reference": "FP64 oracle (torch CPU restatement of the reference, float64) from the same "
                             "float64 c0, %.0f s on the host" % host_s}


class ChForward:
    """Plain CH forward steps (configs 1 and 5)."""

    def __init__(self, torch, device, n=100, steps_per=100, seed=1, shape=None):
        from evoxels_gb300.problem_definition import CahnHilliard
        from evoxels_gb300.timesteppers import PseudoSpectralIMEX
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        self.torch = torch
        self.shape = tuple(shape) if shape else (n, n, n)
        self.n = int(np.prod(self.shape))
        self.nspec = self.shape[0] * self.shape[1] * (self.shape[2] // 2 + 1)
        self.T = steps_per
        vf = VoxelFields(self.shape, domain_size=self.shape)
        vg = VoxelGridGB300(vf.grid_info(), device=device)
        self.st = PseudoSpectralIMEX(CahnHilliard(vg), 0.1)
        c0 = 0.5 + 0.1 * np.random.default_rng(seed).random(self.shape)
        self.c0_host = torch.tensor(c0, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.c0 = self.c0_host.to(device)
        self.out_host = torch.empty_like(self.c0_host).pin_memory()
        self.units_per_step = self.n * self.T
        self.config = {"workload": f"ch{n}_fwd", "grid": list(self.shape), "imex_steps_per_bench_step": self.T,
                       "dt": 0.1, "eps": 3.0, "D": 1.0, "bc": "periodic", "seed": seed,
                       "l2": "working set (state, update, rhs, spectrum) %s L2" %
                             ("larger than" if 16 * self.n > 129e6 else "fits in")}

    def step(self):
        return self.st.advance(self.c0, self.T)

    def step_e2e(self):
        self.c0.copy_(self.c0_host, non_blocking=True)
        u = self.step()
        self.out_host.copy_(u, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def e2e_bytes(self):
        return 4 * self.n, 4 * self.n


class AcRk4:
    """Two-phase Allen-Cahn, RungeKutta4 (run_allen_cahn_solver's scheme) or RKC2
    (polygrad 4), 256^3, Neumann BCs, reference defaults (eps 2, gab 1, M 1,
    force 0, curvature 0.01), dt 0.5."""

    def __init__(self, torch, device, n=256, steps_per=20, seed=7, shape=None, scheme="rk4"):
        from evoxels_gb300.problem_definition import TwoPhaseAllenCahn
        from evoxels_gb300.timesteppers import RKC2, RungeKutta4
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        self.torch = torch
        self.shape = tuple(shape) if shape else (n, n, n)
        self.n = int(np.prod(self.shape))
        self.nspec = 0
        self.T = steps_per
        vf = VoxelFields(self.shape, domain_size=self.shape)
        vg = VoxelGridGB300(vf.grid_info(), device=device)
        self.st = (RungeKutta4 if scheme == "rk4" else RKC2)(TwoPhaseAllenCahn(vg), 0.5)
        u0 = np.random.default_rng(seed).random(self.shape)
        self.c0_host = torch.tensor(u0, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.c0 = self.c0_host.to(device)
        self.out_host = torch.empty_like(self.c0_host).pin_memory()
        self.units_per_step = self.n * self.T
        self.config = {"workload": "ac%d_%s" % (self.shape[0], scheme), "grid": list(self.shape),
                       f"{scheme}_steps_per_bench_step": self.T,
                       "dt": 0.5, "eps": 2.0, "gab": 1.0, "M": 1.0, "force": 0.0, "curvature": 0.01,
                       "bc": "neumann x, y, z", "seed": seed,
                       "l2": "working set (state, 4 stages, stage input) larger than L2"}

    def step(self):
        u = self.c0
        for _ in range(self.T):
            u = self.st.step(0.0, u)
        return u

    def step_e2e(self):
        self.c0.copy_(self.c0_host, non_blocking=True)
        u = self.step()
        self.out_host.copy_(u, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def e2e_bytes(self):
        return 4 * self.n, 4 * self.n


class ChEtd1:
    """Cahn-Hilliard with ExponentialEuler (ETD1, Pade phi1 table), 256^3 periodic, dt 0.1,
    eps 3, D 1: ExponentialEuler.advance (evx_ch_forward_mult: per step the rhs pass with the
    previous update fused in, the (y, z) transforms, the x-pass with the table multiply, the
    inverse (y, z) transforms)."""

    def __init__(self, torch, device, n=256, steps_per=20, seed=1, shape=None):
        from evoxels_gb300.problem_definition import CahnHilliard
        from evoxels_gb300.timesteppers import ExponentialEuler
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        self.torch = torch
        self.shape = tuple(shape) if shape else (n, n, n)
        self.n = int(np.prod(self.shape))
        self.nspec = self.shape[0] * self.shape[1] * (self.shape[2] // 2 + 1)
        self.T = steps_per
        vf = VoxelFields(self.shape, domain_size=self.shape)
        vg = VoxelGridGB300(vf.grid_info(), device=device)
        self.st = ExponentialEuler(CahnHilliard(vg), 0.1)
        c0 = 0.5 + 0.1 * np.random.default_rng(seed).random(self.shape)
        self.c0_host = torch.tensor(c0, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.c0 = self.c0_host.to(device)
        self.out_host = torch.empty_like(self.c0_host).pin_memory()
        self.units_per_step = self.n * self.T
        self.config = {"workload": "ch%d_etd1" % self.shape[0], "grid": list(self.shape),
                       "etd1_steps_per_bench_step": self.T, "dt": 0.1, "eps": 3.0, "D": 1.0, "bc": "periodic",
                       "seed": seed, "l2": "working set (state, rhs, spectrum, table) larger than L2"}

    def step(self):
        return self.st.advance(self.c0, self.T)

    def step_e2e(self):
        self.c0.copy_(self.c0_host, non_blocking=True)
        u = self.step()
        self.out_host.copy_(u, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def e2e_bytes(self):
        return 4 * self.n, 4 * self.n


class Driver:
    """The drop-in driver end to end: run_cahn_hilliard_solver on a 256^3 host field with the
    reference defaults (dt 0.1, 10 frames, 100 iterations); every bench step is one solve, host
    numpy in, 11 exported host frames out (NaN checks included).  The same solve with the
    synchronous frame export is timed once for comparison."""

    def __init__(self, torch, device, n=256, steps_per=100, seed=1, shape=None):
        import evoxels_gb300 as evo
        self.torch = torch
        self.evo = evo
        self.shape = tuple(shape) if shape else (n, n, n)
        self.n = int(np.prod(self.shape))
        self.nspec = self.shape[0] * self.shape[1] * (self.shape[2] // 2 + 1)
        self.T = steps_per
        self.vf = evo.VoxelFields(self.shape, domain_size=self.shape)
        self.c0 = 0.5 + 0.1 * np.random.default_rng(seed).random(self.shape)
        self.vf.add_field("c", self.c0.copy())
        self.units_per_step = self.n * self.T
        self.config = {"workload": "driver%d" % self.shape[0], "grid": list(self.shape), "max_iters": self.T,
                       "frames": 10, "dt": 0.1, "eps": 3.0, "D": 1.0, "bc": "periodic", "seed": seed,
                       "api": "run_cahn_hilliard_solver (host numpy field in, host frames out)",
                       "l2": "working set larger than L2"}

    def _solve(self, async_output=True):
        from evoxels_gb300.problem_definition import CahnHilliard
        from evoxels_gb300.solvers import TimeDependentSolver
        from evoxels_gb300.timesteppers import PseudoSpectralIMEX
        self.vf.fields["c"] = self.c0.copy()
        solver = TimeDependentSolver(self.vf, "c", "torch", problem_cls=CahnHilliard,
                                     timestepper_cls=PseudoSpectralIMEX, async_output=async_output)
        solver.solve(time_increment=0.1, frames=10, max_iters=self.T, verbose=False, jit=False)

    def step(self):
        self.evo.run_cahn_hilliard_solver(self.vf, "c", "torch", jit=False, time_increment=0.1, frames=10,
                                          max_iters=self.T, verbose=False)

    def step_e2e(self):
        self.step()

    def e2e_bytes(self):
        return 4 * self.n, 11 * 4 * self.n

    def sync_reference(self, reps=2):
        """Seconds per solve with the synchronous frame export, and with the default one."""
        out = {}
        for mode in (False, True):
            self._solve(mode)
            t0 = time.perf_counter()
            for _ in range(reps):
                self._solve(mode)
            out[mode] = (time.perf_counter() - t0) / reps
        return out


class FdForward:
    """Explicit FD diffusion, 512^3, Dirichlet x / Neumann y,z, dt = 1/60 (config 2)."""

    def __init__(self, torch, device, n=512, steps_per=100, seed=2, spp=0):
        import warnings
        from evoxels_gb300.problem_definition import ReactionDiffusion
        from evoxels_gb300.timesteppers import ForwardEuler
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        self.torch = torch
        self.shape = (n, n, n)
        self.n = n ** 3
        self.nspec = 0
        self.T = steps_per
        vf = VoxelFields(self.shape, domain_size=self.shape)
        vg = VoxelGridGB300(vf.grid_info(), device=device)
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            prob = ReactionDiffusion(vg, D=1.0, bc=(("dirichlet", (0, 0)), "neumann", "neumann"))
        u0 = np.random.default_rng(seed).random(self.shape)
        self.c0_host = torch.tensor(u0, dtype=torch.float32).unsqueeze(0).pin_memory()
        self.c0 = self.c0_host.to(device)
        tuned = spp == 0
        if tuned:   # fastest of 1, 2, 4 steps per HBM pass on this GPU
            from evoxels_gb300.autotune import tune_fd_steps_per_pass
            spp = tune_fd_steps_per_pass(prob, 0.1 / 6, self.c0, steps=8, use_cache=False)
        self.st = ForwardEuler(prob, 0.1 / 6, steps_per_pass=spp)
        self.out_host = torch.empty_like(self.c0_host).pin_memory()
        self.units_per_step = self.n * self.T
        self.config = {"workload": f"fd{n}", "grid": list(self.shape), "fe_steps_per_bench_step": self.T,
                       "dt": 0.1 / 6, "D": 1.0, "bc": "dirichlet(0,0) x, neumann y, z", "steps_per_pass": spp,
                       "steps_per_pass_autotuned": tuned,
                       "seed": seed, "l2": "inputs larger than L2 (%.2f GB per field)" % (4 * self.n / 1e9)}

    def step(self):
        return self.st.advance(self.c0, self.T)

    def step_e2e(self):
        self.c0.copy_(self.c0_host, non_blocking=True)
        u = self.step()
        self.out_host.copy_(u, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def e2e_bytes(self):
        return 4 * self.n, 4 * self.n


class Batched:
    """64 uneven periodic CH instances (sides from {32,48,64,96,128}, seed 4), per-instance
    mobility M ~ U[0.5,2] and kappa ~ U[0.5,3] (eps = kappa/2, bulk pinned to 18/3),
    dt = 0.1; forward, or forward (trajectory and increment spectra kept) + adjoint with
    parameter gradients."""

    def __init__(self, torch, device, steps_per=50, adjoint=False, n_inst=64, autotune=True, rank=0, world=1):
        from evoxels_gb300.batched import BatchedCahnHilliard, BatchTuning
        self.torch = torch
        self.sharded = world > 1   # under torchrun each rank advances its share of the 64 instances
        rng = np.random.default_rng(4)
        sides = rng.choice([32, 48, 64, 96, 128], n_inst)
        M = rng.uniform(0.5, 2.0, n_inst)
        kappa = rng.uniform(0.5, 3.0, n_inst)
        all_shapes = [(int(a),) * 3 for a in sides]
        all_fields = [0.5 + 0.1 * np.random.default_rng([4, i]).random(s) for i, s in enumerate(all_shapes)]
        if self.sharded:
            from evoxels_gb300.partition import shard
            idx, self.shapes, M, kappa, self.fields = shard(all_shapes, rank, world, M, kappa, all_fields)
            M, kappa = np.array(M), np.array(kappa)
        else:
            idx, self.shapes, self.fields = list(range(n_inst)), all_shapes, all_fields
        self.M, self.eps = M, kappa / 2
        self.pin = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)
        tuning = BatchTuning()
        tuned = None
        if autotune:
            from evoxels_gb300 import autotune as at
            tuning = at.tune_batched(self.shapes, M, self.eps, 0.1, mu_hom=self.pin, steps=10)
            tuned = dict(tuning.__dict__)
        self.b = BatchedCahnHilliard(self.shapes, M, self.eps, 0.1, mu_hom=self.pin, tuning=tuning)
        self.T = steps_per
        self.adj = adjoint
        self.n = self.b.voxels
        self.nspec = sum(s[0] * s[1] * (s[2] // 2 + 1) for s in self.shapes)
        self.fft_plans = len(set(self.shapes)) if tuning.fft_group_max == 0 else \
            sum(-(-sum(1 for t in self.shapes if t == s) // tuning.fft_group_max) for s in set(self.shapes))
        self.u0 = self.b.pack(self.fields)
        self.u0_host = self.u0.cpu().pin_memory()
        self.out_host = torch.empty_like(self.u0_host).pin_memory()
        if adjoint:
            self.states = torch.empty((self.T + 1) * self.b.total, dtype=torch.float32, device=device)
            self.lam = torch.empty(self.b.total, dtype=torch.float32, device=device).uniform_(-1e-3, 1e-3)
            self.grads = torch.zeros((self.b.n, 3), dtype=torch.float64, device=device)
        self.units_per_step = self.n * self.T
        self.config = {"workload": "batched64_fwd_adj" if adjoint else "batched64_fwd", "instances": n_inst,
                       "shard": ("rank %d of %d: %d instances (balanced by voxel count, no collective)"
                                 % (rank, world, len(idx))) if self.sharded else "all instances on one GPU",
                       "sides": sorted(set(int(a) for a in sides)), "total_voxels": self.n,
                       "steps_per_bench_step": self.T, "dt": 0.1, "M_range": [0.5, 2.0], "kappa_range": [0.5, 3.0],
                       "bulk": "pinned 18/3", "seed": 4, "tuning": tuned or "defaults",
                       "stored_spectra": bool(adjoint),
                       "work_items": self.b.work_items,
                       "l2": "inputs larger than L2 (%.2f GB per packed field)" % (4 * self.b.total / 1e9)}

    def step(self, runner=None):
        b = runner or self.b
        if not self.adj:
            return b.forward(self.u0, self.T)
        t = b.total
        spec = getattr(b, "_bench_spectra", None)
        if spec is None:   # the stored increment spectra of the T steps (spectral parameter gradients)
            spec = b._bench_spectra = b.new_spectra(self.T)
        self.states[:t].copy_(self.u0)
        b.forward(self.states[:t], self.T, traj=self.states[t:], spectra=spec)
        self.grads.zero_()
        return b.adjoint(self.states, self.T, self.lam, self.grads, spectra=spec)

    def prof_step(self):
        """The step without CUDA graphs, so every kernel gets its own timing events."""
        if getattr(self, "b_prof", None) is None:
            from evoxels_gb300.batched import BatchedCahnHilliard, BatchTuning
            t = BatchTuning(**{k: v for k, v in self.b.tuning.__dict__.items()})
            t.graph_steps = 0
            self.b_prof = BatchedCahnHilliard(self.shapes, self.M, self.eps, 0.1, mu_hom=self.pin, tuning=t)
        return self.step(self.b_prof)

    def step_e2e(self):
        self.u0.copy_(self.u0_host, non_blocking=True)
        out = self.step()
        self.out_host.copy_(out, non_blocking=True)
        self.torch.cuda.current_stream().synchronize()

    def e2e_bytes(self):
        return 4 * self.b.total, 4 * self.b.total

    def plain(self, steps):
        """Same work through the single-grid path, one instance at a time (ms per bench step):
        PseudoSpectralIMEX.advance, or for the adjoint workload CahnHilliardAdjoint's forward with
        the trajectory (and the increment spectra where the grid has the x-pass) and its adjoint
        with the parameter gradients."""
        from evoxels_gb300.adjoint import CahnHilliardAdjoint
        from evoxels_gb300.problem_definition import CahnHilliard
        from evoxels_gb300.timesteppers import PseudoSpectralIMEX
        from evoxels_gb300.voxelfields import VoxelFields
        from evoxels_gb300.voxelgrid import VoxelGridGB300
        torch = self.torch
        dev = self.u0.device
        runs = []
        for i, s in enumerate(self.shapes):
            vg = VoxelGridGB300(VoxelFields(s, domain_size=s).grid_info(), device=dev)
            u = torch.tensor(self.fields[i], dtype=torch.float32, device=dev).unsqueeze(0)
            if not self.adj:
                st = PseudoSpectralIMEX(CahnHilliard(vg, eps=float(self.eps[i]), D=float(self.M[i]), mu_hom=self.pin),
                                        0.1)
                runs.append((st, u))
                continue
            r = CahnHilliardAdjoint(vg, 0.1, pinned_w=18 / 3.0)
            traj = torch.empty((self.T + 1,) + s, dtype=torch.float32, device=dev)
            traj[0] = u[0]
            lam = torch.empty_like(u).uniform_(-1e-3, 1e-3)
            runs.append((r, traj, r.new_spectra(self.T), lam, torch.zeros(3, dtype=torch.float64, device=dev),
                         float(self.M[i]), float(self.eps[i])))

        def one():
            if not self.adj:
                for st, u in runs:
                    st.advance(u, self.T)
                return
            for r, traj, spec, lam, g, d, e in runs:
                r.forward(traj[0:1], self.T, d, e, traj=traj[1:], spectra=spec)
                g.zero_()
                r.adjoint(traj, self.T, lam, d, e, g, spec)
        for _ in range(3):   # the third call replays the graphs the second one captured
            one()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(steps):
            one()
        b.record()
        b.synchronize()
        return a.elapsed_time(b) / steps


def batched_summary(torch, device, steps, warmup):
    """The batched forward + adjoint workload (64 uneven instances) timed as the headline one (CUDA
    events, device-resident inputs larger than L2), its plain per-grid counterpart on the same GPU, and
    the forward error of a sample of instances against the FP64 oracle."""
    import oracle
    wl = Batched(torch, device, 20, adjoint=True)
    for _ in range(warmup):
        wl.step()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        wl.step()
    b.record()
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    plain_ms = wl.plain(max(2, min(steps, 5)))
    # one forward step of a sample of instances (every side length once) against FP64
    out = wl.b.unpack(wl.b.forward(wl.u0, 1))
    errs = {}
    for side in sorted(set(s[0] for s in wl.shapes)):
        i = next(k for k, s in enumerate(wl.shapes) if s[0] == side)
        r64 = oracle.ch_imex_run(torch.tensor(wl.fields[i]).unsqueeze(0), 1, 0.1, float(wl.eps[i]), float(wl.M[i]),
                                 mu_hom=wl.pin)
        errs["instance %d (%d^3)" % (i, side)] = float("%.3g" % oracle.rel_to_max(out[i].cpu().numpy(), r64.numpy()))
    return {"workload": "batched64_fwd_adj", "value": round(wl.units_per_step / (ms / 1e3), 1),
            "unit": "voxel-steps/s", "ms_per_step": round(ms, 3), "steps": steps,
            "plain_value": round(wl.units_per_step / (plain_ms / 1e3), 1), "plain_ms_per_step": round(plain_ms, 3),
            "vs_plain": round(plain_ms / ms, 3),
            "plain_path": "single-grid CahnHilliardAdjoint forward (trajectory, increment spectra) + adjoint with "
                          "parameter gradients, one instance at a time, same GPU",
            "config": {k: wl.config[k] for k in ("instances", "sides", "total_voxels", "steps_per_bench_step",
                                                 "tuning", "l2")},
            "err_vs_fp64_forward_1_step": errs}


def make_workload(name, torch, device, inner=None, spp=0, shape=None, rank=0, world=1):
    if name == "batched64_fwd":
        return Batched(torch, device, inner or 50, adjoint=False, rank=rank, world=world)
    if name == "batched64_fwd_adj":
        return Batched(torch, device, inner or 20, adjoint=True, rank=rank, world=world)
    if name == "ch256_fwd_adj":
        return ChFwdAdj(torch, device, 256, inner or 10, 6, shape=shape)
    if name == "ch512_fwd_adj":   # large single grid: forward + adjoint with stored trajectory
        return ChFwdAdj(torch, device, 512, inner or 10, 5, shape=shape)
    if name == "ch128_inversion":
        return ChFwdAdj(torch, device, 128, inner or 200, 3, shape=shape)
    if name == "ch100_fwd":
        return ChForward(torch, device, 100, inner or 100, 1, shape=shape)
    if name == "ch512_fwd":
        return ChForward(torch, device, 512, inner or 20, 5, shape=shape)
    if name == "ac256_rk4":
        return AcRk4(torch, device, 256, inner or 20, 7, shape=shape)
    if name == "ac256_rkc2":
        return AcRk4(torch, device, 256, inner or 20, 7, shape=shape, scheme="rkc2")
    if name == "ch256_etd1":
        return ChEtd1(torch, device, 256, inner or 20, 1, shape=shape)
    if name == "driver256":
        return Driver(torch, device, 256, inner or 100, 1, shape=shape)
    if name == "fd512":
        return FdForward(torch, device, 512, inner or 100, 2, spp=spp)
    raise SystemExit(f"unknown workload {name}")


# ---------------------------------------------------------------------------
# CPU baselines (the oracle port of the reference's torch path)
# ---------------------------------------------------------------------------

def _oracle_step_fn(workload_name, torch):
    """One oracle step (fp32, torch CPU) of the 256^3 RKC2 / ETD1 workloads, and its description."""
    import oracle
    shape = (256, 256, 256)
    if workload_name == "ac256_rkc2":
        u0 = torch.tensor(oracle.seeded_unit_field(shape, 7), dtype=torch.float32).unsqueeze(0)
        k = oracle.rkc_coeffs(2, dtype=torch.float32)
        return (lambda: oracle.rkc_step(u0, 0.5, oracle.ac_rhs, k)), "256^3, 1 Allen-Cahn RKC2 step, fp32"
    u0 = torch.tensor(oracle.seeded_ch_field(shape, 1), dtype=torch.float32).unsqueeze(0)
    m = oracle.etd1_multiplier(-2 * 3.0 * 1.0 * 0.25 * oracle.rfft_k_squared(shape) ** 2, 0.1)
    return (lambda: oracle.imex_step(u0, m, oracle.ch_rhs)), "256^3, 1 Cahn-Hilliard ETD1 step, fp32"


def cpu_sample(workload_name, torch, seconds_cap=30.0):
    """Time the oracle (torch CPU, all host threads) on a bounded sample of the workload."""
    import oracle
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    if workload_name.startswith("batched"):
        rng = np.random.default_rng(4)
        sides = rng.choice([32, 48, 64, 96, 128], 64)
        kappa = (rng.uniform(0.5, 2.0, 64), rng.uniform(0.5, 3.0, 64))[1]
        adj = workload_name.endswith("adj")
        pin = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)  # noqa: E731
        fields = [torch.tensor(0.5 + 0.1 * np.random.default_rng([4, i]).random((int(a),) * 3),
                               dtype=torch.float32).unsqueeze(0) for i, a in enumerate(sides)]

        def one():
            for i, u in enumerate(fields):
                oracle.ch_imex_run(u, 1, 0.1, float(kappa[i] / 2), 1.0, mu_hom=pin)
                if adj:
                    oracle.ch_imex_vjp(u, u, 0.1, float(kappa[i] / 2), 1.0, mu_hom=pin)
        units = sum(int(a) ** 3 for a in sides)
        sample = "all 64 instances, 1 IMEX step each%s, fp32" % (" + 1 adjoint step (torch autograd)" if adj else "")
    elif workload_name in ("ch256_fwd_adj", "ch128_inversion", "ch512_fwd_adj"):
        n = {"ch256_fwd_adj": 256, "ch128_inversion": 128, "ch512_fwd_adj": 512}[workload_name]
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 6), dtype=torch.float32).unsqueeze(0)
        lam = torch.tensor(oracle.seeded_unit_field(shape, 7) - 0.5, dtype=torch.float32).unsqueeze(0)

        def one():
            oracle.ch_imex_run(u0, 1, 0.1)                   # forward step
            oracle.ch_imex_vjp(u0, lam, 0.1, 3.0, 1.0)       # adjoint step (autograd through the step)
        units = n ** 3
        sample = f"{n}^3, 1 forward IMEX step + 1 adjoint step (torch autograd), fp32"
    elif workload_name in ("ch100_fwd", "ch512_fwd"):
        n = 100 if workload_name == "ch100_fwd" else 512
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 1), dtype=torch.float32).unsqueeze(0)

        def one():
            oracle.ch_imex_run(u0, 1, 0.1)
        units = n ** 3
        sample = f"{n}^3, 1 IMEX step, fp32"
    elif workload_name == "ac256_rk4":
        n = 256
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_unit_field(shape, 7), dtype=torch.float32).unsqueeze(0)

        def one():
            oracle.ac_rk4_run(u0, 1, 0.5)
        units = n ** 3
        sample = f"{n}^3, 1 Allen-Cahn RungeKutta4 step, fp32"
    elif workload_name in ("ac256_rkc2", "ch256_etd1"):
        one, sample = _oracle_step_fn(workload_name, torch)
        units = 256 ** 3
    elif workload_name == "driver256":
        shape = (256, 256, 256)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 1), dtype=torch.float32).unsqueeze(0)

        def one():
            oracle.ch_imex_run(u0, 1, 0.1)
        units = 256 ** 3
        sample = "256^3, 1 IMEX step of the driver's loop (no frame export), fp32"
    else:
        n = 512
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_unit_field(shape, 2), dtype=torch.float32).unsqueeze(0)
        bc = (("dirichlet", (0, 0)), "neumann", "neumann")

        def one():
            oracle.rd_fe_run(u0, 1, 0.1 / 6, 1.0, bc)
        units = n ** 3
        sample = f"{n}^3, 1 forward-Euler step, fp32"
    one()  # warm-up
    reps, t0 = 0, time.perf_counter()
    while True:
        one()
        reps += 1
        el = time.perf_counter() - t0
        if el > seconds_cap / 3 or reps >= 5:
            break
    return {"value": units * reps / el, "unit": "voxel-steps/s", "cores": threads, "kind": "port",
            "sample": f"{sample}; {reps} reps after 1 warm-up, {el:.1f} s"}, el / reps, units


# ---------------------------------------------------------------------------
# main
# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ch256_fwd_adj")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="headline workload only: skip the FP64 error statement and the batched line")
    ap.add_argument("--inner-steps", type=int, default=None,
                    help="override the IMEX/FE steps per bench step (profiling runs)")
    ap.add_argument("--fd-steps-per-pass", type=int, default=0, choices=[0, 1, 2, 4],
                    help="temporal blocking of the finite-difference workload (0: autotuned)")
    ap.add_argument("--ref-device", default="cpu", choices=["cpu", "cuda"],
                    help="reference arm: the oracle port of the reference's torch path on the host cores (the "
                         "default) or on the GPU (the same-box GPU baseline of the reference's torch path)")
    ap.add_argument("--ref-compile", action="store_true",
                    help="reference arm on the GPU: the Cahn-Hilliard step under torch.compile, as the "
                         "reference's jit=True")
    ap.add_argument("--grid", default=None,
                    help="NX,NY,NZ: run a Cahn-Hilliard workload on another grid (profiling runs; "
                         "the metric then names the grid)")
    args = ap.parse_args()
    args.shape = tuple(int(v) for v in args.grid.split(",")) if args.grid else None
    if args.shape and (len(args.shape) != 3 or not args.workload.startswith("ch")):
        raise SystemExit("--grid takes NX,NY,NZ and a Cahn-Hilliard workload")
    warmup = max(3, args.warmup)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        return run_reference(args, torch, warmup)

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    device = torch.device("cuda", local_rank if world > 1 else torch.cuda.current_device())
    torch.cuda.set_device(device)

    from evoxels_gb300 import _lib
    L = _lib.lib()
    wl = make_workload(args.workload, torch, device, args.inner_steps, args.fd_steps_per_pass, args.shape,
                       rank=rank, world=world)
    sharded = getattr(wl, "sharded", False)

    for _ in range(warmup):
        wl.step()
    torch.cuda.synchronize()

    # ---- timed region (device-resident inputs) ------------------------------------
    props = torch.cuda.get_device_properties(device)
    dev_id = getattr(props, "uuid", None)
    dev_id = f"GPU-{dev_id}" if dev_id is not None else str(device.index)
    sampler = ClockSampler(dev_id)
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = L.evx_launch_count()
    ev0.record(stream)
    for _ in range(args.steps):
        wl.step()
    ev1.record(stream)
    torch.cuda.synchronize()
    launches = L.evx_launch_count() - launches0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    ms = ev0.elapsed_time(ev1)
    if dist:
        t = torch.tensor([ms], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t)
    if sharded:   # each rank advanced its own share: sum the voxel-steps over ranks
        t = torch.tensor([float(wl.units_per_step)], device=device, dtype=torch.float64)
        dist.all_reduce(t)
        units_total = float(t) * args.steps
    else:         # replicas: every rank advanced the whole workload
        units_total = wl.units_per_step * args.steps * world
    value = units_total / (ms / 1e3)

    # ---- end to end: host buffers through the public API -------------------------
    for _ in range(2):
        wl.step_e2e()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        wl.step_e2e()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    if dist:
        t = torch.tensor([e2e_s], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t)
    h2d, d2h = wl.e2e_bytes()
    e2e = {"value": units_total / e2e_s, "unit": "voxel-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h}

    # ---- per-kernel breakdown (separate pass, CUDA events on the launching stream) --
    L.evx_prof_reset()
    L.evx_prof_enable(1)
    nprof = 3
    for _ in range(nprof):
        (wl.prof_step if hasattr(wl, "prof_step") else wl.step)()
    torch.cuda.synchronize()
    L.evx_prof_enable(0)
    prof = _lib.prof_read()
    peak, peak_kind = read_peaks()
    breakdown = {}
    total_ms = sum(v[0] for v in prof.values()) or 1.0
    per_group = getattr(wl, "fft_plans", 1)   # batched FFT slots launch once per shape group
    for slot, (tms, cnt) in sorted(prof.items(), key=lambda kv: -kv[1][0]):
        b = algorithmic_bytes(slot, wl.n, wl.nspec)
        if b and slot.startswith("batch_cufft"):
            b = b / per_group
        avg = tms / max(cnt, 1)
        breakdown[slot] = {"launches": cnt // nprof, "avg_us": round(avg * 1e3, 2),
                           "share": round(tms / total_ms, 4),
                           "achieved_gbs": round(b / (avg / 1e3) / 1e9, 1) if b else None}
    # our kernels with an algorithmic byte count (not cuFFT, not whole-graph replay slots)
    ours = {k: v for k, v in prof.items()
            if not k.startswith(("cufft", "batch_cufft")) and algorithmic_bytes(k, wl.n, wl.nspec) is not None}
    dom = max(ours, key=lambda k: ours[k][0]) if ours else None
    roofline = None
    if dom:
        tms, cnt = ours[dom]
        b = algorithmic_bytes(dom, wl.n, wl.nspec)
        achieved = b / (tms / cnt / 1e3) / 1e9
        tr = NCU_DRAM_BYTES_PER_VOXEL.get(dom)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                    "unit": "GB/s", "frac": round(achieved / peak, 4), "peak_source": peak_kind,
                    "algorithmic_bytes_per_launch": b,
                    "traffic": (tr * wl.n) if tr is not None else None}
    step_bytes = None
    if args.workload.startswith("batched"):
        step_bytes = (64 if wl.adj else 32) * wl.units_per_step
    elif args.workload in ("ch256_fwd_adj", "ch128_inversion", "ch512_fwd_adj"):
        step_bytes = 64 * wl.units_per_step    # 32 B forward + 32 B adjoint per voxel-step
    elif args.workload in ("ch100_fwd", "ch512_fwd"):
        step_bytes = 32 * wl.units_per_step
    elif args.workload.startswith("fd"):
        step_bytes = 8 * wl.units_per_step
    elif args.workload == "ac256_rkc2":
        step_bytes = 116 * wl.units_per_step   # 4 x rhs 8 + first stage 12 + 3 x RKC2 stage 24
    elif args.workload.startswith("ac"):
        step_bytes = 92 * wl.units_per_step    # 4 x rhs 8 + 3 x stage input 12 + combine 24
    elif args.workload == "ch256_etd1":
        step_bytes = 42 * wl.units_per_step    # fused rhs 16, R2C 8, x-pass 10, C2R 8 (nspec ~ n/2)
    step_roofline = None
    if step_bytes:
        gbs = step_bytes * args.steps / (ms / 1e3) / 1e9
        step_roofline = {"achieved": round(gbs, 1), "peak": peak, "unit": "GB/s", "frac": round(gbs / peak, 4),
                         "bytes_per_voxel_step": step_bytes // wl.units_per_step}

    vs_plain = None
    if isinstance(wl, Batched) and not sharded:
        plain_ms = wl.plain(max(2, min(args.steps, 5)))
        vs_plain = {"plain_ms_per_step": round(plain_ms, 3), "plain_value": round(wl.units_per_step / (plain_ms / 1e3), 1),
                    "speedup": round(plain_ms / (ms / args.steps), 3),
                    "plain_path": ("single-grid CahnHilliardAdjoint forward (trajectory, increment spectra) + "
                                   "adjoint with parameter gradients per instance, same GPU" if wl.adj else
                                   "single-grid PseudoSpectralIMEX.advance per instance, same GPU")}
    if isinstance(wl, Driver):
        t = wl.sync_reference()
        vs_plain = {"sync_output_s_per_solve": round(t[False], 4), "async_output_s_per_solve": round(t[True], 4),
                    "speedup": round(t[False] / t[True], 3),
                    "plain_path": "the same solve with the synchronous frame export (async_output=False)"}
    out = {
        "metric": (METRIC if args.workload == "ch256_fwd_adj" and not args.shape
                   else f"voxel-steps/s {args.workload}" + ("@%dx%dx%d" % args.shape if args.shape else "")),
        "value": round(value, 1),
        "unit": "voxel-steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": warmup,
        "ms_per_step": round(ms / args.steps, 4),
        "higher_is_better": True,
        "scaling": "strong" if sharded else "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded U[0,1) fields, no dataset)",
        "config": dict(wl.config, parallelism=("instances sharded x%d" % world) if sharded else
                       ("replicas x%d" % world) if world > 1 else "single GPU"),
        "roofline": roofline,
        "step_roofline": step_roofline,
        "kernel_breakdown": breakdown,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "vs_plain": vs_plain,
        "clocks": clocks,
    }
    if world == 1 and args.workload == "ch256_fwd_adj" and not args.shape and not args.no_extras:
        # the metric's second half (batched uneven grids against the plain per-grid path, same GPU)
        # and the error statement of the headline run
        out["err_vs_fp64"] = wl.fp64_errors()
        del wl
        torch.cuda.empty_cache()
        out["batched"] = batched_summary(torch, device, args.steps, warmup)
    if rank == 0 and world == 1 and not args.no_cpu_baseline and not args.shape:
        cb, _, _ = cpu_sample(args.workload, torch)
        out["cpu_baseline"] = cb
    if rank == 0:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()
    return 0


def run_reference(args, torch, warmup):
    """Reference arm: the oracle port of the reference's torch path on host cores, or with
    ``--ref-device cuda`` the same torch ops on the GPU (the reference selects its device with
    ``torch.set_default_device``, evoxels/voxelgrid.py:156-189), eager or under torch.compile."""
    import oracle
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    wl = args.workload
    on_gpu = args.ref_device == "cuda"
    if args.ref_compile and not on_gpu:
        raise SystemExit("--ref-compile needs --ref-device cuda")
    if on_gpu:
        torch.set_default_device("cuda")
    if wl.startswith("batched"):
        rng = np.random.default_rng(4)
        sides = rng.choice([32, 48, 64, 96, 128], 64)
        units = sum(int(a) ** 3 for a in sides)
        kappa = (rng.uniform(0.5, 2.0, 64), rng.uniform(0.5, 3.0, 64))[1]
        pin = lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c)  # noqa: E731
        fields = [torch.tensor(0.5 + 0.1 * np.random.default_rng([4, i]).random((int(a),) * 3),
                               dtype=torch.float32).unsqueeze(0) for i, a in enumerate(sides)]
        adj = wl.endswith("adj")

        def one():
            for i, u in enumerate(fields):
                oracle.ch_imex_run(u, 1, 0.1, float(kappa[i] / 2), 1.0, mu_hom=pin)
                if adj:
                    oracle.ch_imex_vjp(u, u, 0.1, float(kappa[i] / 2), 1.0, mu_hom=pin)
        shape = (int(round(units ** (1 / 3))),) * 3
        sample = "all 64 instances, 1 IMEX step each%s per bench step, fp32" % (" + 1 adjoint step" if adj else "")
        n = round(units ** (1 / 3))
    elif wl in ("ch256_fwd_adj", "ch128_inversion", "ch512_fwd_adj"):
        n = {"ch256_fwd_adj": 256, "ch128_inversion": 128, "ch512_fwd_adj": 512}[wl]
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 6), dtype=torch.float32).unsqueeze(0)
        lam = torch.tensor(oracle.seeded_unit_field(shape, 7) - 0.5, dtype=torch.float32).unsqueeze(0)

        def one():
            u1 = oracle.ch_imex_run(u0, 1, 0.1)
            oracle.ch_imex_vjp(u0, lam, 0.1, 3.0, 1.0)
            return u1
        sample = f"{n}^3: 1 forward IMEX step + 1 adjoint step (torch autograd) per bench step, fp32"
    elif wl in ("ch100_fwd", "ch512_fwd"):
        n = 100 if wl == "ch100_fwd" else 512
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 1), dtype=torch.float32).unsqueeze(0)

        def one():
            return oracle.ch_imex_run(u0, 1, 0.1)
        sample = f"{n}^3: 1 IMEX step per bench step, fp32"
    elif wl == "ac256_rk4":
        n = 256
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_unit_field(shape, 7), dtype=torch.float32).unsqueeze(0)

        def one():
            return oracle.ac_rk4_run(u0, 1, 0.5)
        sample = f"{n}^3: 1 Allen-Cahn RungeKutta4 step per bench step, fp32"
    elif wl in ("ac256_rkc2", "ch256_etd1"):
        n = 256
        shape = (n, n, n)
        one, sample = _oracle_step_fn(wl, torch)
        sample += " per bench step"
    elif wl == "driver256":
        n = 256
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_ch_field(shape, 1), dtype=torch.float32).unsqueeze(0)

        def one():
            return oracle.ch_imex_run(u0, 1, 0.1)
        sample = f"{n}^3: 1 IMEX step of the driver's loop per bench step (no frame export), fp32"
    else:
        n = 512
        shape = (n, n, n)
        u0 = torch.tensor(oracle.seeded_unit_field(shape, 2), dtype=torch.float32).unsqueeze(0)

        def one():
            return oracle.rd_fe_run(u0, 1, 0.1 / 6, 1.0, (("dirichlet", (0, 0)), "neumann", "neumann"))
        sample = f"{n}^3: 1 forward-Euler step per bench step, fp32"
    if args.ref_compile:
        one, sample = _compiled_reference_step(torch, oracle, wl, shape, sample)
    sync = torch.cuda.synchronize if on_gpu else (lambda: None)
    for _ in range(warmup):
        one()
    sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one()
    sync()
    el = time.perf_counter() - t0
    units_ref = units if wl.startswith("batched") else n ** 3
    value = units_ref * args.steps / el
    out = {
        "metric": METRIC if wl == "ch256_fwd_adj" else f"voxel-steps/s {wl}",
        "impl": "reference",
        "value": round(value, 1),
        "unit": "voxel-steps/s",
        "n_gpus": 1,
        "steps": args.steps,
        "warmup": warmup,
        "ms_per_step": round(el / args.steps * 1e3, 3),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded U[0,1) fields, no dataset)",
        "config": {"workload": wl, "grid": "64 uneven instances" if wl.startswith("batched") else list(shape)},
        "cpu_baseline": {"value": round(value, 1), "unit": "voxel-steps/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 1), "unit": "voxel-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if on_gpu:
        out["cpu_baseline"] = None
        out["ref_device"] = "cuda"
        out["gpu_torch_baseline"] = {"value": round(value, 1), "unit": "voxel-steps/s",
                                     "mode": "torch.compile" if args.ref_compile else "eager",
                                     "device": torch.cuda.get_device_name(0), "sample": sample}
    print(json.dumps(out))
    return 0


def _compiled_reference_step(torch, oracle, wl, shape, sample):
    """The Cahn-Hilliard IMEX step of the reference's torch path under torch.compile (its jit=True):
    forward workloads step with it, forward + adjoint workloads add the VJP through it (dL/du, dL/dD,
    dL/deps) as the eager arm's ch_imex_vjp does."""
    fwd_only = wl in ("ch100_fwd", "ch512_fwd", "driver256")
    if not fwd_only and wl not in ("ch256_fwd_adj", "ch128_inversion", "ch512_fwd_adj"):
        raise SystemExit(f"--ref-compile covers the Cahn-Hilliard IMEX workloads, not {wl}")
    k2 = oracle.rfft_k_squared(shape)
    seed_u, seed_l = (1, None) if fwd_only else (6, 7)

    def step_fn(u, Dt, et):
        prefac = 0.1 / (1 - 0.1 * (-2 * et * Dt * 0.25 * k2 ** 2))
        mh = lambda c, lib=None: 18 / et * c * (1 - c) * (1 - 2 * c)  # noqa: E731
        return oracle.imex_step(u, prefac, lambda v: oracle.ch_rhs(v, et, Dt, None, (1.0, 1.0, 1.0), mh))
    cstep = torch.compile(step_fn)
    u0 = torch.tensor(oracle.seeded_ch_field(shape, seed_u), dtype=torch.float32).unsqueeze(0)
    d0, e0 = torch.tensor(1.0), torch.tensor(3.0)
    if fwd_only:
        def one():
            with torch.no_grad():
                return cstep(u0, d0, e0)
        return one, sample + " (torch.compile)"
    lam = torch.tensor(oracle.seeded_unit_field(shape, seed_l) - 0.5, dtype=torch.float32).unsqueeze(0)

    def one():
        with torch.no_grad():
            u1 = cstep(u0, d0, e0)
        u = u0.detach().clone().requires_grad_(True)
        Dt = torch.tensor(1.0, requires_grad=True)
        et = torch.tensor(3.0, requires_grad=True)
        torch.autograd.grad(cstep(u, Dt, et), (u, Dt, et), grad_outputs=lam)
        return u1
    return one, sample + " (torch.compile)"


if __name__ == "__main__":
    sys.exit(main())
