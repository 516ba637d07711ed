"""evoxels_gb300: the evoxels time-stepping hot path on NVIDIA GB300 (sm_103a).

Drop-in names for the reference's torch path: ``VoxelFields``,
``run_cahn_hilliard_solver``, ``run_allen_cahn_solver``, ``TimeDependentSolver``,
``SteadyStatePseudoTimeSolver``, ``CahnHilliard``, ``ReactionDiffusion``, ``TwoPhaseAllenCahn``,
``PseudoSpectralIMEX``, ``ForwardEuler``, ``RungeKutta4``, ``ExponentialEuler``,
``RKC1``, ``RKC2``.  All compute
runs in ``libevx.so`` (hand-written CUDA + cuFFT) through the C ABI declared in
``include/evx.h``; importing this package does not load the library, the first
compute call does, and it raises if the library is missing.
"""

from .voxelfields import Grid, VoxelFields

__all__ = [
    "VoxelFields",
    "Grid",
    "run_cahn_hilliard_solver",
    "run_allen_cahn_solver",
    "TimeDependentSolver",
    "SteadyStatePseudoTimeSolver",
    "CahnHilliard",
    "ReactionDiffusion",
    "TwoPhaseAllenCahn",
    "PseudoSpectralIMEX",
    "ForwardEuler",
    "RungeKutta4",
    "ExponentialEuler",
    "RKC1",
    "RKC2",
    "VoxelGridGB300",
]


def __getattr__(name):
    if name == "run_cahn_hilliard_solver":
        from .precompiled_solvers.cahn_hilliard import run_cahn_hilliard_solver
        return run_cahn_hilliard_solver
    if name == "run_allen_cahn_solver":
        from .precompiled_solvers.allen_cahn import run_allen_cahn_solver
        return run_allen_cahn_solver
    if name in ("TimeDependentSolver", "SteadyStatePseudoTimeSolver"):
        from . import solvers
        return getattr(solvers, name)
    if name in ("CahnHilliard", "ReactionDiffusion", "TwoPhaseAllenCahn"):
        from . import problem_definition
        return getattr(problem_definition, name)
    if name in ("PseudoSpectralIMEX", "ForwardEuler", "RungeKutta4", "ExponentialEuler", "RKC1", "RKC2"):
        from . import timesteppers
        return getattr(timesteppers, name)
    if name == "VoxelGridGB300":
        from .voxelgrid import VoxelGridGB300
        return VoxelGridGB300
    raise AttributeError(name)
