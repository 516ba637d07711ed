"""CPU oracle for the evoxels time-stepping hot path (test infrastructure only).

This package restates, operation by operation, the reference's torch-backend
arithmetic for the Cahn-Hilliard pseudo-spectral IMEX step (periodic and
mirrored-x), the explicit finite-difference (7-point Laplacian + ghost padding
+ forward Euler) step, and the two-phase Allen-Cahn rhs (19-point normal
Laplacian) with the classical Runge-Kutta scheme, on CPU tensors.  It is the checker the GPU kernels are compared against; it is
never the thing measured or shipped.  Only ``tests/``, ``__graft_entry__.smoke``
and the CPU-baseline / reference legs of ``bench.py`` may import it.

The restatement is pinned against outputs of the reference itself: the golden
fixtures under ``tests/golden/`` were produced by importing the reference
package and running its own ``CahnHilliard``, ``ReactionDiffusion``,
``PseudoSpectralIMEX``, ``ForwardEuler`` and ``run_cahn_hilliard_solver`` on
seeded inputs (script: ``tests/golden/make_golden.py``).
"""

from .evx_oracle import *  # noqa: F401,F403
from .evx_oracle import __all__  # noqa: F401
