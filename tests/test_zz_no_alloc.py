"""The allocation-free forward-Euler entry point against the regular one.

``evx_fd_forward_noalloc`` is for callers that cannot let a library allocate
device memory (their device memory comes from their own pre-reserved pool, or
their buffers come from a foreign allocator).  It keeps its ping-pong scratch
in a built-in device array instead of a caller-provided field.  Here it is
called through the C ABI, twice in a row on different inputs, and must give
the same bits as ``evx_fd_forward`` with caller scratch (the finite-difference
path is bit-exact across implementations), and reject grids larger than the
built-in array.  This file is collected last on purpose.
"""

import ctypes as C
import warnings

import numpy as np
import pytest
import torch

import oracle

pytestmark = pytest.mark.gpu


def _setup(shape, bc):
    from evoxels_gb300.problem_definition import ReactionDiffusion
    from evoxels_gb300.voxelfields import VoxelFields
    from evoxels_gb300.voxelgrid import VoxelGridGB300
    vf = VoxelFields(shape, domain_size=shape)
    vg = VoxelGridGB300(vf.grid_info(), device="cuda")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        prob = ReactionDiffusion(vg, D=1.0, bc=bc)
    return vg, prob


@pytest.mark.parametrize("shape,spp", [((40, 36, 64), 2), ((33, 17, 9), 1)])
def test_noalloc_matches_regular_entry_point_twice(cuda_lib, shape, spp):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    L = cuda_lib
    bc = (("dirichlet", (0.0, 0.0)), "neumann", "neumann")
    vg, prob = _setup(shape, bc)
    g = vg.evx_grid()
    dt = float(np.float32(1.0 / 60))
    nsteps = 7   # several passes, so the scratch field is used
    for seed in (1, 2):   # two calls in a row; the built-in array keeps the previous contents
        u0 = torch.tensor(oracle.seeded_unit_field(shape, seed), dtype=torch.float32, device="cuda")
        ref = torch.empty_like(u0)
        scratch = torch.empty_like(u0)
        _lib.check(L.evx_fd_forward(u0.data_ptr(), ref.data_ptr(), scratch.data_ptr(), g, prob._evx_bc, 1.0, dt,
                                    nsteps, spp, cuda_stream()), "evx_fd_forward")
        out = torch.full_like(u0, float("nan"))
        _lib.check(L.evx_fd_forward_noalloc(u0.data_ptr(), out.data_ptr(), g, prob._evx_bc, 1.0, dt, nsteps, spp,
                                            cuda_stream()), "evx_fd_forward_noalloc")
        torch.cuda.synchronize()
        torch.testing.assert_close(out, ref, rtol=0, atol=0)


def test_noalloc_rejects_grids_beyond_the_builtin_scratch(cuda_lib):
    from evoxels_gb300 import _lib
    L = cuda_lib
    g = _lib.EvxGrid()
    g.nx, g.ny, g.nz = 256, 256, 128   # 2^23 voxels > 2^22
    for a in range(3):
        g.h[a], g.inv_h[a], g.inv_h2[a] = 1.0, 1.0, 1.0
    g.inv_h2_sum = 3.0
    rc = L.evx_fd_forward_noalloc(C.c_void_p(256), C.c_void_p(512), g, None, 1.0, 0.01, 3, 1, None)
    assert rc == _lib.EVX_ERR_TOO_LARGE
    assert b"exceeds" in L.evx_last_error()
