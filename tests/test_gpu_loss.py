"""The device loss of the inversion workload (`evx_mse_grad`): mean((u - target)^2) and its gradient
2 (u - target) / n against float64, on the 16-byte path (aligned arrays, n a multiple of 4), with a
ragged tail (n not a multiple of 4) and on the element path (arrays off 16-byte alignment)."""

import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.mark.parametrize("n,off", [(4096, 0), (1_000_003, 0), (777, 1), (256 ** 3, 0)])
@pytest.mark.parametrize("with_grad", [True, False])
def test_mse_grad_matches_fp64(cuda_lib, n, off, with_grad):
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import cuda_stream
    g = torch.Generator(device=DEV).manual_seed(n + off)
    u = torch.rand(n + off, device=DEV, generator=g)[off:]
    t = torch.rand(n + off, device=DEV, generator=g)[off:]
    lam = torch.full((n + off,), float("nan"), device=DEV)[off:] if with_grad else None
    loss = torch.empty(1, dtype=torch.float64, device=DEV)
    scratch = torch.empty(int(cuda_lib.evx_mse_scratch_bytes(n)), dtype=torch.uint8, device=DEV)
    _lib.check(cuda_lib.evx_mse_grad(u.data_ptr(), t.data_ptr(), n, lam.data_ptr() if with_grad else None,
                                     loss.data_ptr(), scratch.data_ptr(), scratch.numel(), cuda_stream()),
               "evx_mse_grad")
    d = u.double() - t.double()
    ref = float((d * d).mean())
    # float partial sums per thread (tens of terms), double across threads
    assert abs(float(loss) - ref) <= 1e-6 * ref
    if with_grad:
        # (u - t) rounds once in float32, then one product by the float32 scale
        exp = (u - t) * torch.tensor(2.0 / n, dtype=torch.float32)
        assert torch.equal(lam, exp)
