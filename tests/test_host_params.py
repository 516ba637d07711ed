"""Host-side pieces of the drop-in on CPU: the bulk-term probe of ``mu_hom``
(evoxels/problem_definition.py:304-305 default ``18/eps*c(1-c)(1-2c)``), the float32 constants handed
to the C ABI, and ``VoxelFields``' geometry and field checks (evoxels/voxelfields.py:65-169)."""

import numpy as np
import pytest


def test_double_well_probe():
    from evoxels_gb300.problem_definition import double_well_coefficient as dw
    assert dw(None, 3.0) == 6.0 and dw(None, 1.5) == 12.0
    assert dw(lambda c, lib=None: 18 / 3.0 * c * (1 - c) * (1 - 2 * c), 1.0) == pytest.approx(6.0, rel=1e-12)
    assert dw(lambda c: 2.5 * c * (1 - c) * (1 - 2 * c), 1.0) == pytest.approx(2.5, rel=1e-12)
    with pytest.raises(NotImplementedError):
        dw(lambda c, lib=None: c ** 3 - c, 1.0)                 # not a double-well derivative
    with pytest.raises(NotImplementedError):
        dw(lambda c, lib=None: lib.log(c) - lib.log(1 - c), 1.0)   # logarithmic potential


def test_ch_params_are_float32_roundings():
    from evoxels_gb300.problem_definition import ch_params
    f = lambda x: float(np.float32(x))  # noqa: E731
    eps, D, A, dt = 1.7, 0.3, 0.25, 0.1
    p = ch_params(eps, D, A, dt)
    assert (p.D, p.kappa, p.w, p.A, p.dt) == (f(D), f(2 * eps), f(18 / eps), f(A), f(dt))
    assert p.sym_coef == f(-2 * eps * D * A)                   # the reference's python-double product
    assert ch_params(eps, D, A, dt, w=6.0).w == 6.0


def test_voxelfields_geometry_and_checks():
    from evoxels_gb300.voxelfields import VoxelFields
    vf = VoxelFields((10, 20, 40), domain_size=(1.0, 2.0, 2.0))
    assert vf.spacing == (0.1, 0.1, 0.05) and vf.origin == (0.05, 0.05, 0.025)
    g = vf.grid_info()
    assert (g.shape, g.spacing, g.origin, g.convention) == ((10, 20, 40), vf.spacing, vf.origin, "cell_center")
    st = VoxelFields((11, 4, 4), domain_size=(1.0, 1.0, 1.0), convention="staggered_x")
    assert st.spacing == (0.1, 0.25, 0.25) and st.origin == (0, 0.125, 0.125)
    with pytest.raises(ValueError, match="cell_center or staggered_x"):
        VoxelFields((4, 4, 4), convention="vertex")
    with pytest.raises(ValueError, match="three integers"):
        VoxelFields((4, 4))
    with pytest.raises(ValueError, match="three elements"):
        VoxelFields((4, 4, 4), domain_size=(1, 1))
    with pytest.raises(ValueError, match="integers or floats"):
        VoxelFields((4, 4, 4), domain_size=(1, "1", 1))
    with pytest.warns(UserWarning, match="questionable"):
        VoxelFields((4, 4, 4), domain_size=(1, 1, 100))
    vf.add_field("c")
    assert vf.fields["c"].shape == (10, 20, 40) and not vf.fields["c"].any()
    with pytest.raises(ValueError, match="shape"):
        vf.set_field("c", np.zeros((10, 20, 41)))
    with pytest.raises(TypeError):
        vf.set_field("c", [[0.0]])
    # staggered average counts the end slabs as half cells
    st.add_field("u", np.ones(st.shape))
    st.fields["u"][0] = st.fields["u"][-1] = 3.0
    assert st.average("u") == pytest.approx((9 * 16 + 0.5 * 3 * 16 * 2) / (10 * 16))


def test_voxel_sphere_is_symmetric():
    from evoxels_gb300.voxelfields import VoxelFields
    vf = VoxelFields((16, 16, 16), domain_size=(16, 16, 16))
    vf.add_field("s")
    vf.set_voxel_sphere("s", (8.0, 8.0, 8.0), 4.0)
    s = vf.fields["s"]
    assert s.sum() > 0 and np.array_equal(s, s[::-1]) and np.array_equal(s, s.transpose(1, 0, 2))


def test_checkpoint_interval_is_the_largest_that_fits():
    """``(K+1)`` segment states + ``K`` stored spectra + ``ceil(n/K)`` checkpoints within the budget."""
    import math
    from evoxels_gb300.adjoint import default_checkpoint_interval

    class VG:
        shape = (512, 512, 512)
    field = 4 * 512 ** 3
    spec = 4 * 512 * 512 * 257 * 2
    for n, budget in [(100, 16 * 2 ** 30), (100, 200 * 2 ** 30), (1000, 40 * 2 ** 30), (7, 1)]:
        K = default_checkpoint_interval(VG(), n, budget_bytes=budget, spectrum_bytes=spec)
        need = lambda k: (k + 1) * field + k * spec + math.ceil(n / k) * field  # noqa: E731
        assert 1 <= K <= n
        assert K == 1 or need(K) <= budget
        assert all(need(k) > budget for k in range(K + 1, n + 1))
    # everything fits: the whole trajectory is kept
    assert default_checkpoint_interval(VG(), 100, budget_bytes=2 ** 40, spectrum_bytes=spec) == 100


def test_ac_params_are_float32_roundings():
    """The two-phase Allen-Cahn constants (evoxels/problem_definition.py:420-447: ``potential/2/eps``
    with the default ``18/eps`` well, ``3/eps`` forcing, ``curvature`` and ``1 - curvature``)."""
    from evoxels_gb300.problem_definition import ac_params
    f = lambda x: float(np.float32(x))  # noqa: E731
    eps, gab, M, force, curv = 2.5, 0.8, 1.3, 0.2, 0.03
    p = ac_params(eps, gab, M, force, curv)
    assert (p.w, p.eps, p.gab, p.M, p.force) == (f(18 / eps), f(eps), f(gab), f(M), f(force))
    assert (p.three_over_eps, p.curvature, p.one_minus_curvature) == (f(3 / eps), f(curv), f(1 - curv))
    assert ac_params(eps, gab, M, force, curv, w=4.0).w == 4.0
