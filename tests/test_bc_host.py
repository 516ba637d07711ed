"""Boundary-condition host logic on CPU: normalisation and its errors against the oracle's restatement
of evoxels/problem_definition.py:60-103, the FFT-timestepper check of :138-167 (error types and
messages), and the C-ABI encoding of the normalised spec (kind codes, Dirichlet 2v in float32)."""

import warnings

import numpy as np
import pytest

import oracle

SPECS = [
    None, "fully_periodic",
    ("periodic", "periodic", "periodic"),
    ("neumann", "periodic", "neumann"),
    (("dirichlet", (0.0, 0.0)), "neumann", "neumann"),
    (("dirichlet", (10.0, 20.0)), "neumann", "periodic"),
    ("periodic", ("dirichlet", (0.1, 0.3)), ("neumann", None)),
    (("periodic", None), ("neumann", None), ("periodic", None)),
    # malformed
    ("periodic", "periodic"),
    ("dirichlet", "periodic", "periodic"),
    ("robin", "periodic", "periodic"),
    (("dirichlet", (1.0,)), "periodic", "periodic"),
    (("dirichlet", None), "periodic", "periodic"),
    (("neumann", (1.0, 2.0)), "periodic", "periodic"),
    (("robin", None), "periodic", "periodic"),
    (("dirichlet", (0.0, 1.0), "extra"), "periodic", "periodic"),
]


def _outcome(fn, spec):
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            return ("ok", fn(spec))
    except Exception as e:  # noqa: BLE001 - the type and message are what is compared
        return (type(e).__name__, str(e))


@pytest.mark.parametrize("spec", SPECS, ids=[repr(s) for s in SPECS])
def test_normalize_bc_matches_oracle(spec):
    from evoxels_gb300.voxelgrid import normalize_bc
    assert _outcome(normalize_bc, spec) == _outcome(oracle.normalize_bc, spec)


def test_dirichlet_on_cell_centres_warns():
    from evoxels_gb300.voxelgrid import normalize_bc
    with pytest.warns(UserWarning, match="order of convergence to 0.5"):
        normalize_bc((("dirichlet", (0.0, 1.0)), "periodic", "periodic"))


class _FakeBCs:
    pad_fft_periodic = pad_fft_dirichlet_periodic = pad_fft_zero_flux_periodic = staticmethod(lambda u: u)


class _FakeGrid:
    convention = "cell_center"
    bc = _FakeBCs()


@pytest.mark.parametrize("spec,err", [
    (None, None),
    (("neumann", "periodic", "periodic"), None),
    ((("dirichlet", (0.0, 1.0)), "periodic", "periodic"), None),
    (("neumann", "neumann", "periodic"), ("ValueError", "at most one non-periodic axis")),
    (("periodic", "neumann", "periodic"), ("NotImplementedError", "only implement the single non-periodic axis")),
    (("periodic", "periodic", ("dirichlet", (0.0, 0.0))), ("NotImplementedError", "case for x")),
])
def test_fft_bc_check_matches_reference(spec, err):
    from evoxels_gb300.problem_definition import _BCMixin
    p = object.__new__(_BCMixin)
    p.vg, p.bc = _FakeGrid(), spec
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        p.initialize_boundary_conditions()
    if err is None:
        p.verify_fft_bc_config()
        return
    with pytest.raises(Exception) as e:
        p.verify_fft_bc_config()
    assert type(e.value).__name__ == err[0] and err[1] in str(e.value)


def test_bc_encoding_for_the_c_abi():
    from evoxels_gb300 import _lib
    from evoxels_gb300.voxelgrid import evx_bc, normalize_bc
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        s = evx_bc(normalize_bc((("dirichlet", (0.1, -2.5)), "neumann", "periodic")))
    assert list(s.kind) == [_lib.BC_CODES["dirichlet"], _lib.BC_CODES["neumann"], _lib.BC_CODES["periodic"]]
    assert s.two_v_lo[0] == float(np.float32(0.2)) and s.two_v_hi[0] == -5.0
    assert s.two_v_lo[1] == s.two_v_hi[1] == 0.0
