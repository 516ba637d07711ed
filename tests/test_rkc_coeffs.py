"""RKC1 / RKC2 stage coefficients (computed on the host, evoxels/timesteppers.py:202-295) against the
coefficients stored in the reference fixtures ``rkc_*``: equal to within one float32 ulp (libm's
``cosh`` / ``arccosh`` may round differently between hosts), together with the kernel-side constants
each stage hands to the C ABI."""

import numpy as np
import pytest

from conftest import load_golden


@pytest.mark.parametrize("i", range(5))
def test_rkc_coefficients_match_reference(i):
    from evoxels_gb300.timesteppers import RKC1, RKC2
    g = load_golden(f"rkc_{i}")
    skw = eval(str(g["skw"]), {"__builtins__": {}}, {})
    cls = RKC1 if str(g["scheme"]) == "RKC1" else RKC2
    st = cls(None, float(g["dt"]), **skw)
    names = ["mu0", "mu1", "mu11", "nu", "c"] + (["gamma"] if cls is RKC2 else [])
    for k in names:
        ours = np.asarray(getattr(st, k), dtype=np.float32)
        np.testing.assert_array_max_ulp(ours, g[k].astype(np.float32), maxulp=1)
    # the per-stage constants (float32 tensor products, as the reference's mu1[j]*dt)
    for j in range(st.polygrad - 1):
        c = st._stage_coeffs(j)
        assert c.mu0 == float(st.mu0[j]) and c.nu == float(st.nu[j])
        assert c.mu1_dt == float(st.mu1[j] * st.dt)
        assert c.gamma_dt == (float(st.gamma[j] * st.dt) if cls is RKC2 else 0.0)
