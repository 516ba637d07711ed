"""ExponentialEuler's multiplier table ``phi1(dt*L)`` (built on the host side of the drop-in with the
reference's formula, Pade(6,6) where |z| < 0.5; evoxels/timesteppers.py:136-189) against the tables
stored in the reference fixtures ``etd1_*``, on CPU tensors."""

import numpy as np
import pytest

from conftest import load_golden
from test_oracle import etd1_case


class _Problem:
    """Just what ``ExponentialEuler.phi1`` uses: the grid's masked assignment."""

    class vg:
        @staticmethod
        def set(field, index, value):
            from evoxels_gb300.voxelgrid import VoxelGridGB300
            return VoxelGridGB300.set(None, field, index, value)


@pytest.mark.parametrize("i", range(5))
def test_phi1_table_matches_reference(i):
    from evoxels_gb300.timesteppers import ExponentialEuler
    g = load_golden(f"etd1_{i}")
    sym, _, _ = etd1_case(g)
    st = object.__new__(ExponentialEuler)
    st.problem = _Problem()
    table = st.phi1(float(g["dt"]) * sym)
    # float32 exp of this host against the fixture's: an ulp or so
    np.testing.assert_allclose(table.numpy(), g["phi1"], rtol=3e-7, atol=0)
    z = float(g["dt"]) * sym
    assert bool((z.abs() < 0.5).any())   # the Pade branch is exercised
