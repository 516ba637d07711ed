"""C-ABI checks that need no GPU: the library builds, loads, exports every entry
point declared in include/evx.h, and rejects bad arguments before touching a device."""

import ctypes as C
import os
import re

import numpy as np
import pytest
import torch

import oracle
from conftest import ROOT


@pytest.fixture(scope="module")
def L():
    from evoxels_gb300 import _lib, build
    build.build()
    return _lib.lib()


def header_functions():
    text = open(os.path.join(ROOT, "include", "evx.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(evx_\w+)\s*\(", text, flags=re.M)))


def test_every_declared_symbol_is_exported(L):
    from evoxels_gb300 import _lib
    names = header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/evx.h but not exported by libevx.so"
    assert set(names) == set(_lib.exported_symbols()), "ctypes signature table out of sync with the header"


def test_version(L):
    assert L.evx_version() >= 10000


@pytest.mark.parametrize("shape,spacing", [((8, 8, 8), (1.0, 1.0, 1.0)), ((100, 100, 100), (1.0, 1.0, 1.0)),
                                           ((5, 7, 9), (0.5, 0.75, 1.25)), ((12, 10, 6), (1 / 3, 0.1, 2.0))])
def test_k2_tables_bitexact_vs_reference_kgrid(L, shape, spacing):
    nx, ny, nz = shape
    kx2 = np.zeros(nx, np.float32)
    ky2 = np.zeros(ny, np.float32)
    kz2 = np.zeros(nz // 2 + 1, np.float32)
    rc = L.evx_k2_tables_host(nx, ny, nz, *spacing, kx2.ctypes.data, ky2.ctypes.data, kz2.ctypes.data)
    assert rc == 0
    k2 = (kx2[:, None, None] + ky2[None, :, None]) + kz2[None, None, :]
    ref = oracle.rfft_k_squared(shape, spacing, torch.float32).numpy()
    np.testing.assert_array_equal(k2, ref)


def test_bad_arguments_rejected_without_gpu(L):
    from evoxels_gb300 import _lib
    g = _lib.EvxGrid()
    g.nx, g.ny, g.nz = 0, 4, 4
    for a in range(3):
        g.h[a], g.inv_h[a], g.inv_h2[a] = 1.0, 1.0, 1.0
    g.inv_h2_sum = 3.0
    plan = C.c_void_p()
    assert L.evx_ch_plan_create(C.byref(plan), g, 0) == _lib.EVX_ERR_BAD_SHAPE
    assert b"positive" in L.evx_last_error()
    g.nx = 4
    bc = _lib.EvxBC()
    bc.kind[1] = 7
    assert L.evx_fd_forward(1, 2, None, g, bc, 1.0, 0.1, 1, 1, None) == _lib.EVX_ERR_BAD_BC
    bc.kind[1] = 0
    assert L.evx_fd_forward(None, 2, None, g, bc, 1.0, 0.1, 1, 1, None) == _lib.EVX_ERR_BAD_ARG
    assert L.evx_fd_forward(1, 1, None, g, bc, 1.0, 0.1, 1, 1, None) == _lib.EVX_ERR_BAD_ARG
    assert L.evx_fd_forward(1, 2, None, g, bc, 1.0, 0.1, 3, 3, None) == _lib.EVX_ERR_BAD_ARG
    assert L.evx_fd_forward(1, 2, None, g, bc, 1.0, 0.1, 3, 1, None) == _lib.EVX_ERR_WORKSPACE
    big = _lib.EvxGrid()
    big.nx = big.ny = big.nz = 2048
    for a in range(3):
        big.h[a], big.inv_h[a], big.inv_h2[a] = 1.0, 1.0, 1.0
    assert L.evx_ch_plan_create(C.byref(plan), big, 0) == _lib.EVX_ERR_TOO_LARGE
    p = _lib.EvxChParams()
    p.D = float("nan")
    assert L.evx_ch_rhs(1, 2, g, None, p, None) == _lib.EVX_ERR_BAD_ARG


def test_status_mapping_matches_reference_exceptions(L):
    from evoxels_gb300 import _lib
    with pytest.raises(ValueError):
        _lib.check(_lib.EVX_ERR_BAD_SHAPE)
    with pytest.raises(ValueError):
        _lib.check(_lib.EVX_ERR_BAD_BC)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.EVX_ERR_UNSUPPORTED)
    with pytest.raises(_lib.EvxError):
        _lib.check(_lib.EVX_ERR_CUFFT)
