"""ctypes binding of ``libevx.so`` (the C ABI declared in ``include/evx.h``).

The library is the only compute path: if it is missing or cannot be loaded,
every entry point raises instead of falling back to anything else.
"""

from __future__ import annotations

import ctypes as C
import os
import threading

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libevx.so")

EVX_OK = 0
EVX_ERR_BAD_SHAPE = 1
EVX_ERR_BAD_ARG = 2
EVX_ERR_BAD_BC = 3
EVX_ERR_CUFFT = 4
EVX_ERR_CUDA = 5
EVX_ERR_NONFINITE = 6
EVX_ERR_TOO_LARGE = 7
EVX_ERR_WORKSPACE = 8
EVX_ERR_UNSUPPORTED = 9

BC_CODES = {"periodic": 0, "neumann": 1, "dirichlet": 2}


class EvxBC(C.Structure):
    _fields_ = [("kind", C.c_int32 * 3), ("two_v_lo", C.c_float * 3), ("two_v_hi", C.c_float * 3)]


class EvxGrid(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("reserved", C.c_int32),
                ("h", C.c_double * 3), ("inv_h", C.c_float * 3), ("inv_h2", C.c_float * 3),
                ("inv_h2_sum", C.c_float)]


EVX_BULK_DOUBLE_WELL = 0
EVX_BULK_REGULAR_SOLUTION = 1


class EvxChParams(C.Structure):
    _fields_ = [("D", C.c_float), ("kappa", C.c_float), ("w", C.c_float), ("A", C.c_float),
                ("sym_coef", C.c_float), ("dt", C.c_float), ("bulk", C.c_int32)]


class EvxAcParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("w", "eps", "gab", "M", "force", "three_over_eps", "curvature",
                                         "one_minus_curvature")]


class EvxRkcCoeffs(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("mu0", "nu", "one_minus_mu0_nu", "mu1_dt", "gamma_dt")]


class EvxBatchInstance(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("reserved", C.c_int32),
                ("h", C.c_double * 3), ("inv_h", C.c_float * 3), ("inv_h2", C.c_float * 3),
                ("inv_h2_sum", C.c_float), ("params", EvxChParams)]


class EvxBatchTuning(C.Structure):
    _fields_ = [("tile_variant", C.c_int32), ("x_chunk", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("fft_group_max", C.c_int32), ("graph_steps", C.c_int32)]


# name -> (restype, argtypes); mirrors include/evx.h
_P = C.c_void_p
_SIGS = {
    "evx_last_error": (C.c_char_p, []),
    "evx_version": (C.c_int, []),
    "evx_k2_tables_host": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _P, _P, _P]),
    "evx_rd_rhs": (C.c_int, [_P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.c_float, _P]),
    "evx_fd_forward": (C.c_int, [_P, _P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.c_float, C.c_float,
                                 C.c_int, C.c_int, _P]),
    "evx_fd_forward_noalloc": (C.c_int, [_P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.c_float, C.c_float,
                                         C.c_int, C.c_int, _P]),
    "evx_fd_adjoint": (C.c_int, [_P, _P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.c_float, C.c_float,
                                 C.c_int, _P]),
    "evx_fe_update": (C.c_int, [_P, _P, C.c_float, _P, C.c_size_t, _P]),
    "evx_ch_rhs": (C.c_int, [_P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.POINTER(EvxChParams), _P]),
    "evx_ch_plan_create": (C.c_int, [C.POINTER(_P), C.POINTER(EvxGrid), C.c_int]),
    "evx_ch_plan_create_bc": (C.c_int, [C.POINTER(_P), C.POINTER(EvxGrid), C.POINTER(EvxBC), C.c_int]),
    "evx_ch_plan_destroy": (C.c_int, [_P]),
    "evx_ch_workspace_bytes": (C.c_size_t, [_P]),
    "evx_spectral_update": (C.c_int, [_P, _P, _P, _P, _P, _P, _P]),
    "evx_ch_forward_mult": (C.c_int, [_P, _P, _P, C.c_int, _P, C.POINTER(EvxChParams), _P, _P, _P]),
    "evx_ch_mult_layout": (C.c_int, [_P]),
    "evx_ch_step": (C.c_int, [_P, _P, _P, C.POINTER(EvxChParams), _P, _P]),
    "evx_ch_forward": (C.c_int, [_P, _P, _P, C.c_int, _P, C.POINTER(EvxChParams), _P, _P, _P]),
    "evx_ch_adjoint": (C.c_int, [_P, _P, C.c_int, _P, _P, C.POINTER(EvxChParams), _P, _P, _P]),
    "evx_ch_spectrum_floats": (C.c_size_t, [_P]),
    "evx_device_status": (C.c_int, [C.c_int]),
    "evx_device_status_async": (C.c_int, [_P, _P]),
    "evx_set_wait_polls": (C.c_int, [C.c_int]),
    "evx_ac_rhs": (C.c_int, [_P, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC), C.POINTER(EvxAcParams), _P]),
    "evx_ac_rhs_stage": (C.c_int, [_P, _P, C.c_float, _P, C.POINTER(EvxGrid), C.POINTER(EvxBC),
                                   C.POINTER(EvxAcParams), _P]),
    "evx_rk4_combine": (C.c_int, [_P, _P, _P, _P, _P, C.c_float, _P, C.c_size_t, _P]),
    "evx_rkc_stage": (C.c_int, [_P, _P, _P, _P, _P, C.POINTER(EvxRkcCoeffs), _P, C.c_size_t, _P]),
    "evx_fft_yz_r2c": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P]),
    "evx_fft_yz_c2r": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P]),
    "evx_fft_z_r2c": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P]),
    "evx_fft_z_c2r": (C.c_int, [_P, _P, C.c_int, C.c_int, C.c_int, _P]),
    "evx_ch_forward_spectra": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, C.POINTER(EvxChParams), _P, _P, _P]),
    "evx_ch_adjoint_spectra": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, C.POINTER(EvxChParams), _P, _P, _P]),
    "evx_set_tile_variant": (C.c_int, [C.c_int]),
    "evx_batch_create": (C.c_int, [C.POINTER(_P), C.POINTER(EvxBatchInstance), C.c_int, C.POINTER(EvxBatchTuning),
                                   C.c_int]),
    "evx_batch_destroy": (C.c_int, [_P]),
    "evx_batch_field_floats": (C.c_size_t, [_P]),
    "evx_batch_workspace_bytes": (C.c_size_t, [_P]),
    "evx_batch_work_items": (C.c_int, [_P]),
    "evx_batch_offsets": (C.c_int, [_P, _P]),
    "evx_batch_forward": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, _P, _P]),
    "evx_batch_adjoint": (C.c_int, [_P, _P, C.c_int, _P, _P, _P, _P, _P]),
    "evx_batch_spectrum_floats": (C.c_size_t, [_P]),
    "evx_batch_forward_spectra": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, _P, _P, _P]),
    "evx_batch_adjoint_spectra": (C.c_int, [_P, _P, _P, C.c_int, _P, _P, _P, _P, _P]),
    "evx_mse_scratch_bytes": (C.c_size_t, [C.c_size_t]),
    "evx_nan_flag": (C.c_int, [_P, C.c_size_t, _P, _P]),
    "evx_mse_grad": (C.c_int, [_P, _P, C.c_size_t, _P, _P, _P, C.c_size_t, _P]),
    "evx_prof_enable": (None, [C.c_int]),
    "evx_prof_collect": (C.c_int, []),
    "evx_prof_reset": (None, []),
    "evx_prof_query": (C.c_int, [C.c_int, C.c_char_p, C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_longlong)]),
    "evx_launch_count": (C.c_ulonglong, []),
    "evx_set_graphs": (None, [C.c_int]),
    "evx_graphs_enabled": (C.c_int, []),
}

_lock = threading.Lock()
_lib = None


class EvxError(RuntimeError):
    """A non-zero status from libevx."""

    def __init__(self, code, msg):
        super().__init__(f"libevx error {code}: {msg}")
        self.code = code


def lib():
    """Load (once) and return the CDLL; raises if the library was not built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise ImportError(
                    f"{LIB_PATH} is missing: build the CUDA library first "
                    "(python -m evoxels_gb300.build, or __graft_entry__.build()).")
            d = C.CDLL(LIB_PATH)
            for name, (res, args) in _SIGS.items():
                fn = getattr(d, name)
                fn.restype = res
                fn.argtypes = args
            _lib = d
    return _lib


def exported_symbols():
    """The entry points the header declares (used by the ABI tests)."""
    return list(_SIGS)


def prof_read():
    """{slot name: (total ms, launches)} accumulated since the last reset."""
    L = lib()
    _lib_check = L.evx_prof_collect()
    if _lib_check:
        check(_lib_check, "evx_prof_collect")
    out = {}
    name = C.create_string_buffer(64)
    ms = C.c_double()
    cnt = C.c_longlong()
    i = 0
    while L.evx_prof_query(i, name, 64, C.byref(ms), C.byref(cnt)) == 0:
        out[name.value.decode()] = (ms.value, cnt.value)
        i += 1
    return out


EVX_STATUS_WAIT_GAVE_UP = 1


class DeviceWaitError(RuntimeError):
    """A bounded wait inside a kernel gave up: the results of the calls since the last check are invalid."""


def raise_device_status(status, where=""):
    """Raise ``DeviceWaitError`` for a non-zero device status word (and clear it on the device)."""
    if not status:
        return
    lib().evx_device_status(1)
    what = "a bounded wait of the x-pass on its tile loads gave up" if status & EVX_STATUS_WAIT_GAVE_UP else \
        "device status %#x" % status
    raise DeviceWaitError(f"{where + ': ' if where else ''}{what}; the results computed since the last check "
                          "are invalid")


def check_device_status(where=""):
    """Synchronous read of the device status word; raises ``DeviceWaitError`` if a kernel gave up."""
    v = lib().evx_device_status(0)
    if v < 0:
        check(EVX_ERR_CUDA, where or "evx_device_status")
    raise_device_status(v, where)


def check(code, what=""):
    """Raise the Python exception the reference raises for the same failure class."""
    if code == EVX_OK:
        return
    msg = lib().evx_last_error().decode(errors="replace")
    if what:
        msg = f"{what}: {msg}"
    if code in (EVX_ERR_BAD_SHAPE, EVX_ERR_BAD_BC):
        raise ValueError(msg)
    if code == EVX_ERR_UNSUPPORTED:
        raise NotImplementedError(msg)
    raise EvxError(code, msg)
