"""ctypes binding of libkpm (declared in include/kpm.h).

The library is the only compute path of this package: if it is missing or
does not load, every operation raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

KPM_OK = 0
KPM_ERR_INVALID_ARG = 1
KPM_ERR_SHAPE = 2
KPM_ERR_DTYPE = 3
KPM_ERR_OOM = 4
KPM_ERR_CUDA = 5
KPM_ERR_TIMEOUT = 6
KPM_ERR_INDEX = 7
KPM_ERR_UNSUPPORTED = 8
KPM_ERR_NONFINITE = 9
KPM_ERR_TOO_LARGE = 10

KPM_C128 = 0
KPM_C64 = 1
KPM_C128F = 2  # complex128 accuracy in float-float arithmetic (moments only)

KPM_FLAG_DEVICE_PTRS = 1
KPM_FLAG_SPLIT_DIAG = 2
KPM_FLAG_DOUBLING = 4
KPM_FLAG_COMPLEX = 8

DTYPES = {"c128": KPM_C128, "complex128": KPM_C128, "c64": KPM_C64, "complex64": KPM_C64, "c128f": KPM_C128F}

# Every symbol include/kpm.h declares, with (restype, argtypes).
_P = ctypes.c_void_p
_I = ctypes.c_int
_I64 = ctypes.c_int64
_D = ctypes.c_double
_U = ctypes.c_uint
SIGNATURES = {
    "kpm_strerror": (ctypes.c_char_p, [_I]),
    "kpm_version": (_I, []),
    "kpm_ell_create": (_I, [ctypes.POINTER(_P), _I64, _I, _P, _P, _U, _P]),
    "kpm_ell_destroy": (_I, [_P]),
    "kpm_ell_info": (_I, [_P, ctypes.POINTER(_I64), ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I64)]),
    "kpm_ell_reserve": (_I, [_P, _I, _I, _I]),
    "kpm_ell_check": (_I, [_P, _P]),
    "kpm_ell_step_config": (_I, [_P, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                 ctypes.POINTER(ctypes.c_float)]),
    "kpm_ell_series_config": (_I, [_P, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                   ctypes.POINTER(ctypes.c_float)]),
    "kpm_ell_dot": (_I, [_P, _D, _D, _D, _D, _P, _P, _I, _P]),
    "kpm_cheb_moments": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P]),
    "kpm_cheb_series": (_I, [_P, _I, _I, _I, _P, _P, _P, _P]),
    "kpm_time_evolve": (_I, [_P, _I, _I, _I, _P, _I, _P, _P, _P]),
    "kpm_cheb_commutator_series": (_I, [_P, _P, _I, _I, _I, _P, _P, _P, _P]),
    "kpm_cheb_commutator_table": (_I, [_P, _P, _I, _I, _I, _P, _P, _P, _P]),
    "kpm_time_sigma": (_I, [_P, _P, _P, _I, _I, _P, _I, _P, _I, _I, _P, _P, _P]),
    "rec_A_tab": (None, [_P, _P, _I, _I, _P, _P, _I]),
    "kpm_host_cache_release": (_I, []),
    "rec_A_tab_2": (None, [_P, _P, _I, _I, _P, _P, _P, _I]),
    "for_time": (None, [_P, _P, _I, _I, _P, _I, _P, _P, _I]),
    "for_time_sigma": (None, [_P, _P, _P, _P, _I, _I, _P, _P, _I, _P, _P, _I, _I]),
    "kpm_last_status": (_I, []),
    "kpm_ell_set_values": (_I, [_P, _P, _U, _P]),
    "kpm_adjoint_forward": (_I, [_P, _I, _I, _I, _P, _P, _P]),
    "kpm_adjoint_backward": (_I, [_P, _P, _P, _P]),
    "kpm_cheb_moments_noalloc": (_I, [_P, _P, _I, _I64, _P, _I, _P, _P]),
    "kpm_cheb_table": (_I, [_P, _P, _I, _P, _P, _P, _P]),
    "kpm_cheb_clenshaw_table": (_I, [_P, _P, _I, _P, _P, _P]),
    "kpm_ell_slot_sum": (_I, [_P, _I, _P, _P, _I64, _P, _I64, _I, _P, _P]),
    "kpm_mu_nm": (_I, [_P, _P, _I, _I, _P, _P, _P]),
    "kpm_mu_contract": (_I, [_P, _P, _I64, _I64, _I, _D, _I, _P, _P]),
    "kpm_batch_create": (_I, [ctypes.POINTER(_P), _I, _P, _I, _P, _P, _P]),
    "kpm_batch_destroy": (_I, [_P]),
    "kpm_batch_info": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I64), ctypes.POINTER(_I64), ctypes.POINTER(_I)]),
    "kpm_batch_moments": (_I, [_P, _I, _I, _I, _P, _P, _P]),
    "kpm_ell_props": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "kpm_ell_set_doubling": (_I, [_P, _I]),
    "kpm_adjoint_backward_ex": (_I, [_P, _P, _P, _I, _P]),
    "kpm_batch_props": (_I, [_P, ctypes.POINTER(_I), ctypes.POINTER(_I)]),
    "kpm_batch_set_doubling": (_I, [_P, _I]),
    "kpm_csr_row_max": (_I, [_I64, _P, ctypes.POINTER(_I), _P]),
    "kpm_csr_to_ell": (_I, [_I64, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "kpm_honeycomb_ell": (_I, [_I, _I, _I, _D, _P, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "kpm_ell_gershgorin_partner": (_I, [_I64, _I, _P, _P, _P, _D, ctypes.POINTER(_D), _P]),
    "kpm_ell_scale_values": (_I, [_I64, _D, _P, _P]),
    "kpm_light_modifier": (_I, [_I64, _P, _P, _P, _P, _P, _P]),
    "kpm_ell_light_update": (_I, [_P, _P, _P, _P, _P, _P]),
    "kpm_phonon_modifier": (_I, [_I64, _I, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "kpm_batch_step_config": (_I, [_P, _I, _I, ctypes.POINTER(_I), ctypes.POINTER(_I), ctypes.POINTER(_I),
                                   ctypes.POINTER(ctypes.c_float), _P]),
    "kpm_batch_check": (_I, [_P, _P]),
    "kpm_ell_test_timeout": (_I, [_P, _I64, _P]),
    "kpm_ell_profile": (_I, [_P, _I]),
    "kpm_ell_profile_read": (_I, [_P, ctypes.POINTER(_D), ctypes.POINTER(_I64), ctypes.POINTER(_I64)]),
    "kpm_measure_fp64_fma_rate": (_I, [ctypes.POINTER(_D), _P]),
    "kpm_mu_gemm_path": (_I, []),
}

_lock = threading.Lock()
_lib = None


class KPMError(RuntimeError):
    """A libkpm call returned a non-zero status."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = _strerror(status)
        super().__init__("%s: %s (status %d)" % (what or "libkpm", msg, status))


def _strerror(status: int) -> str:
    try:
        return lib().kpm_strerror(status).decode()
    except Exception:  # pragma: no cover - library missing
        return "status %d" % status


def library_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    """Load libkpm; raise if it is not built (or build it when asked)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = library_path()
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(
                    "libkpm is not built (%s missing); run `python -c \"import __graft_entry__ as g; g.build()\"` "
                    "or minijclsquant_gb300._build.build()" % path)
        cdll = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(cdll, name)
            fn.restype = res
            fn.argtypes = args
        _lib = cdll
        return _lib


def lib() -> ctypes.CDLL:
    return load(build_if_missing=False)


def check(status: int, what: str = "") -> None:
    if status != KPM_OK:
        raise KPMError(status, what)


def dtype_code(dtype) -> int:
    if isinstance(dtype, int):
        if dtype in (KPM_C128, KPM_C64, KPM_C128F):
            return dtype
    elif str(dtype) in DTYPES:
        return DTYPES[str(dtype)]
    elif str(dtype).replace("torch.", "") in DTYPES:
        return DTYPES[str(dtype).replace("torch.", "")]
    raise ValueError("unknown KPM dtype %r (use 'c128', 'c64' or 'c128f')" % (dtype,))
