"""ctypes binding of libpm_gb300.so (declarations in include/pm_gb300.h)."""
from __future__ import annotations

import ctypes
import os

from .build import LIB

c_int, c_ll, c_double, c_void_p, c_size_t = (ctypes.c_int, ctypes.c_longlong, ctypes.c_double,
                                              ctypes.c_void_p, ctypes.c_size_t)
c_char_p = ctypes.c_char_p
P_int = ctypes.POINTER(ctypes.c_int)
P_double = ctypes.POINTER(ctypes.c_double)

PM_OK, PM_ERR_ARG, PM_ERR_CUDA, PM_ERR_OOM, PM_ERR_DEVICE, PM_ERR_ADMIT = range(6)
PM_FLAG_FIX_COSMO_F = 1
PM_FLAG_KEEP_DENSITY = 2
PM_FLAG_SPECTRAL_GRADIENT = 4
DEVICE_BITS = {1: "cell out of range / non-finite position", 2: "particle outside its deposit tile",
               4: "non-finite kick/drift result"}


class PMConfigC(ctypes.Structure):
    _fields_ = [("n_cells", c_int), ("n_parts", c_int), ("box_size", c_double), ("omega_m0", c_double),
                ("omega_b0", c_double), ("omega_k0", c_double), ("omega_lambda0", c_double),
                ("h0", c_double), ("a_init", c_double), ("a_end", c_double), ("steps", c_int),
                ("flags", c_int)]


class PMICParamsC(ctypes.Structure):
    _fields_ = [("power", c_double), ("lcdm_transfer", c_int), ("jitter_state", ctypes.c_ulonglong * 2),
                ("jitter_inc", ctypes.c_ulonglong * 2)]


# name -> (restype, argtypes)
SIGNATURES = {
    "pm_ctx_create": (c_int, [ctypes.POINTER(PMConfigC), c_int, ctypes.POINTER(c_void_p)]),
    "pm_ctx_destroy": (None, [c_void_p]),
    "pm_last_error": (c_char_p, [c_void_p]),
    "pm_check_device": (c_int, [c_void_p, c_void_p, P_int]),
    "pm_supported_n": (c_int, [c_int]),
    "pm_density": (c_int, [c_void_p, c_void_p, c_ll, c_double, c_void_p, c_void_p]),
    "pm_fourier_grid": (c_int, [c_void_p, c_void_p, c_void_p]),
    "pm_potential": (c_int, [c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p]),
    "pm_integrate": (c_int, [c_void_p, c_void_p, c_void_p, c_ll, c_double, c_double, c_double, c_void_p,
                             c_void_p]),
    "pm_advance_time": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_ll, c_void_p, c_double, c_double,
                                c_void_p]),
    "pm_step": (c_int, [c_void_p, c_void_p, c_void_p, c_ll, c_double, c_double, c_double, c_void_p,
                        c_void_p]),
    "pm_step_host": (c_int, [c_void_p, c_void_p, c_void_p, c_ll, c_double, c_double, c_double, c_void_p]),
    "pm_cosmo_f": (c_double, [c_double, c_double, c_double, c_double]),
    "pm_sort_keys": (c_int, [c_void_p, c_void_p, c_ll, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pm_project": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "pm_power_spectrum": (c_int, [c_void_p, c_void_p, c_double, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pm_density_noalloc": (c_int, [c_void_p, c_ll, c_int, c_double, c_void_p, c_void_p]),
    "pm_ics_create": (c_int, [c_int, c_int, ctypes.POINTER(c_void_p)]),
    "pm_ics_destroy": (None, [c_void_p]),
    "pm_ics_last_error": (c_char_p, [c_void_p]),
    "pm_ics_generate": (c_int, [c_void_p, ctypes.POINTER(PMConfigC), ctypes.POINTER(PMICParamsC), c_void_p,
                                c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "pm_batch_create": (c_int, [c_int, c_size_t, ctypes.POINTER(c_void_p)]),
    "pm_batch_destroy": (None, [c_void_p]),
    "pm_batch_last_error": (c_char_p, [c_void_p]),
    "pm_sim_footprint": (c_size_t, [ctypes.POINTER(PMConfigC)]),
    "pm_batch_add": (c_int, [c_void_p, ctypes.POINTER(PMConfigC), c_void_p, c_void_p, c_int, P_int]),
    "pm_batch_admits": (c_int, [c_void_p, ctypes.POINTER(PMConfigC)]),
    "pm_batch_step": (c_int, [c_void_p, c_int, c_void_p]),
    "pm_batch_get": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, P_double, P_int, c_void_p]),
    "pm_batch_active": (c_int, [c_void_p, c_int]),
    "pm_batch_density": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
    "pm_batch_remove": (c_int, [c_void_p, c_int]),
    "pm_batch_set_graphs": (c_int, [c_void_p, c_int]),
    "pm_batch_check": (c_int, [c_void_p, c_void_p, P_int]),
    "pm_batch_profile": (c_int, [c_void_p, c_int, ctypes.POINTER(ctypes.c_float), c_int, c_void_p]),
    "pm_batch_launches_per_step": (c_int, [c_void_p]),
    "pm_batch_host_seconds": (c_int, [c_void_p, P_double, c_int]),
    "pm_batch_set_autotune": (c_int, [c_void_p, c_int]),
    "pm_batch_schedule": (c_int, [c_void_p, P_int, c_int]),
}
PROFILE_PHASES = ("sort", "rows", "deposit", "x_r2c", "y_fwd", "z_green", "y_inv", "x_c2r", "kick", "coef")

_lib = None


def load(path: str | None = None):
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA engine first "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class PMError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code
