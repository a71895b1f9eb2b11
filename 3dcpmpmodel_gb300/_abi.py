"""ctypes declarations of include/cpmp.h."""
from __future__ import annotations

import ctypes as C
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcpmp.so")
Q = 19

CPMP_OK, CPMP_ERR_PARAM, CPMP_ERR_CUDA, CPMP_ERR_NOMEM, CPMP_ERR_COCURVE = 0, 1, 2, 3, 4
CPMP_ERR_NONFINITE, CPMP_ERR_TIMEOUT, CPMP_ERR_UNSUPPORTED, CPMP_ERR_SIZE = 5, 6, 7, 8
STATUS_NAMES = {0: "CPMP_OK", 1: "CPMP_ERR_PARAM", 2: "CPMP_ERR_CUDA", 3: "CPMP_ERR_NOMEM",
                4: "CPMP_ERR_COCURVE", 5: "CPMP_ERR_NONFINITE", 6: "CPMP_ERR_TIMEOUT",
                7: "CPMP_ERR_UNSUPPORTED", 8: "CPMP_ERR_SIZE"}
CPMP_F64, CPMP_F32 = 0, 1

MODEL = {"CPVDW": 201, "CPPRW": 202, "CPPRM": 203, "CPRKE": 204, "CPRKS": 205, "CPCSE": 206}
WALL = {"none": 0, "z": 1}
STORE = {"f64": 0, "f32": 1, "f16": 2, "bf16": 3}
SCHEME = {"plain": 0, "fused": 1}
FIELD = {"rho": 0, "u": 1, "mv": 2, "mu": 3, "force": 4, "dist": 5, "type": 6}


class CpmpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Params(C.Structure):
    _fields_ = [
        ("dx", C.c_int), ("dy", C.c_int), ("dz", C.c_int),
        ("model", C.c_int),
        ("tr", C.c_double), ("k", C.c_double), ("ka", C.c_double),
        ("k1", C.c_double), ("k2", C.c_double), ("tau", C.c_double),
        ("ts", C.c_double * Q), ("ts_from_tau", C.c_int),
        ("base_pt", C.c_double),
        ("eos_a", C.c_double), ("eos_b", C.c_double), ("eos_omega", C.c_double),
        ("den_g", C.c_double), ("den_l", C.c_double),
        ("cocurve_dir", C.c_char_p),
        ("wall_mode", C.c_int), ("lap_order", C.c_int), ("complex_bc", C.c_int),
        ("storage", C.c_int), ("scheme", C.c_int), ("device", C.c_int),
    ]


class Droplet(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double),
                ("radius", C.c_double), ("width", C.c_double), ("ref_centre", C.c_int)]


class Diag(C.Structure):
    _fields_ = [("mass", C.c_double), ("max_speed", C.c_double), ("nonfinite", C.c_int),
                ("ca_left", C.c_double), ("ca_right", C.c_double), ("ca_cap", C.c_double),
                ("x_left", C.c_double), ("x_right", C.c_double),
                ("cap_h", C.c_double), ("cap_l", C.c_double),
                ("lap_r", C.c_double), ("lap_dp", C.c_double), ("lap_sigma", C.c_double),
                ("step", C.c_longlong)]


class Impact(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("v", "v_xy", "v_z", "mv", "mv_xy", "mv_z", "energy", "energy_xy",
                                           "energy_z", "tangential", "m_tangential", "drop_momentum",
                                           "drop_mass", "drop_velocity")]


# name -> (restype, argtypes)
SIGNATURES = {
    "cpmp_params_default": (None, [C.c_void_p]),
    "cpmp_create": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cpmp_destroy": (None, [C.c_void_p]),
    "cpmp_init_droplet": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cpmp_set_base_pt": (C.c_int, [C.c_void_p, C.c_double]),
    "cpmp_set_wall_field": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.c_size_t]),
    "cpmp_step": (C.c_int, [C.c_void_p, C.c_int]),
    "cpmp_sync": (C.c_int, [C.c_void_p]),
    "cpmp_get_field": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
    "cpmp_set_field": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_size_t]),
    "cpmp_reduce": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cpmp_impact_diag": (C.c_int, [C.c_void_p, C.c_void_p]),
    "cpmp_get_eos": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_double)] * 6),
    "cpmp_coexistence": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                                   C.c_char_p] + [C.POINTER(C.c_double)] * 6),
    "cpmp_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "cpmp_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "cpmp_set_tile_ex": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "cpmp_get_tile": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 4),
    "cpmp_set_tile_form": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]),
    "cpmp_get_form": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "cpmp_stream": (C.c_void_p, [C.c_void_p]),
    "cpmp_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "cpmp_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong),
                                    C.POINTER(C.c_double), C.c_int]),
    "cpmp_launch_count": (C.c_longlong, [C.c_void_p]),
    "cpmp_tecplot_write": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "cpmp_write_tecplot": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_double]),
    "cpmp_get_dims": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "cpmp_set_kappa": (C.c_int, [C.c_void_p, C.c_double]),
    "cpmp_adjoint": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.POINTER(C.c_double),
                               C.c_void_p, C.POINTER(C.c_double)]),
    "cpmp_batch_create": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "cpmp_batch_handle": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "cpmp_batch_count": (C.c_int, [C.c_void_p]),
    "cpmp_batch_nodes": (C.c_longlong, [C.c_void_p]),
    "cpmp_batch_step": (C.c_int, [C.c_void_p, C.c_int]),
    "cpmp_batch_sync": (C.c_int, [C.c_void_p]),
    "cpmp_batch_reduce": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "cpmp_batch_set_tile": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "cpmp_batch_set_tile_ex": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int]),
    "cpmp_batch_get_tile": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 4),
    "cpmp_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                      C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "cpmp_batch_set_kernel_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "cpmp_batch_kernel_times": (C.c_int, [C.c_void_p, C.POINTER(C.c_char_p), C.POINTER(C.c_longlong),
                                          C.POINTER(C.c_double), C.c_int]),
    "cpmp_batch_launch_count": (C.c_longlong, [C.c_void_p]),
    "cpmp_batch_stream": (C.c_void_p, [C.c_void_p]),
    "cpmp_batch_destroy": (None, [C.c_void_p]),
    "cpmp_mass_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p,
                                    C.c_void_p]),
    "cpmp_last_error": (C.c_char_p, []),
}

_lib = None
_lock = threading.Lock()


def lib(path: str | None = None):
    """Load libcpmp.so (built in-tree by build.py).  Raises if it is missing:
    there is no fallback implementation."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise FileNotFoundError(
                    f"{p} is not built; run `python -c \"import __graft_entry__ as g; g.build()\"`")
            L = C.CDLL(p)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(L, name)
                fn.restype = res
                fn.argtypes = args
            _lib = L
        return _lib


def check(status: int):
    if status != CPMP_OK:
        raise CpmpError(status, (lib().cpmp_last_error() or b"").decode(errors="replace"))
