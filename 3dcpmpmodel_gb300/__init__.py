"""GB300 chemical-potential multiphase D3Q19 MRT lattice-Boltzmann step.

Python host side over the C ABI in ``include/cpmp.h`` (``libcpmp.so``, built
in-tree by ``build.py``).  The names follow the reference program
(zhou-yiling/3DCPMPmodel, FluidCuda.cu): ``Solver`` bundles what the
reference's globals, ``Initialize``/``SetMultiphase``/``CudaInitialize``,
``SetFlowField``, the step loop body and ``CalcMacroCPU``/``ContactAngle``
did.  There is no CPU fallback: constructing a ``Solver`` loads the CUDA
library and fails loudly if it is missing or no GPU is present.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _abi
from ._abi import (CPMP_F32, CPMP_F64, FIELD, MODEL, SCHEME, STORE, WALL, CpmpError,
                   Diag, Droplet, Impact, Params, lib)

__all__ = ["Solver", "Batch", "Params", "Droplet", "Diag", "Impact", "CpmpError", "lib", "default_params",
           "coexistence", "MODEL", "SCHEME", "STORE", "WALL", "FIELD", "reference_ts"]

Q = 19


def reference_ts(tau: float):
    """MRT rates of the reference's Initialize (FluidCuda.cu:154-157)."""
    ts = [1.0] * Q
    for q in (2, 4, 6, 8):
        ts[q] = 1.1
    for q in (9, 11, 13, 14, 15):
        ts[q] = 1.0 / tau
    return ts


def default_params(**kw) -> Params:
    """cpmp_params_default() with keyword overrides (field names of cpmp_params)."""
    p = Params()
    lib().cpmp_params_default(C.byref(p))
    for k, v in kw.items():
        if k == "ts":
            for q in range(Q):
                p.ts[q] = float(v[q])
            p.ts_from_tau = 0
        elif k == "cocurve_dir":
            p.cocurve_dir = None if v is None else v.encode()
        else:
            if not hasattr(p, k):
                raise AttributeError(f"cpmp_params has no field {k!r}")
            setattr(p, k, v)
    return p


def tecplot_write(path: str, title: str, zone: str, variables: dict, shape):
    """Write one ordered zone: variables = {name: numpy array (float32,
    float64, int32, int16 or int8), I fastest}; shape = (imax, jmax, kmax)."""
    codes = {np.dtype(np.float32): 1, np.dtype(np.float64): 2, np.dtype(np.int32): 3,
             np.dtype(np.int16): 4, np.dtype(np.int8): 5}
    arrs = [np.ascontiguousarray(v) for v in variables.values()]
    nv = len(arrs)
    names = (C.c_char_p * nv)(*[k.encode() for k in variables])
    types = (C.c_int * nv)(*[codes[a.dtype] for a in arrs])
    ptrs = (C.c_void_p * nv)(*[a.ctypes.data for a in arrs])
    _abi.check(lib().cpmp_tecplot_write(path.encode(), title.encode(), zone.encode(), nv, names, types, ptrs,
                                        int(shape[0]), int(shape[1]), int(shape[2])))


def dim_velocity(radius: float, diameter: float, tau: float) -> float:
    """DimV of the reference's DimConversion(Radius*2, Diameter, 7.2, 1.0,
    Viscosity, 0.01) (FluidCuda.cu:137-139, 474-486), same operation order."""
    visc = (tau * 2 - 1) / 6
    dim_len = diameter / (radius * 2)
    dim_time = visc / 0.01 * (dim_len * dim_len)
    return dim_len / dim_time


def coexistence(model: int, tr: float, eos_a=0.0, eos_b=0.0, eos_omega=0.0, cocurve_dir=None):
    """SetMultiphase stand-alone: dict of den_g, den_l, A, B, Tc, Rc."""
    out = [C.c_double() for _ in range(6)]
    _abi.check(lib().cpmp_coexistence(int(model), float(tr), float(eos_a), float(eos_b),
                                      float(eos_omega),
                                      None if cocurve_dir is None else cocurve_dir.encode(),
                                      *[C.byref(o) for o in out]))
    return dict(zip(("den_g", "den_l", "A", "B", "Tc", "Rc"), [o.value for o in out]))


class Solver:
    """One simulation box on one GPU (a cpmp_handle)."""

    def __init__(self, params: Params | None = None, _borrowed=None, **kw):
        self._owned = _borrowed is None
        self.params = params if params is not None else default_params(**kw)
        if params is not None and kw:
            raise TypeError("give either a Params or keyword overrides")
        self._lib = lib()
        self._h = C.c_void_p()
        if _borrowed is None:
            _abi.check(self._lib.cpmp_create(C.byref(self.params), C.byref(self._h)))
        else:
            self._h = _borrowed
        p = self.params
        self.dx, self.dy, self.dz = p.dx, p.dy, p.dz
        self.n = p.dx * p.dy * p.dz
        g, l, A, B, T, Rc = (C.c_double() for _ in range(6))
        _abi.check(self._lib.cpmp_get_eos(self._h, C.byref(g), C.byref(l), C.byref(A), C.byref(B),
                                          C.byref(T), C.byref(Rc)))
        self.den_g, self.den_l, self.A, self.B, self.T, self.Rc = (g.value, l.value, A.value,
                                                                   B.value, T.value, Rc.value)

    # life cycle -----------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None) and self._h.value and getattr(self, "_owned", True):
            self._lib.cpmp_destroy(self._h)
        self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # reference operations ----------------------------------------------------------
    def set_flow_field(self, radius=None, width=None, centre=None):
        """SetFlowField: centre None -> the reference's placement (DX/2, DY/2, R+2)."""
        d = Droplet()
        d.radius = float(radius if radius is not None else 60.0)
        d.width = float(width if width is not None else 10.0)
        if centre is None:
            d.ref_centre = 1
        else:
            d.ref_centre = 0
            d.cx, d.cy, d.cz = (float(c) for c in centre)
        _abi.check(self._lib.cpmp_init_droplet(self._h, C.byref(d)))
        return self

    def set_base_pt(self, base_pt: float):
        _abi.check(self._lib.cpmp_set_base_pt(self._h, C.c_double(base_pt)))

    def set_wall_field(self, wall: np.ndarray):
        w = np.ascontiguousarray(wall, dtype=np.float64).reshape(-1)
        _abi.check(self._lib.cpmp_set_wall_field(self._h, w.ctypes.data_as(C.POINTER(C.c_double)),
                                                 C.c_size_t(w.size)))

    def step(self, n: int = 1):
        _abi.check(self._lib.cpmp_step(self._h, int(n)))
        return self

    def sync(self):
        _abi.check(self._lib.cpmp_sync(self._h))

    def get(self, field: str, dtype=np.float64) -> np.ndarray:
        f = FIELD[field]
        comps = {"rho": 1, "mu": 1, "u": 3, "mv": 3, "force": 3, "dist": Q, "type": 1}[field]
        if field == "type":
            out = np.empty(self.n, np.uint8)
            _abi.check(self._lib.cpmp_get_field(self._h, f, 0, out.ctypes.data_as(C.c_void_p),
                                                C.c_size_t(out.nbytes)))
            return out
        dt = np.dtype(dtype)
        out = np.empty(comps * self.n, dt)
        code = CPMP_F64 if dt == np.float64 else CPMP_F32
        _abi.check(self._lib.cpmp_get_field(self._h, f, code, out.ctypes.data_as(C.c_void_p),
                                            C.c_size_t(out.nbytes)))
        return out

    def set(self, field: str, values: np.ndarray):
        a = np.ascontiguousarray(values)
        if a.dtype not in (np.float64, np.float32):
            a = a.astype(np.float64)
        code = CPMP_F64 if a.dtype == np.float64 else CPMP_F32
        _abi.check(self._lib.cpmp_set_field(self._h, FIELD[field], code,
                                            a.ctypes.data_as(C.c_void_p), C.c_size_t(a.nbytes)))

    def impact(self) -> dict:
        """Droplet-impact sums of the current state (ComputeEnergy,
        Computetangential_velocity, SaveSpreadtime), on the device."""
        d = Impact()
        _abi.check(self._lib.cpmp_impact_diag(self._h, C.byref(d)))
        return {k: getattr(d, k) for k, _ in Impact._fields_}

    def reduce(self, allow_nonfinite: bool = False) -> dict:
        """CalcMacroCPU + ContactAngle(0, DY/2) + the Laplace probe, on the device."""
        d = Diag()
        rc = self._lib.cpmp_reduce(self._h, C.byref(d))
        if rc != 0 and not (allow_nonfinite and rc == _abi.CPMP_ERR_NONFINITE):
            _abi.check(rc)
        return {k: getattr(d, k) for k, _ in Diag._fields_}

    def write_tecplot(self, path: str, layout: str = "savetask", decimate: int = 5,
                      reference_stride: bool = False, vel_scale: float = 1.0):
        """Tecplot binary output in the reference's SaveTask / SaveAllByType
        layouts; vel_scale is the reference's DimV (see dim_velocity)."""
        lay = {"savetask": 0, "allbytype": 1}[layout]
        _abi.check(self._lib.cpmp_write_tecplot(self._h, path.encode(), lay, int(decimate),
                                                1 if reference_stride else 0, float(vel_scale)))

    def set_kappa(self, ka: float):
        _abi.check(self._lib.cpmp_set_kappa(self._h, C.c_double(ka)))

    def adjoint(self, steps: int, target_rho: np.ndarray, checkpoint_every: int = 0):
        """Loss sum_fluid (rho^T - target)^2 after `steps` steps from the
        current state, and its gradients w.r.t. the wall field (2*DX*DY) and
        kappa (sqrt(T) checkpoint-and-recompute).  Returns (loss, grad_wall,
        grad_kappa); the state is left at step `steps`."""
        t = np.ascontiguousarray(target_rho, dtype=np.float64).reshape(-1)
        if t.size != self.n:
            raise ValueError("target must have N values")
        gw = np.zeros(2 * self.dx * self.dy, np.float64)
        loss, gk = C.c_double(), C.c_double()
        _abi.check(self._lib.cpmp_adjoint(self._h, int(steps), int(checkpoint_every),
                                          t.ctypes.data_as(C.c_void_p), C.byref(loss),
                                          gw.ctypes.data_as(C.c_void_p), C.byref(gk)))
        return loss.value, gw, gk.value

    def autotune(self) -> dict:
        """Pick the fused kernel's tile shape and march length by timing them
        on a scratch copy of the current state."""
        ty, tz, xl, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _abi.check(self._lib.cpmp_autotune(self._h, C.byref(ty), C.byref(tz), C.byref(xl), C.byref(ms)))
        t = self.tile()
        t["collide_ms"] = ms.value
        return t

    def set_tile(self, tile_y: int, tile_z: int, march_x: int, nodes_per_thread: int = 1, form: int = 0):
        """Column tile (tile_y x tile_z nodes), x-march length and nodes per
        thread (1, or 2 for the paired kernel) of the fused collide; form 0
        runs it in one pass, 1 as a force pass (the tile is its) and a
        collide-stream pass (node pairs)."""
        _abi.check(self._lib.cpmp_set_tile_form(self._h, int(tile_y), int(tile_z), int(march_x),
                                                int(nodes_per_thread), int(form)))

    def tile(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        _abi.check(self._lib.cpmp_get_tile(self._h, *(C.byref(x) for x in v)))
        t = dict(zip(("tile_y", "tile_z", "march_x", "nodes_per_thread"), (x.value for x in v)))
        f = C.c_int()
        _abi.check(self._lib.cpmp_get_form(self._h, C.byref(f)))
        t["form"] = f.value
        return t

    # timing ------------------------------------------------------------------------
    @property
    def stream(self) -> int:
        return self._lib.cpmp_stream(self._h) or 0

    def kernel_timing(self, on: bool):
        _abi.check(self._lib.cpmp_set_kernel_timing(self._h, 1 if on else 0))

    def kernel_times(self) -> dict:
        cap = 16
        names = (C.c_char_p * cap)()
        launches = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        k = self._lib.cpmp_kernel_times(self._h, names, launches, ms, cap)
        return {names[i].decode(): (launches[i], ms[i]) for i in range(min(k, cap))}

    @property
    def launch_count(self) -> int:
        return int(self._lib.cpmp_launch_count(self._h))


class Batch:
    """Many independent boxes stepped by one persistent launch (cpmp_batch).

    ``boxes[i]`` is a borrowed ``Solver`` view of box i for initialisation,
    field access and reductions; step the whole batch with ``step``."""

    def __init__(self, params_list):
        self._lib = lib()
        arr = (Params * len(params_list))(*params_list)
        self._b = C.c_void_p()
        _abi.check(self._lib.cpmp_batch_create(arr, len(params_list), C.byref(self._b)))
        self.boxes = []
        for i, p in enumerate(params_list):
            h = C.c_void_p()
            _abi.check(self._lib.cpmp_batch_handle(self._b, i, C.byref(h)))
            self.boxes.append(Solver(params=p, _borrowed=h))
        self.nodes = int(self._lib.cpmp_batch_nodes(self._b))

    def step(self, n: int = 1):
        _abi.check(self._lib.cpmp_batch_step(self._b, int(n)))
        return self

    def sync(self):
        _abi.check(self._lib.cpmp_batch_sync(self._b))

    def reduce(self, allow_nonfinite: bool = False) -> list:
        """Solver.reduce of every box, in four launches for the whole batch
        (the same values, bit for bit)."""
        arr = (Diag * len(self.boxes))()
        rc = self._lib.cpmp_batch_reduce(self._b, arr, len(self.boxes))
        if rc != 0 and not (allow_nonfinite and rc == _abi.CPMP_ERR_NONFINITE):
            _abi.check(rc)
        return [{k: getattr(d, k) for k, _ in Diag._fields_} for d in arr]

    def set_tile(self, tile_y: int, tile_z: int, march_x: int, nodes_per_thread: int = 1):
        _abi.check(self._lib.cpmp_batch_set_tile_ex(self._b, int(tile_y), int(tile_z), int(march_x),
                                                    int(nodes_per_thread)))

    def tile(self) -> dict:
        v = [C.c_int() for _ in range(4)]
        _abi.check(self._lib.cpmp_batch_get_tile(self._b, *(C.byref(x) for x in v)))
        return dict(zip(("tile_y", "tile_z", "march_x", "nodes_per_thread"), (x.value for x in v)))

    def autotune(self) -> dict:
        ty, tz, xl, ms = C.c_int(), C.c_int(), C.c_int(), C.c_double()
        _abi.check(self._lib.cpmp_batch_autotune(self._b, C.byref(ty), C.byref(tz), C.byref(xl),
                                                 C.byref(ms)))
        t = self.tile()
        t["step_ms"] = ms.value
        return t

    @property
    def stream(self) -> int:
        return self._lib.cpmp_batch_stream(self._b) or 0

    @property
    def launch_count(self) -> int:
        return int(self._lib.cpmp_batch_launch_count(self._b))

    def kernel_timing(self, on: bool):
        _abi.check(self._lib.cpmp_batch_set_kernel_timing(self._b, 1 if on else 0))

    def kernel_times(self) -> dict:
        cap = 16
        names = (C.c_char_p * cap)()
        launches = (C.c_longlong * cap)()
        ms = (C.c_double * cap)()
        k = self._lib.cpmp_batch_kernel_times(self._b, names, launches, ms, cap)
        return {names[i].decode(): (launches[i], ms[i]) for i in range(min(k, cap))}

    def close(self):
        if getattr(self, "_b", None) and self._b.value:
            for s in self.boxes:
                s._h = C.c_void_p()
            self._lib.cpmp_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
