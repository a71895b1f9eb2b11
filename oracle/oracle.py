"""Python driver for the CPU checkers.  TEST INFRASTRUCTURE ONLY.

Two interchangeable FP64 CPU implementations of the reference time step:

* ``backend="oracle"``: ``oracle/cpmp_oracle.c``, the restatement of the
  reference algorithm (all EOS, periodic or walled boxes, wall fields);
* ``backend="ref"``: ``oracle/_ref/libref.so``, the reference's own kernel
  bodies compiled for the host (PR mu0 only, always walled, scalar BasePt).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU legs import this
module; the CUDA library never does.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")
Q = 19

# Model ids, reference Common.h:54-59
MP_CPVDW, MP_CPPRW, MP_CPPRM, MP_CPRKE, MP_CPRKS, MP_CPCSE = 201, 202, 203, 204, 205, 206
EOS_PR, EOS_VDW, EOS_CS, EOS_RK = 0, 1, 2, 3
EOS_OF_MODEL = {MP_CPVDW: EOS_VDW, MP_CPPRW: EOS_PR, MP_CPPRM: EOS_PR,
                MP_CPRKE: EOS_RK, MP_CPRKS: EOS_RK, MP_CPCSE: EOS_CS}
TAG_OF_MODEL = {MP_CPVDW: "VDW", MP_CPPRW: "PRW", MP_CPPRM: "PRM",
                MP_CPRKE: "RKE", MP_CPRKS: "RKS", MP_CPCSE: "CSE"}


def build(quiet: bool = True) -> str:
    """Compile the oracle (plain C, OpenMP, no FMA contraction)."""
    src = os.path.join(HERE, "cpmp_oracle.c")
    if (not os.path.exists(ORACLE_SO)) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.run(["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                        "-o", ORACLE_SO, src, "-lm"], check=True)
    return ORACLE_SO


def build_ref() -> str | None:
    import importlib.util
    spec = importlib.util.spec_from_file_location("cpmp_build_ref", os.path.join(HERE, "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    out = mod.build()
    try:  # the reference's Tecplot writer, where the reference tree is present
        mod.build_tecplot()
    except Exception:
        pass
    return out


def eos_constants(model: int, tr: float, a: float | None = None, b: float | None = None,
                  omega: float | None = None):
    """(A, B, Tc, Rc) as the reference's SetMultiphase (FluidCuda.cu:1318-1344).

    ``a``/``b`` override the CS constants (A = a, B = b/4, Tc and Rc scaled by
    corresponding states); ``omega`` overrides the PR/RKS acentric factor."""
    if model == MP_CPVDW:
        return 9 / 49, 2 / 21, 4 / 7, 7 / 2
    if model == MP_CPCSE:
        A, B, Tc, Rc = 1.0, 1.0, 0.09432870, 0.13044388
        if a is not None or b is not None:
            aa = 1.0 if a is None else a
            bb = 4.0 if b is None else b
            A, B = aa, bb / 4
            Tc = 0.09432870 * aa / (bb / 4)
            Rc = 0.13044388 / (bb / 4)
        return A, B, Tc, Rc
    if model == MP_CPRKE:
        Tc = 0.196133
        return 2 / 49 * (1 / math.sqrt(Tc * tr)), 2 / 21, Tc, 2.729171
    if model == MP_CPRKS:
        w = 0.344 if omega is None else omega
        return (2 / 49 * (1 + (0.480 + 1.574 * w - 0.176 * w * w) * (1 - math.sqrt(tr))) ** 2,
                2 / 21, 0.086861, 2.729171)
    if model in (MP_CPPRW, MP_CPPRM):
        w = (0.344 if model == MP_CPPRW else 0.011) if omega is None else omega
        return (2 / 49 * (1 + (0.37464 + 1.54226 * w - 0.26992 * w * w) * (1 - math.sqrt(tr))) ** 2,
                2 / 21, 0.072919, 2.65730416)
    raise ValueError(f"unsupported model id {model}")


def read_cocurve(path: str, tr: float):
    """Row matching T/Tc == tr within 1e-12 (reference Common.h:157-160,
    FluidCuda.cu:1370-1383).  Returns reduced (gas, liquid) or None."""
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) < 3:
                continue
            try:
                t0, g, l = float(parts[0]), float(parts[1]), float(parts[2])
            except ValueError:
                continue
            if abs(t0 - tr) < 1e-12:
                return g, l
    return None


def mu0(eos, A, B, T, rho):
    """numpy mirror of the oracle's mu0 (no density cap)."""
    rho = np.asarray(rho, dtype=np.float64)
    if eos == EOS_VDW:
        return T * np.log(rho / (1 - B * rho)) + T / (1 - B * rho) - 2 * A * rho
    if eos == EOS_CS:
        e = B * rho
        return T * np.log(rho) + T + T * (8 * e - 9 * e * e + 3 * e ** 3) / (1 - e) ** 3 - 2 * A * rho
    if eos == EOS_RK:
        return (T * np.log(rho / (1 - B * rho)) + T / (1 - B * rho) - A / B * np.log(1 + B * rho)
                - A * rho / (1 + B * rho))
    s2 = 1.4142135623730950488016887242097
    return (T * np.log(rho / (1 - B * rho)) - A / (s2 * 2 * B) * np.log((s2 - 1 + B * rho) / (s2 + 1 - B * rho))
            + T / (1 - B * rho) - A * rho / (1 + B * rho * 2 - (B * rho) ** 2))


def pressure(eos, A, B, T, rho):
    rho = np.asarray(rho, dtype=np.float64)
    if eos == EOS_VDW:
        return T * rho / (1 - B * rho) - A * rho * rho
    if eos == EOS_CS:
        e = B * rho
        return rho * T * (1 + e + e * e - e ** 3) / (1 - e) ** 3 - A * rho * rho
    if eos == EOS_RK:
        return T * rho / (1 - B * rho) - A * rho * rho / (1 + B * rho)
    return T * rho / (1 - B * rho) - A * rho * rho / (1 + B * rho * 2 - (B * rho) ** 2)


def reference_ts(tau: float):
    """MRT rates of the reference's Initialize (FluidCuda.cu:154-157)."""
    ts = [1.0] * Q
    for q in (2, 4, 6, 8):
        ts[q] = 1.1
    for q in (9, 11, 13, 14, 15):
        ts[q] = 1.0 / tau
    return ts


class _OrcParams(C.Structure):
    _fields_ = [("dx", C.c_int), ("dy", C.c_int), ("dz", C.c_int),
                ("K", C.c_double), ("A", C.c_double), ("B", C.c_double), ("T", C.c_double),
                ("Ka", C.c_double), ("K1", C.c_double), ("K2", C.c_double),
                ("ts", C.c_double * Q), ("eos", C.c_int), ("lap_order", C.c_int),
                ("complex_bc", C.c_int), ("wall_mode", C.c_int), ("base_pt", C.c_double),
                ("wall_pot", C.POINTER(C.c_double))]


class _OrcDroplet(C.Structure):
    _fields_ = [("cx", C.c_double), ("cy", C.c_double), ("cz", C.c_double),
                ("radius", C.c_double), ("width", C.c_double), ("den_g", C.c_double),
                ("den_l", C.c_double), ("ref_centre", C.c_int)]


@dataclass
class Setup:
    """Physical set-up of one run; defaults are the reference's Initialize()
    (FluidCuda.cu:119-163) with model CP-PRW."""
    dx: int = 32
    dy: int = 8
    dz: int = 24
    model: int = MP_CPPRW
    tr: float = 0.7
    K: float = 0.2
    Ka: float = 0.001
    K1: float = 0.0
    K2: float = 0.0
    tau: float = 0.8
    ts: list | None = None
    base_pt: float = -0.08
    radius: float = 60.0
    width: float = 10.0
    wall_mode: int = 1
    lap_order: int = 5
    complex_bc: int = 1
    den_g: float | None = None
    den_l: float | None = None
    eos_a: float | None = None
    eos_b: float | None = None
    eos_omega: float | None = None
    centre: tuple | None = None  # None: reference placement (DX/2, DY/2, R+2)
    wall_pot: np.ndarray | None = field(default=None, repr=False)

    def constants(self):
        A, B, Tc, Rc = eos_constants(self.model, self.tr, self.eos_a, self.eos_b, self.eos_omega)
        return A, B, Tc, Rc, self.tr * Tc

    @property
    def n(self):
        return self.dx * self.dy * self.dz


IMPACT_KEYS = ("v", "v_xy", "v_z", "mv", "mv_xy", "mv_z", "energy", "energy_xy", "energy_z", "tangential",
               "m_tangential", "drop_momentum", "drop_mass")


class State:
    """Fields of one run in the reference layout, advanced by a CPU backend."""

    def __init__(self, setup: Setup, den_g: float, den_l: float, backend: str = "oracle"):
        self.s = setup
        self.backend = backend
        self.den_g, self.den_l = den_g, den_l
        n = setup.n
        self.type = np.zeros(n, np.uint8)
        z = lambda: np.zeros(n, np.float64)
        self.dens, self.pote = z(), z()
        self.vx, self.vy, self.vz = z(), z(), z()
        self.fx, self.fy, self.fz = z(), z(), z()
        self.mvx, self.mvy, self.mvz = z(), z(), z()
        self.dist = np.zeros(Q * n, np.float64)
        self.temp = np.zeros(Q * n, np.float64)
        A, B, Tc, Rc, T = setup.constants()
        self.A, self.B, self.T, self.Rc = A, B, T, Rc
        ts = setup.ts if setup.ts is not None else reference_ts(setup.tau)
        if backend == "oracle":
            self.lib = C.CDLL(build())
            p = _OrcParams()
            p.dx, p.dy, p.dz = setup.dx, setup.dy, setup.dz
            p.K, p.A, p.B, p.T, p.Ka, p.K1, p.K2 = setup.K, A, B, T, setup.Ka, setup.K1, setup.K2
            for q in range(Q):
                p.ts[q] = ts[q]
            p.eos = EOS_OF_MODEL[setup.model]
            p.lap_order, p.complex_bc, p.wall_mode = setup.lap_order, setup.complex_bc, setup.wall_mode
            p.base_pt = setup.base_pt
            self._wall = None
            if setup.wall_pot is not None:
                self._wall = np.ascontiguousarray(setup.wall_pot, dtype=np.float64).reshape(-1)
                assert self._wall.size == 2 * setup.dx * setup.dy
                p.wall_pot = self._wall.ctypes.data_as(C.POINTER(C.c_double))
            self.p = p
        elif backend == "ref":
            if not os.path.exists(REF_SO):
                raise FileNotFoundError("oracle/_ref/libref.so is not built")
            if setup.wall_mode != 1 or setup.wall_pot is not None:
                raise ValueError("the reference step always has z walls and a scalar BasePt")
            self.lib = C.CDLL(REF_SO)
            self.variant = {(5, 1): 0, (5, 0): 1, (7, 1): 2}[(setup.lap_order, setup.complex_bc)]
            self._ts = (C.c_double * Q)(*ts)
        else:
            raise ValueError(backend)

    def _ptr(self, a):
        return a.ctypes.data_as(C.c_void_p)

    def _ref_bind(self):
        s = self.s
        self.lib.ref_set_grid(s.dx, s.dy, s.dz)
        d = C.c_double
        self.lib.ref_set_params(d(s.K), d(self.A), d(self.B), d(self.T), d(s.Ka), d(s.K1), d(s.K2),
                                d(self.den_g), d(self.den_l), d(s.base_pt), d(s.radius),
                                d(s.width), self._ts)

    def init(self):
        s = self.s
        if self.backend == "ref":
            if s.centre is not None:
                raise ValueError("the reference places the droplet at (DX/2, DY/2, R+2)")
            self._ref_bind()
            self.lib.ref_init(self._ptr(self.type), self._ptr(self.dens), self._ptr(self.pote),
                              self._ptr(self.dist), self._ptr(self.temp))
            self.vx[:] = self.vy[:] = self.vz[:] = 0
            return self
        d = _OrcDroplet()
        if s.centre is None:
            d.ref_centre = 1
        else:
            d.ref_centre = 0
            d.cx, d.cy, d.cz = s.centre
        d.radius, d.width, d.den_g, d.den_l = s.radius, s.width, self.den_g, self.den_l
        self.lib.orc_init(C.byref(self.p), C.byref(d), self._ptr(self.type), self._ptr(self.dens),
                          self._ptr(self.pote), self._ptr(self.dist), self._ptr(self.vx),
                          self._ptr(self.vy), self._ptr(self.vz))
        return self

    def step(self, n: int = 1):
        args = [self._ptr(a) for a in (self.type, self.dens, self.pote, self.dist, self.temp,
                                       self.vx, self.vy, self.vz, self.fx, self.fy, self.fz,
                                       self.mvx, self.mvy, self.mvz)]
        if self.backend == "ref":
            self._ref_bind()
            rc = self.lib.ref_step(self.variant, int(n), *args)
            if rc != 0:
                raise RuntimeError("ref_step failed")
        else:
            self.lib.orc_step(C.byref(self.p), int(n), *args)
        return self

    # diagnostics -------------------------------------------------------------
    def mass(self):
        out = (C.c_double * 3)()
        if self.backend != "oracle":
            raise ValueError("diagnostics run on the oracle backend")
        self.lib.orc_mass(C.byref(self.p), self._ptr(self.type), self._ptr(self.dens),
                          self._ptr(self.mvx), self._ptr(self.mvy), self._ptr(self.mvz), out)
        return out[0], out[1], bool(out[2])

    def contact_angle(self, tier: int | None = None):
        out = (C.c_double * 7)()
        t = self.s.dy // 2 if tier is None else tier
        self.lib.orc_contact_angle(C.byref(self.p), self._ptr(self.dens), C.c_int(t),
                                   C.c_double(self.den_g), C.c_double(self.den_l), out)
        return dict(zip(("ca_left", "ca_right", "ca_cap", "x_left", "x_right", "h", "l"), list(out)))

    def impact(self):
        """Droplet-impact sums (ComputeEnergy, Computetangential_velocity,
        SaveSpreadtime): dict in the order of cpmp_impact."""
        out = (C.c_double * 13)()
        self.lib.orc_impact(C.byref(self.p), self._ptr(self.type), self._ptr(self.dens), self._ptr(self.mvx),
                            self._ptr(self.mvy), self._ptr(self.mvz), C.c_double(self.den_g),
                            C.c_double(self.den_l), out)
        return dict(zip(IMPACT_KEYS, list(out)))

    def laplace(self, dens=None):
        """Laplace-law probe of SaveDataOriDen (FluidCuda.cu:1159-1199).

        Along the row (DX/2, j, DZ/2): MidDen is the mean of the densities at
        j = 0 (outside) and j = DY/2 (inside); the radius is DY/2 minus the
        first j in 0..DY/2 with rho(j) <= MidDen < rho(j+1), linearly
        interpolated (0 when there is none); dp is the EOS pressure at the
        inside probe minus that at the outside probe (EosPressure,
        FluidCuda.cu:1561-1573, here for every EOS).  The reference scales the
        surface tension by K (:1181); ``sigma_k`` is that value, ``sigma``
        the one consistent with mu = K^2 mu0 (K^2 dp R / 2)."""
        s = self.s
        d = self.dens if dens is None else dens
        D = lambda j: float(d[((s.dx // 2) * s.dy + j) * s.dz + s.dz // 2])  # noqa: E731
        tout, tin = D(0), D(s.dy // 2)
        mid = (tout + tin) / 2
        rad = 0.0
        for j in range(0, s.dy // 2 + 1):
            if j + 1 >= s.dy:
                break
            t1, t2 = D(j), D(j + 1)
            if t1 <= mid and t2 > mid:
                rad = float(s.dy // 2) - (j + (mid - t1) / (t2 - t1))
                break
        eos = EOS_OF_MODEL[s.model]
        dp = float(pressure(eos, self.A, self.B, self.T, tin) - pressure(eos, self.A, self.B, self.T, tout))
        return dict(lap_r=rad, lap_dp=dp, sigma_k=s.K * dp * rad / 2, sigma=s.K * s.K * dp * rad / 2)

    def view(self, a):
        return a.reshape(self.s.dx, self.s.dy, self.s.dz)


def _bind_signatures():
    pass


def coexistence(model: int, tr: float, a=None, b=None, omega=None):
    """Maxwell construction, FP64: (den_g, den_l) in lattice units with
    mu0(g) = mu0(l) and p(g) = p(l).  Newton on the two conditions from the
    spinodal bracket.  Used to check the CoCurve tables and the library's own
    solver."""
    A, B, Tc, Rc = eos_constants(model, tr, a, b, omega)
    T = tr * Tc
    eos = EOS_OF_MODEL[model]
    # spinodal points: dp/drho = 0 on a fine grid
    rmax = 0.999 / B if eos != EOS_CS else 0.999 / B
    r = np.linspace(1e-6, rmax, 200001)
    p = pressure(eos, A, B, T, r)
    dp = np.diff(p)
    sign = np.where(np.diff(np.sign(dp)) != 0)[0]
    if len(sign) < 2:
        raise ValueError("supercritical temperature")
    r_sp1, r_sp2 = r[sign[0] + 1], r[sign[1] + 1]
    g, l = r_sp1 * 0.5, min(r_sp2 * 1.5, rmax * 0.99)
    # equal-area guess: scan pressure levels
    for _ in range(200):
        mg, ml = mu0(eos, A, B, T, g), mu0(eos, A, B, T, l)
        pg, pl = pressure(eos, A, B, T, g), pressure(eos, A, B, T, l)
        h = 1e-7
        dmg = (mu0(eos, A, B, T, g * (1 + h)) - mu0(eos, A, B, T, g * (1 - h))) / (2 * g * h)
        dml = (mu0(eos, A, B, T, l * (1 + h)) - mu0(eos, A, B, T, l * (1 - h))) / (2 * l * h)
        # dp/drho = rho dmu/drho
        J = np.array([[dmg, -dml], [g * dmg, -l * dml]])
        F = np.array([mg - ml, pg - pl])
        dx_ = np.linalg.solve(J, -F)
        step = 1.0
        while True:
            ng, nl = g + step * dx_[0], l + step * dx_[1]
            if 0 < ng < r_sp1 and r_sp2 < nl < rmax:
                break
            step *= 0.5
            if step < 1e-12:
                break
        g, l = ng, nl
        if abs(F[0]) < 1e-15 and abs(F[1]) < 1e-15:
            break
    return float(g), float(l)
