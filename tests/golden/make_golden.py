"""Generate the committed golden fixtures from the reference itself.

Run where the reference tree is present, giving its location:

    python tests/golden/make_golden.py --src <reference tree>

(or set CPMP_REFERENCE_SRC to that location).

Writes into tests/golden/:
  * cocurve_rows.json  -- rows of the reference's CoCurve_<EOS>_2.txt tables
    at the temperatures the tests and benchmarks use (reduced units);
  * ref_<case>.npz     -- initial state and the state after N steps produced
    by the reference's own kernels (FluidCuda.cu:188-463) compiled for the
    host by oracle/build_ref.py, for small grids.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402
import build_ref  # noqa: E402,F401

TRS = [0.6, 0.65, 0.7, 0.75, 0.8, 0.85, 0.9]

# name: (Setup kwargs, steps)
CASES = {
    # reference defaults (CP-PRW, Tr 0.7, K 0.2, Ka 0.001, tau 0.8), 3-D box with walls
    "prw_walls_complex5": (dict(dx=24, dy=6, dz=20, radius=6.0, width=4.0, base_pt=-0.04), 40),
    # the committed reference grid is quasi-2-D (DY = 1)
    "prw_quasi2d": (dict(dx=28, dy=1, dz=18, radius=7.0, width=4.0, base_pt=0.02), 40),
    # SIMPLECHEMBOUNDARY
    "prw_walls_simple5": (dict(dx=16, dy=8, dz=18, radius=5.0, width=4.0, complex_bc=0,
                               base_pt=-0.06), 30),
    # PTCALCSEVENPOINT
    "prw_walls_complex7": (dict(dx=18, dy=7, dz=20, radius=5.0, width=4.0, lap_order=7,
                                base_pt=0.0), 30),
    # K1/K2 pressure-tensor term and the PRM model
    "prm_k1k2": (dict(dx=16, dy=6, dz=18, radius=5.0, width=4.0, model=O.MP_CPPRM, K1=0.002,
                      K2=-0.002, tau=1.0), 25),
}


def cocurve(src: str) -> dict:
    out = {}
    for model, tag in O.TAG_OF_MODEL.items():
        rows = {}
        for tr in TRS:
            r = O.read_cocurve(os.path.join(src, "CoCurve", f"CoCurve_{tag}_2.txt"), tr)
            if r is not None:
                rows[f"{tr:.3f}"] = [r[0], r[1]]
        out[tag] = rows
    return out


def run_case(name: str, kw: dict, steps: int, src: str):
    s = O.Setup(**kw)
    tag = O.TAG_OF_MODEL[s.model]
    g, l = O.read_cocurve(os.path.join(src, "CoCurve", f"CoCurve_{tag}_2.txt"), s.tr)
    A, B, Tc, Rc, T = s.constants()
    st = O.State(s, g * Rc, l * Rc, backend="ref").init()
    init_dens, init_dist = st.dens.copy(), st.dist.copy()
    st.step(steps)
    np.savez_compressed(
        os.path.join(HERE, f"ref_{name}.npz"),
        setup=json.dumps({k: v for k, v in kw.items()}),
        steps=steps, den_g=g * Rc, den_l=l * Rc,
        type=st.type, init_dens=init_dens, init_dist=init_dist,
        dens=st.dens, pote=st.pote, dist=st.dist,
        vx=st.vx, vy=st.vy, vz=st.vz, fx=st.fx, fy=st.fy, fz=st.fz,
        mvx=st.mvx, mvy=st.mvy, mvz=st.mvz)


# Diameter (cm) of the Tecplot fixture's DimConversion; the reference's
# default 0 would make every liquid velocity NaN
TEC_DIAMETER = 0.05


def dim_velocity(radius, diameter, tau):
    """DimV of DimConversion(Radius*2, Diameter, 7.2, 1.0, Viscosity, 0.01)
    (FluidCuda.cu:137-139, 474-486), in the reference's operation order."""
    visc = (tau * 2 - 1) / 6
    dim_len = diameter / (radius * 2)
    dim_time = visc / 0.01 * (dim_len * dim_len)
    return dim_len / dim_time


def tecplot_arrays(case="prw_walls_complex5", DR=5):
    """The SaveTask and SaveAllByType arrays of a fixture state, indexed the
    way the reference builds them (FluidCuda.cu:466-472, 901-927, 1032-1092)."""
    z = np.load(os.path.join(HERE, f"ref_{case}.npz"))
    kw = json.loads(str(z["setup"]))
    DX, DY, DZ = kw["dx"], kw["dy"], kw["dz"]
    LX, LY, LZ = DX // DR, DY // DR, DZ // DR
    n = LX * LY * LZ
    mi = np.zeros(n, np.int16); mj = np.zeros(n, np.int16); mk = np.zeros(n, np.int16)
    dens = np.zeros(n)
    for i in range(LX):
        for j in range(LY):
            for k in range(LZ):
                m = i * LY * LZ + j * LZ + k
                mi[m], mj[m], mk[m] = i, j, k
                dens[m] = z["dens"][(i * DY * DZ + j * DZ + k) * DR]
    N = DX * DY * DZ
    ai = np.zeros(N); aj = np.zeros(N); ak = np.zeros(N)
    ux = np.zeros(N); uy = np.zeros(N); uz = np.zeros(N); ad = np.zeros(N)
    mid = (float(z["den_g"]) + float(z["den_l"])) / 2
    dimv = dim_velocity(kw["radius"], TEC_DIAMETER, kw.get("tau", 0.8))
    for i in range(DX):
        for j in range(DY):
            for k in range(DZ):
                p = i * DY * DZ + j * DZ + k
                x = i + j * DX + k * DY * DX
                ai[x], aj[x], ak[x] = i, j, k
                ad[x] = z["dens"][p]
                liq = z["dens"][p] >= mid
                ux[x] = z["mvx"][p] * dimv if liq else -2
                uy[x] = z["mvy"][p] * dimv if liq else -2
                uz[x] = z["mvz"][p] * dimv if liq else -2
    return (DX, DY, DZ, LX, LY, LZ, int(z["steps"])), (mi, mj, mk, dens), (ai, aj, ak, ux, uy, uz, ad)


def write_tecplot_golden():
    import ctypes as C
    so = O.build_ref and __import__("importlib").import_module("build_ref").build_tecplot()
    if not so:
        raise SystemExit("reference Tecplot writer unavailable")
    L = C.CDLL(so)
    dims, st, ab = tecplot_arrays()
    DX, DY, DZ, LX, LY, LZ, steps = dims
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = L.ref_tec_savetask(HERE.encode(), f"tec_FlowField_{steps}".encode(), LX, LY, LZ, *[P(a) for a in st])
    assert rc == 0
    rc = L.ref_tec_allbytype(HERE.encode(), f"tec_Field_3D_Nowstep={steps}".encode(), DX, DY, DZ,
                             *[P(a) for a in ab])
    assert rc == 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=os.environ.get("CPMP_REFERENCE_SRC"), required="CPMP_REFERENCE_SRC" not in os.environ)
    a = ap.parse_args()
    if O.build_ref() is None:
        sys.exit("oracle/_ref could not be built (reference sources unavailable)")
    with open(os.path.join(HERE, "cocurve_rows.json"), "w") as f:
        json.dump(cocurve(a.src), f, indent=1, sort_keys=True)
    for name, (kw, steps) in CASES.items():
        run_case(name, kw, steps, a.src)
        print("wrote", name)
    write_tecplot_golden()
    print("wrote Tecplot files")


if __name__ == "__main__":
    main()
