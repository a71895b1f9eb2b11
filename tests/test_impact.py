"""Droplet-impact diagnostics: ComputeEnergy (FluidCuda.cu:737-783),
Computetangential_velocity (:786-898) and SaveSpreadtime (:1128-1150).

CPU: the oracle's orc_impact against the reference's own host functions
(compiled from the reference sources into oracle/_ref/libref.so, which print
their sums with the default 6 significant digits to files under data/), and
against a vectorised numpy restatement, on the state of a reference fixture.
GPU: cpmp_impact_diag against the oracle on the PLAIN FP64 trajectory (1e-9
relative, the PLAIN FP64 parity level), and against numpy on the library's
own fields for the FUSED FP16 scheme (FP64 sums in another order: 1e-9).
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

KEYS = ("v", "v_xy", "v_z", "mv", "mv_xy", "mv_z", "energy", "energy_xy", "energy_z", "tangential",
        "m_tangential", "drop_momentum", "drop_mass")


def fixture_state(O, name="prw_walls_complex5"):
    z = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    kw = json.loads(str(z["setup"]))
    st = O.State(O.Setup(**kw), float(z["den_g"]), float(z["den_l"]))
    st.type[:] = z["type"]
    for f in ("dens", "mvx", "mvy", "mvz"):
        getattr(st, f)[:] = z[f]
    return st, kw, z


def numpy_impact(type_, rho, mv, dims, den_g, den_l):
    dx, dy, dz = dims
    r = rho.reshape(dx, dy, dz)
    a, b, c = (m.reshape(dx, dy, dz) for m in mv)
    t = type_.reshape(dx, dy, dz)
    mid = (den_g + den_l) / 2
    i, j, k = np.meshgrid(np.arange(dx), np.arange(dy), np.arange(dz), indexing="ij")
    box = (i >= 2) & (i < dx - 2) & (j >= 2) & (j < dy - 2) & (k >= 2) & (k < dz - 2)
    sel = box & (t == 1) & (r > mid)
    s3, s2 = np.sqrt(a * a + b * b + c * c), np.sqrt(a * a + b * b)
    al = np.arctan2(j - dy // 2, i - dx // 2)
    al = np.where(al < 0, al + 2 * np.pi, al)
    tv = a * np.sin(al) + b * np.cos(al)
    spread = (r > mid) & (k >= 2) & (k < dz - 2)
    vals = [s3[sel].sum(), s2[sel].sum(), c[sel].sum(), (r * s3)[sel].sum(), (r * s2)[sel].sum(),
            (r * c)[sel].sum(), (r * (a * a + b * b + c * c) / 2)[sel].sum(), (r * (a * a + b * b) / 2)[sel].sum(),
            (r * c * c / 2)[sel].sum(), tv[sel].sum(), (tv * r)[sel].sum(), (r * s3)[spread].sum(), r[spread].sum()]
    return dict(zip(KEYS, vals))


def close(got, want, rtol):
    scale = max(abs(v) for v in want.values())
    for k in KEYS:
        assert abs(got[k] - want[k]) <= rtol * max(abs(want[k]), 1e-6 * scale), (k, got[k], want[k])


def test_oracle_matches_numpy(oracle_mod):
    st, kw, z = fixture_state(oracle_mod)
    got = st.impact()
    want = numpy_impact(st.type, st.dens, (st.mvx, st.mvy, st.mvz), (kw["dx"], kw["dy"], kw["dz"]), st.den_g,
                        st.den_l)
    close(got, want, 1e-12)
    assert got["drop_mass"] > 0 and got["energy"] > 0


def test_oracle_matches_reference_host_functions(oracle_mod, tmp_path):
    so = os.path.join(ROOT, "oracle", "_ref", "libref.so")
    if not os.path.exists(so):
        pytest.skip("reference host build not available")
    L = C.CDLL(so)
    if not hasattr(L, "ref_impact"):
        pytest.skip("reference host build predates the impact diagnostics")
    st, kw, z = fixture_state(oracle_mod)
    (tmp_path / "data").mkdir()
    cwd = os.getcwd()
    try:
        os.chdir(tmp_path)
        P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
        L.ref_set_grid(kw["dx"], kw["dy"], kw["dz"])
        L.ref_impact(P(st.type), P(st.dens), P(st.mvx), P(st.mvy), P(st.mvz), C.c_double(st.den_g),
                     C.c_double(st.den_l), C.c_double(-0.04), C.c_int(1))
    finally:
        os.chdir(cwd)
    energy = open(tmp_path / "data" / "N4_Energy_or MV_-0.040.txt").read().splitlines()
    tang = open(tmp_path / "data" / "0722_N4_tangential_velocity_-0.040.txt").read().splitlines()
    assert energy[0].split()[:6] == ["NowStep", "Radius", "Diameter", "Tau", "DropVy", "V"]
    e = [float(v) for v in energy[1].split()]
    t = [float(v) for v in tang[1].split()]
    ref = dict(zip(KEYS[:9], e[5:14]))
    ref.update(tangential=t[5], m_tangential=t[6])
    got = st.impact()
    scale = max(abs(v) for v in ref.values())
    for k, v in ref.items():  # the reference prints 6 significant digits
        assert abs(got[k] - v) <= 6e-6 * max(abs(v), 1e-3 * scale), (k, got[k], v)


@pytest.mark.gpu
def test_device_impact_sums(cpmp, oracle_mod):
    from test_gpu_parity import load_case, solver_for
    O = oracle_mod
    z, kw = load_case("prw_walls_complex5")
    den = (float(z["den_g"]), float(z["den_l"]))
    s = solver_for(cpmp, kw, den=den)
    s.step(int(z["steps"]))
    got = s.impact()
    st, _, _ = fixture_state(O)
    close(got, st.impact(), 1e-9)  # the PLAIN FP64 trajectory against the reference's state
    assert got["drop_velocity"] == pytest.approx(got["drop_momentum"] / got["drop_mass"], rel=1e-15)
    s.close()
    s = solver_for(cpmp, kw, scheme="fused", storage="f16", den=den)
    s.step(int(z["steps"]))
    got = s.impact()
    n = kw["dx"] * kw["dy"] * kw["dz"]
    mv = s.get("mv")
    want = numpy_impact(s.get("type"), s.get("rho"), (mv[:n], mv[n:2 * n], mv[2 * n:]),
                        (kw["dx"], kw["dy"], kw["dz"]), *den)
    close(got, want, 1e-9)
    s.close()
