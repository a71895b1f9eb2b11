"""CPU: the FP64 oracle against the reference's own kernels (golden fixtures
generated by tests/golden/make_golden.py) and the coexistence known answers."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = sorted(f[4:-4] for f in os.listdir(GOLDEN) if f.startswith("ref_") and f.endswith(".npz"))
FIELDS = ("dens", "pote", "dist", "vx", "vy", "vz", "fx", "fy", "fz", "mvx", "mvy", "mvz")


def load_case(name):
    z = np.load(os.path.join(GOLDEN, f"ref_{name}.npz"))
    return z, json.loads(str(z["setup"]))


@pytest.mark.parametrize("case", CASES)
def test_oracle_bit_identical_to_reference_kernels(oracle_mod, case):
    O = oracle_mod
    z, kw = load_case(case)
    st = O.State(O.Setup(**kw), float(z["den_g"]), float(z["den_l"]), "oracle").init()
    assert np.array_equal(st.type, z["type"])
    assert np.array_equal(st.dens, z["init_dens"])
    assert np.array_equal(st.dist, z["init_dist"])
    st.step(int(z["steps"]))
    for f in FIELDS:
        assert np.array_equal(getattr(st, f), z[f]), f


@pytest.mark.parametrize("case", CASES)
def test_reference_host_build_reproduces_fixture(oracle_mod, case):
    O = oracle_mod
    if not os.path.exists(O.REF_SO):
        pytest.skip("oracle/_ref not built on this machine")
    z, kw = load_case(case)
    st = O.State(O.Setup(**kw), float(z["den_g"]), float(z["den_l"]), "ref").init()
    st.step(int(z["steps"]))
    for f in FIELDS:
        assert np.array_equal(getattr(st, f), z[f]), f


# Tolerances: the reference gives Tc and rho_c to 6-8 digits, so its tables
# agree with an exact Maxwell construction only to that precision.
TOL = {"VDW": 1e-12, "PRW": 2e-9, "PRM": 2e-9, "CSE": 5e-7, "RKE": 5e-5, "RKS": 5e-5}


def test_cocurve_rows_are_maxwell_coexistence(oracle_mod):
    O = oracle_mod
    rows = json.load(open(os.path.join(GOLDEN, "cocurve_rows.json")))
    model_of = {v: k for k, v in O.TAG_OF_MODEL.items()}
    n = 0
    for tag, by_tr in rows.items():
        model = model_of[tag]
        for trs, (g, l) in by_tr.items():
            tr = float(trs)
            A, B, Tc, Rc = O.eos_constants(model, tr)
            gg, ll = O.coexistence(model, tr)
            assert abs(gg / (g * Rc) - 1) < TOL[tag], (tag, tr)
            assert abs(ll / (l * Rc) - 1) < TOL[tag], (tag, tr)
            eos = O.EOS_OF_MODEL[model]
            T = tr * Tc
            dmu = O.mu0(eos, A, B, T, g * Rc) - O.mu0(eos, A, B, T, l * Rc)
            dp = O.pressure(eos, A, B, T, g * Rc) - O.pressure(eos, A, B, T, l * Rc)
            assert abs(dmu) < 50 * TOL[tag] and abs(dp) < 50 * TOL[tag], (tag, tr, dmu, dp)
            n += 1
    assert n >= 36


def test_oracle_mass_conserved_walls_and_periodic(oracle_mod):
    O = oracle_mod
    for kw in (dict(dx=20, dy=6, dz=18, radius=5.0, width=4.0),
               dict(dx=16, dy=16, dz=16, radius=4.0, width=3.0, wall_mode=0, centre=(8, 8, 8),
                    model=O.MP_CPCSE, tr=0.85, eos_a=0.5, eos_b=4.0, Ka=0.01, tau=1.0)):
        s = O.Setup(**kw)
        g, l = O.coexistence(s.model, s.tr, s.eos_a, s.eos_b)
        st = O.State(s, g, l, "oracle").init()
        st.step(1)
        m0 = st.mass()[0]
        st.step(60)
        m1 = st.mass()[0]
        assert abs(m1 - m0) <= 1e-12 * m0


def test_contact_angle_straight_interface(oracle_mod):
    """A straight liquid/vapour interface meeting the wall at angle theta:
    the reference's crossing-and-extrapolation gives theta back."""
    O = oracle_mod
    dx, dy, dz = 200, 1, 60
    dg, dl = 0.1, 8.0
    for theta in (35.0, 60.0, 90.0, 120.0, 145.0):
        s = O.Setup(dx=dx, dy=dy, dz=dz)
        st = O.State(s, dg, dl, "oracle")
        t = np.radians(theta)
        i = np.arange(dx)[:, None].astype(float)
        k = np.arange(dz)[None, :].astype(float)
        # left edge of the liquid at x = 60 on the plane k = 2, leaning by theta;
        # the right edge mirrored about the centre line
        xl = 60 + (k - 2) / np.tan(t)
        xr = dx - 60 - (k - 2) / np.tan(t)
        inside = np.minimum(i - xl, xr - i) * np.sin(t)
        rho = (dl + dg) / 2 + (dl - dg) / 2 * np.tanh(inside / 2.5)
        st.dens[:] = rho.reshape(-1)
        ca = st.contact_angle(0)
        assert abs(ca["ca_left"] - theta) < 0.5, (theta, ca)
        assert abs(ca["ca_right"] - theta) < 0.5, (theta, ca)


def test_laplace_probe_on_a_known_sphere(oracle_mod):
    """SaveDataOriDen's radius on a tanh sphere of known radius, and its
    pressure jump from the EOS at the two probe points."""
    O = oracle_mod
    s = O.Setup(dx=32, dy=48, dz=32, wall_mode=0, model=O.MP_CPCSE, tr=0.85, eos_a=0.5, eos_b=4.0)
    dg, dl = 0.03, 0.28
    st = O.State(s, dg, dl, "oracle")
    i, j, k = np.meshgrid(np.arange(32), np.arange(48), np.arange(32), indexing="ij")
    for R in (8.0, 12.5, 17.0):
        r = np.sqrt((i - 16.0) ** 2 + (j - 24.0) ** 2 + (k - 16.0) ** 2)
        st.dens[:] = ((dl + dg) / 2 - (dl - dg) / 2 * np.tanh((r - R) / 1.5)).reshape(-1)
        o = st.laplace()
        assert abs(o["lap_r"] - R) < 0.05, (R, o)
        eos = O.EOS_OF_MODEL[s.model]
        p_in = O.pressure(eos, st.A, st.B, st.T, st.dens[(16 * 48 + 24) * 32 + 16])
        p_out = O.pressure(eos, st.A, st.B, st.T, st.dens[(16 * 48 + 0) * 32 + 16])
        assert o["lap_dp"] == pytest.approx(p_in - p_out, rel=1e-14)
        assert o["sigma"] == pytest.approx(s.K * o["sigma_k"], rel=1e-14)
