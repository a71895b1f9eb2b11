"""cpmp_run, the command-line driver with the reference's host loop
(FluidCuda.cu:1245-1312): BasePt sweep without re-initialisation, the
ShowStep/SaveStep cadence, the ShowData table (:1658-1732) and the
SaveContactAngle file (:1735-1771).

CPU: the sweep values, the contact-angle file name and the option errors.
GPU: a two-value sweep on the 24x6x20 CP-PRW walled box against the FP64
oracle run through the same host loop.  The table's numbers must agree to
the PLAIN FP64 parity tolerance (1e-11 relative on densities and mass) and
to 1e-5 degrees on the contact angles; the column formats (decimals per
column, sticky fixed/precision state) must match the reference's exactly.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

RUNNER = os.path.join(ROOT, "3dcpmpmodel_gb300", "cpmp_run")


@pytest.fixture(scope="module")
def runner(cpmp):
    assert os.path.exists(RUNNER), "cpmp_run was not built"
    return RUNNER


def dry(runner, *args):
    out = subprocess.run([runner, "--dry-run", *args], capture_output=True, text=True, check=True).stdout
    lines = dict(line.split(" ", 1) for line in out.strip().splitlines())
    return lines


def test_reference_sweep_values(runner):
    # for (BasePt = -0.08; BasePt <= -0.015; BasePt += 0.005), in double
    want, b = [], -0.08
    while b <= -0.015:
        want.append(b)
        b += 0.005
    got = [float(v) for v in dry(runner)["basept"].split()]
    assert got == want and len(got) == 14
    got = [float(v) for v in dry(runner, "--basept-from", "0.1", "--basept-to", "0.13",
                                  "--basept-step", "0.01")["basept"].split()]
    want, b = [], 0.1
    while b <= 0.13:
        want.append(b)
        b += 0.01
    assert got == want


def test_contact_angle_file_name(runner):
    d = dry(runner)
    assert d["contact_angle_file"] == "data/CPPRW_MRT_Tau=0.8_FIELD64x64x64_ContactAngle_R60.0_Tr0.7.txt"
    d = dry(runner, "--model", "CP_RKS", "--tau", "1.0", "--tr", "0.75", "--dx", "512", "--dy", "512", "--dz", "512",
            "--radius", "100", "--out-dir", "out")
    assert d["contact_angle_file"] == "out/%s_MRT_Tau=%2.1f_FIELD%dx%dx%d_ContactAngle_R%3.1f_Tr%3.1f.txt" % (
        "CPRKS", 1.0, 512, 512, 512, 100.0, 0.75)


def test_bad_options_exit_2(runner):
    for args in (["--bogus"], ["--storage", "f8"], ["--showstep", "0"], ["--dx"]):
        r = subprocess.run([runner, "--dry-run", *args], capture_output=True, text=True)
        assert r.returncode == 2, args


ROW = re.compile(r"^\s*(\d+)    (-?\d+\.\d{12})    (-?\d+\.\d{16})    (-?\d+\.\d{16})    (-?\d+\.\d{16})    "
                 r"(-?\d+\.\d{6})    (-?\d+\.\d{6})    (-?\d+\.\d{6})    (-?\d+\.\d{6})    (-?\d+\.\d{6})    "
                 r"(-?\d+\.\d{6})    (\d+)$")


@pytest.mark.gpu
def test_sweep_against_oracle_host_loop(runner, cpmp, oracle_mod, tmp_path):
    O = oracle_mod
    kw = dict(dx=24, dy=6, dz=20, radius=6.0, width=4.0)
    sweep = [-0.04, -0.03]
    allstep, show = 40, 20
    r = subprocess.run([runner, "--dx", "24", "--dy", "6", "--dz", "20", "--radius", "6", "--width", "4",
                        "--storage", "f64", "--scheme", "plain", "--allstep", str(allstep), "--showstep", str(show),
                        "--savestep", str(show), "--basept", ",".join(map(str, sweep)), "--out-dir",
                        str(tmp_path), "--ca-header"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = r.stdout.splitlines()
    # the first BasePt prints in the default stream format, later ones in the
    # fixed/precision-6 state ShowData left behind
    assert out[0] == "Now the BasePt = -0.04"
    assert "Now the BasePt = -0.030000" in out
    assert out.count("NowStep    Mass    Den(DX/2 , 0 , 3)    Den(DX/2, DY/2/8, 3)    Den(DX/2, DY/2/4, 3)    "
                     "MaxSpeed    CaLeft    CaRight    CaCap    XLeft    XRight    StepTime") == 2
    rows = [ROW.match(line) for line in out]
    rows = [[float(x) for x in m.groups()] for m in rows if m]
    assert [int(x[0]) for x in rows] == [0, 20, 40, 0, 20, 40]

    # the same host loop over the FP64 oracle
    co = cpmp.coexistence(O.MP_CPPRW, 0.7)  # the densities the driver resolves
    g, l = co["den_g"], co["den_l"]
    st = O.State(O.Setup(base_pt=sweep[0], **kw), g, l).init()
    A, B, Tc, Rc, T = st.s.constants()
    DX, DY, DZ = kw["dx"], kw["dy"], kw["dz"]
    I = lambda i, j, k: (i * DY + j) * DZ + k  # noqa: E731
    want, ca = [], dict(ca_left=0, ca_right=0, ca_cap=0, x_left=0, x_right=0)
    ca_rows = []
    for bp in sweep:
        st.p.base_pt = bp
        for step in range(0, allstep + 1, show):
            if step:
                st.step(show)
                c = st.contact_angle()
                if c["ca_left"] == 0 and c["ca_right"] == 0:  # no crossing: CaCap is kept
                    c["ca_cap"] = ca["ca_cap"]
                ca = c
            mass, vmax, _ = st.mass()
            d = [st.dens[I(DX // 2, j, 3)] / Rc for j in (0, DY // 2 // 8, DY // 2 // 4)]
            want.append([step, mass, *d, vmax, ca["ca_left"], ca["ca_right"], ca["ca_cap"], ca["x_left"],
                         ca["x_right"]])
        ca_rows.append([kw["radius"], bp, allstep, ca["ca_left"], ca["ca_right"], ca["ca_cap"], ca["x_left"],
                        ca["x_right"]])
    got = np.array([x[:11] for x in rows])
    want = np.array(want)
    assert np.array_equal(got[:, 0], want[:, 0])
    np.testing.assert_allclose(got[:, 1], want[:, 1], rtol=1e-11, atol=2e-12)  # mass, 12 decimals printed
    np.testing.assert_allclose(got[:, 2:5], want[:, 2:5], rtol=1e-11, atol=1e-15)
    np.testing.assert_allclose(got[:, 5:], want[:, 5:], rtol=0, atol=1e-5)  # printed to 6 decimals

    files = os.listdir(tmp_path)
    # ContactAngle's x-z slice file, last written at the end of the sweep
    assert "XZ_-0.040000.txt" in files and "XZ_-0.030000.txt" in files
    xz = open(os.path.join(tmp_path, "XZ_-0.030000.txt")).read().splitlines()
    assert xz[0] == "i   j   Den" and len(xz) == 1 + DX * DZ
    v = np.array([[float(t) for t in line.split()] for line in xz[1:]])
    assert np.array_equal(v[:, 0], np.tile(np.arange(DX), DZ)) and np.array_equal(v[:, 1], np.repeat(np.arange(DZ), DX))
    want_slice = np.array([st.dens[I(i, DY // 2, k)] for k in range(DZ) for i in range(DX)])
    np.testing.assert_allclose(v[:, 2], want_slice, rtol=6e-6)  # 6 significant digits
    name = "CPPRW_MRT_Tau=0.8_FIELD24x6x20_ContactAngle_R6.0_Tr0.7.txt"
    assert name in files
    lines = open(os.path.join(tmp_path, name)).read().splitlines()
    assert lines[0] == "Droprad  BasePt  NowStep  CaLeft  CaRight  CaCap  XLeft  XRight  "
    assert len(lines) == 1 + len(sweep)
    for line, w in zip(lines[1:], ca_rows):
        v = [float(x) for x in line.split()]
        assert line.endswith("  ") and line.startswith("6  ")
        np.testing.assert_allclose(v, w, rtol=2e-6, atol=1e-5)  # default stream precision: 6 digits
