"""Contact-angle sweep: FP16-storage FUSED solver against the FP64 PLAIN one.

    python -m 3dcpmpmodel_gb300.contact_sweep [--steps 20000] [--out DIR]

128 x 128 x 96 box with z walls, CP-PRW at T/Tc = 0.7 (the reference's
Initialize() defaults otherwise), a hemispherical droplet of radius 30
centred on the first fluid layer (64, 64, 3), and seven wall potentials
spanning about 30 to 150 degrees in this set-up (the reference's calibration
list, FluidCuda.cu:128, is for another droplet size).  Each BasePt starts from a fresh droplet and runs
`--steps` steps through cpmp_run, the driver with the reference's host loop;
the contact angles are read back from the SaveContactAngle files the two runs
write.  The reference's method needs an interface crossing in the solid row
k = 2 and reports 0 where there is none (strongly hydrophobic walls, films);
so every run is also measured by a circle fit: the mid-density contour of the
x-z slice j = 64 (the XZ_<BasePt>.txt file the driver writes), points at
least four nodes above the wall, least-squares circle, angle where the circle
meets the half-way wall plane z = 2.5.  Prints one JSON line: per BasePt the
FP64 and FP16 angles (left, right, spherical cap, circle fit), the largest
differences, and each run's wall time.
"""
import argparse
import json
import os
import subprocess
import math
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
RUNNER = os.path.join(HERE, "cpmp_run")
# wall potentials for about 30, 50, 70, 90, 110, 130 and 150 degrees in this
# set-up (spherical-cap angle), picked from a scan of FUSED FP32 runs of the
# same box over -0.055 .. 0.105 (below -0.05 the droplet spreads into a film,
# from 0.1 it leaves the wall)
BASEPTS = [-0.044, -0.03, -0.01, 0.01, 0.037, 0.063, 0.09]


def coexistence():
    """Lattice-unit (den_g, den_l) the driver resolves for CP-PRW at 0.7."""
    import importlib
    co = importlib.import_module("3dcpmpmodel_gb300").coexistence(202, 0.7)
    return co["den_g"], co["den_l"]


def run(storage, scheme, steps, out_dir, extra=(), basepts=None):
    cmd = [RUNNER, "--dx", "128", "--dy", "128", "--dz", "96", "--radius", "30", "--width", "5",
           "--centre", "64,64,3", "--storage", storage, "--scheme", scheme, "--allstep", str(steps),
           "--showstep", str(steps), "--savestep", str(steps),
           "--basept", ",".join(map(str, basepts or BASEPTS)),
           "--reinit", "--out-dir", out_dir, *extra]
    t = time.perf_counter()
    r = subprocess.run(cmd, capture_output=True, text=True)
    dt = time.perf_counter() - t
    if r.returncode != 0:
        raise RuntimeError(f"cpmp_run failed ({r.returncode}): {r.stderr.strip()}")
    name = [f for f in os.listdir(out_dir) if f.endswith(".txt") and "ContactAngle" in f]
    assert len(name) == 1, name
    rows = []
    for line in open(os.path.join(out_dir, name[0])):
        v = line.split()
        rows.append(dict(base_pt=float(v[1]), ca_left=float(v[3]), ca_right=float(v[4]), ca_cap=float(v[5])))
    return rows, dt


def circle_fit_angle(xz_path, den_mid, wall=2.5, above=4.0):
    """Contact angle (degrees) of the circle fitted to the mid-density contour
    of an XZ slice file, measured through the liquid at the plane z = wall."""
    v = np.loadtxt(xz_path, skiprows=1)
    nx, nz = int(v[:, 0].max()) + 1, int(v[:, 1].max()) + 1
    d = v[:, 2].reshape(nz, nx).T  # d[i, k]
    pts = []
    for k in range(nz):  # crossings along x in each row
        row = d[:, k]
        for i in range(nx - 1):
            a, b = row[i], row[i + 1]
            if (a - den_mid) * (b - den_mid) < 0:
                pts.append((i + (a - den_mid) / (a - b), k))
    for i in range(nx):  # crossings along z in each column
        col = d[i, :]
        for k in range(nz - 1):
            a, b = col[k], col[k + 1]
            if (a - den_mid) * (b - den_mid) < 0:
                pts.append((i, k + (a - den_mid) / (a - b)))
    p = np.array([q for q in pts if q[1] >= wall + above])
    if len(p) < 8:
        return None
    x, z = p[:, 0], p[:, 1]
    A = np.column_stack([x, z, np.ones_like(x)])
    sol, *_ = np.linalg.lstsq(A, -(x * x + z * z), rcond=None)
    xc, zc = -sol[0] / 2, -sol[1] / 2
    R = math.sqrt(max(xc * xc + zc * zc - sol[2], 0.0))
    c = (wall - zc) / R
    if not -1.0 <= c <= 1.0:
        return None
    return math.degrees(math.acos(c))


def has_line(row):
    """The reference's method found interface crossings on both sides; without
    them its CaCap keeps the previous run's value (a global in the
    reference), which is not reported."""
    return row["ca_left"] != 0.0 and row["ca_right"] != 0.0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--out", default=None, help="keep the contact-angle files here")
    ap.add_argument("--basept", default=None, help="comma-separated wall potentials (default: the calibrated seven)")
    ap.add_argument("--only", default=None, help="one form, e.g. f32:fused, to scan wall potentials")
    a = ap.parse_args()
    basepts = [float(v) for v in a.basept.split(",")] if a.basept else BASEPTS
    base = a.out or tempfile.mkdtemp(prefix="contact_sweep_")
    co = coexistence()
    mid = (co[0] + co[1]) / 2
    if a.only:
        storage, scheme = a.only.split(":")
        d = os.path.join(base, f"{storage}_{scheme}")
        os.makedirs(d, exist_ok=True)
        rows, t = run(storage, scheme, a.steps, d, basepts=basepts)
        for r in rows:
            r["circle_fit"] = circle_fit_angle(os.path.join(d, "XZ_%f.txt" % r["base_pt"]), mid)
            if not has_line(r):
                r["ca_cap"] = None
        print(json.dumps(dict(form=a.only, steps=a.steps, rows=rows, wall_s=t)))
        return
    d64, d16 = os.path.join(base, "f64_plain"), os.path.join(base, "f16_fused")
    for d in (d64, d16):
        os.makedirs(d, exist_ok=True)
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
    r64, t64 = run("f64", "plain", a.steps, d64, basepts=basepts)
    r16, t16 = run("f16", "fused", a.steps, d16, basepts=basepts)
    per, worst, worst_fit = [], 0.0, 0.0
    for x, y in zip(r64, r16):
        line = has_line(x) and has_line(y)
        fit = [circle_fit_angle(os.path.join(d, "XZ_%f.txt" % x["base_pt"]), mid) for d in (d64, d16)]
        if line:
            diff = {k: y[k] - x[k] for k in ("ca_left", "ca_right", "ca_cap")}
            worst = max(worst, max(abs(v) for v in diff.values()))
        if None not in fit:
            worst_fit = max(worst_fit, abs(fit[1] - fit[0]))
        cols = lambda r: [r["ca_left"], r["ca_right"], r["ca_cap"] if line else None]  # noqa: E731
        per.append(dict(base_pt=x["base_pt"], contact_line=line, fp64=cols(x) + [fit[0]], fp16=cols(y) + [fit[1]]))
    print(json.dumps(dict(metric="max |contact angle FP16 fused - FP64 plain|", value=worst, unit="degree",
                          circle_fit_max_diff=worst_fit, steps=a.steps, grid=[128, 128, 96], model="CP_PRW",
                          tr=0.7, radius=30, columns=["CaLeft", "CaRight", "CaCap", "circle fit"],
                          runs_without_contact_line=sum(1 for p in per if not p["contact_line"]),
                          per_base_pt=per, wall_s=dict(f64_plain=t64, f16_fused=t16))))


if __name__ == "__main__":
    main()
