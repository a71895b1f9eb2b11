"""Storage-precision record on the 512^3 wetting box.

    python -m 3dcpmpmodel_gb300.precision_record [--grid 512] [--steps 2000]

The 512^3 precision configuration: z walls (three solid layers at each end;
the droplet sits on the bottom one), CP-RKS at T/Tc = 0.75, a droplet of
radius 100 in the reference's placement (DX/2, DY/2, R+2), tanh width 10,
the reference's Initialize() defaults otherwise (K = 0.2, kappa = 0.001,
tau = 0.8, wall potential -0.04).  The same initial field -- SetFlowField's
droplet, evaluated in FP64 and rounded to each form's storage -- runs
`--steps` steps as PLAIN FP64 (the oracle form: the reference's kernel
sequence in double precision, about 54 GB at 512^3), FUSED FP32 and FUSED
FP16 (populations stored as FP16 deviations from the rest equilibrium of
their writer, FP32 arithmetic).  Against the FP64 run: the largest and the
root-mean-square relative error of rho over fluid nodes, the largest and RMS
velocity error relative to the largest FP64 speed, and the contact angles of
the reference's method (ContactAngle, FluidCuda.cu:557-734: left, right and
spherical-cap angle on the slice j = DY/2).  Prints one JSON line.
"""
import argparse
import importlib
import json
import time

import numpy as np


def run(cp, grid, scheme, storage, steps):
    s = cp.Solver(dx=grid, dy=grid, dz=grid, model=205, tr=0.75, wall_mode=1, base_pt=-0.04, k=0.2,
                  ka=0.001, tau=0.8, scheme=cp.SCHEME[scheme], storage=cp.STORE[storage])
    s.set_flow_field(radius=100.0 * grid / 512, width=10.0)
    if scheme == "fused":
        s.autotune()
    t = time.perf_counter()
    s.step(steps)
    s.sync()
    dt = time.perf_counter() - t
    d = s.reduce()
    rho = s.get("rho")
    u = s.get("u").reshape(3, -1)
    typ = s.get("type")
    s.close()
    return dict(rho=rho, u=u, type=typ, diag=d, seconds=dt)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--steps", type=int, default=2000)
    args = ap.parse_args()
    cp = importlib.import_module("3dcpmpmodel_gb300")
    out = {"grid": [args.grid] * 3, "eos": "RKS", "tr": 0.75, "steps": args.steps, "forms": {}}
    ref = run(cp, args.grid, "plain", "f64", args.steps)
    fluid = ref["type"] == 1
    r64 = ref["rho"][fluid]
    u64 = ref["u"][:, fluid]
    umax = float(np.sqrt((u64 ** 2).sum(0)).max())
    keys = ("ca_left", "ca_right", "ca_cap", "x_left", "x_right", "mass", "max_speed")
    out["forms"]["plain_f64"] = {k: ref["diag"][k] for k in keys}
    out["forms"]["plain_f64"]["seconds"] = round(ref["seconds"], 2)
    out["u_max_f64"] = umax
    del ref
    for storage in ("f32", "f16"):
        r = run(cp, args.grid, "fused", storage, args.steps)
        dr = np.abs(r["rho"][fluid] - r64) / r64
        du = np.sqrt(((r["u"][:, fluid] - u64) ** 2).sum(0)) / umax
        rec = {k: r["diag"][k] for k in keys}
        rec.update(rho_max_rel=float(dr.max()), rho_rms_rel=float(np.sqrt((dr ** 2).mean())),
                   u_max_rel=float(du.max()), u_rms_rel=float(np.sqrt((du ** 2).mean())),
                   seconds=round(r["seconds"], 2))
        for k in ("ca_left", "ca_right", "ca_cap"):
            rec[f"d_{k}"] = rec[k] - out["forms"]["plain_f64"][k]
        out["forms"][f"fused_{storage}"] = rec
        del r
    print(json.dumps(out))


if __name__ == "__main__":
    main()
