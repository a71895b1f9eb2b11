"""Batched droplets against individual runs.

    python -m 3dcpmpmodel_gb300.batch_record [--steps 5000] [--count 96]

The batched wetting set: 96 independent droplet-on-wall boxes (cube edge
uniform in 48..112, EOS drawn from VdW / CS / PR, T/Tc uniform in 0.6-0.9
snapped to the 0.005 grid of the coexistence tables, wall potential uniform in
-0.06..0.15; seed 0), FP16 storage, stepped `--steps` steps by one persistent
collide launch per step (cpmp_batch).  Each box is then run alone as an
ordinary FUSED FP32 handle from the same initial field for the same number of
steps.  Per box: the largest and RMS relative difference of rho over fluid
nodes, and the reference's contact angles (ContactAngle, FluidCuda.cu:557-734)
of both runs where both find a contact line.  Prints one JSON line with the
per-box records and their maxima.
"""
import argparse
import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--count", type=int, default=96)
    a = ap.parse_args()
    sys.path.insert(0, ROOT)
    import bench
    cp = importlib.import_module("3dcpmpmodel_gb300")
    params, drops = bench.c4_params(cp, "f16", 0, a.count)
    b = cp.Batch(params)
    for s, d in zip(b.boxes, drops):
        s.set_flow_field(**d)
    tile = b.autotune()
    t = time.perf_counter()
    b.step(a.steps)
    b.sync()
    t_batch = time.perf_counter() - t
    rows = []
    for i, (s, p, d) in enumerate(zip(b.boxes, params, drops)):
        rb = s.get("rho")
        db = s.reduce(allow_nonfinite=True)
        fluid = s.get("type") == 1
        p32 = cp.default_params(dx=p.dx, dy=p.dy, dz=p.dz, model=p.model, tr=p.tr, base_pt=p.base_pt,
                                scheme=cp.SCHEME["fused"], storage=cp.STORE["f32"])
        ref = cp.Solver(params=p32)
        ref.set_flow_field(**d)
        ref.step(a.steps)
        rr = ref.get("rho")
        dr = ref.reduce(allow_nonfinite=True)
        ref.close()
        rel = np.abs(rb[fluid] - rr[fluid]) / np.abs(rr[fluid])
        line = all(v != 0.0 for v in (db["ca_left"], db["ca_right"], dr["ca_left"], dr["ca_right"]))
        rec = dict(box=i, edge=p.dx, model=p.model, tr=round(p.tr, 3), base_pt=round(p.base_pt, 4),
                   rho_max_rel=float(rel.max()), rho_rms_rel=float(np.sqrt((rel ** 2).mean())),
                   nonfinite=[db["nonfinite"], dr["nonfinite"]], contact_line=line)
        if line:
            rec["ca_fp16_batch"] = [db["ca_left"], db["ca_right"], db["ca_cap"]]
            rec["ca_fp32_alone"] = [dr["ca_left"], dr["ca_right"], dr["ca_cap"]]
            rec["ca_max_diff"] = max(abs(x - y) for x, y in zip(rec["ca_fp16_batch"], rec["ca_fp32_alone"]))
        rows.append(rec)
    with_line = [r for r in rows if r["contact_line"]]
    out = dict(boxes=len(rows), steps=a.steps, tile=tile, batch_seconds=round(t_batch, 2),
               rho_max_rel=max(r["rho_max_rel"] for r in rows),
               rho_rms_rel_max=max(r["rho_rms_rel"] for r in rows),
               boxes_with_contact_line=len(with_line),
               ca_max_diff=max((r["ca_max_diff"] for r in with_line), default=None),
               boxes_nonfinite=sum(1 for r in rows if any(r["nonfinite"])), per_box=rows)
    print(json.dumps(out))
    b.close()


if __name__ == "__main__":
    main()
