"""Run a few steps of one box on the GPU (for profilers and quick checks).

    python -m 3dcpmpmodel_gb300.probe [--grid 256,256,128] [--scheme fused]
                                      [--storage f16] [--steps 6] [--model 205] [--tr 0.75]

Prints the mass after the run.  Exits non-zero on any library error.
"""
import argparse
import importlib


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="256,256,128")
    ap.add_argument("--scheme", choices=["fused", "plain"], default="fused")
    ap.add_argument("--storage", choices=["f16", "bf16", "f32", "f64"], default="f16")
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--model", type=int, default=205)
    ap.add_argument("--tr", type=float, default=0.75)
    ap.add_argument("--radius", type=float, default=40.0)
    ap.add_argument("--tile", default="", help="ty,tz,xl for the fused kernel")
    a = ap.parse_args()
    cp = importlib.import_module("3dcpmpmodel_gb300")
    dx, dy, dz = (int(v) for v in a.grid.split(","))
    s = cp.Solver(dx=dx, dy=dy, dz=dz, model=a.model, tr=a.tr, base_pt=-0.04,
                  scheme=cp.SCHEME[a.scheme], storage=cp.STORE[a.storage])
    s.set_flow_field(radius=a.radius, width=10.0)
    if a.tile:
        s.set_tile(*(int(v) for v in a.tile.split(",")))
    s.step(a.steps)
    s.sync()
    print("mass", s.reduce()["mass"])
    s.close()


if __name__ == "__main__":
    main()
