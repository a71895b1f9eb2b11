"""Time the reference's own CUDA step on this GPU (baseline measurement).

    python oracle/ref_gpu_bench.py [--grid 480,480,480] [--steps 10] [--warmup 3] [--radius 100] [--width 10]

BASELINE MEASUREMENT ONLY.  Compiles oracle/ref_gpu_bench.cu against the
reference kernels generated into oracle/_ref/ by oracle/build_ref.py (the
reference's Initialize() defaults: CP-PRW at T/Tc 0.7, K 0.2, Ka 0.001,
tau 0.8; droplet radius (default 100) and width (default 10) at the
reference's placement;
BasePt -0.04; coexistence densities from the committed CoCurve rows), runs it
and prints its JSON line.  The reference indexes populations with 32-bit int
(f*DXYZ + I), so the grid must satisfy 19*N < 2^31 (N <= 113M nodes; 480^3 is
the largest cube that fits).
"""
import argparse
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_ref  # noqa: E402
import oracle as O  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", default="480,480,480")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--radius", type=float, default=100.0)
    ap.add_argument("--width", type=float, default=10.0)
    a = ap.parse_args()
    dx, dy, dz = (int(v) for v in a.grid.split(","))
    if 19 * dx * dy * dz >= 2 ** 31 - 1:
        sys.exit("grid too large for the reference's 32-bit population index")
    exe = build_ref.build_gpu_bench(dx, dy, dz)
    A, B, Tc, Rc = O.eos_constants(O.MP_CPPRW, 0.7)
    rows = json.load(open(os.path.join(os.path.dirname(HERE), "tests", "golden", "cocurve_rows.json")))
    g, l = rows["PRW"]["0.700"]
    args = [a.steps, a.warmup, 0.2, A, B, 0.7 * Tc, 0.001, g * Rc, l * Rc, -0.04, a.radius, a.width, 0.8]
    r = subprocess.run([exe, *[repr(float(x)) if not isinstance(x, int) else str(x) for x in args]],
                       capture_output=True, text=True)
    if r.returncode != 0:
        sys.exit(f"reference GPU step failed ({r.returncode}): {r.stderr.strip()}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out.update(impl="reference CUDA kernels (FluidCuda.cu:188-463), FP64, 64-thread blocks",
               model="CP_PRW", tr=0.7, nodes=dx * dy * dz, radius=a.radius)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
