"""Build recipe for oracle/_ref: the reference's kernels compiled for the host.

TEST INFRASTRUCTURE ONLY.  Generates, into oracle/_ref/ (git-ignored):

* ``Common_rt.h``: the reference's Common.h with the grid constants made
  run-time ints.  The only lines changed are the five ``const int`` grid
  declarations (Common.h:25-27 and :33-34); everything else is verbatim.
* ``ref_kernels.inc``: FluidCuda.cu lines 115-116 (the GridIndex/LineIndex
  launch-index macros) and 188-463 (the kernels), verbatim.
* ``ref_impact.inc``: FluidCuda.cu lines 737-783 and 786-898 (the host
  diagnostics ComputeEnergy and Computetangential_velocity), verbatim.

and compiles ``oracle/ref_shim.cpp`` against them into ``oracle/_ref/libref.so``.

Generation needs the reference tree (``--src`` or the CPMP_REFERENCE_SRC
environment variable); compiling needs only the generated files, so a machine
without the reference tree can still build the library from a copied
``_ref/``.
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# location of the reference tree: --src, the CPMP_REFERENCE_SRC environment
# variable, or the read-only mount this recipe reads it from; where none of
# them holds the tree, only an existing generated copy is compiled
DEFAULT_SRC = os.environ.get("CPMP_REFERENCE_SRC") or "/root/reference"

GRID_LINES = {  # Common.h line (1-based) -> expected declaration prefix
    25: "const int DY",
    26: "const int DX",
    27: "const int DZ",
    33: "const int DXYZ",
    34: "const int DXY",
}
INDEX_FIRST, INDEX_LAST = 115, 116
# host diagnostics ComputeEnergy and Computetangential_velocity
IMPACT_RANGES = ((737, 783, "void ComputeEnergy()"), (786, 898, "void Computetangential_velocity()"))
KERNEL_FIRST, KERNEL_LAST = 188, 463


def generate(src: str) -> None:
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(src, "Common.h"), encoding="latin-1") as f:
        common = f.read().split("\n")
    for ln, prefix in GRID_LINES.items():
        line = common[ln - 1]
        if not line.startswith(prefix):
            raise RuntimeError(f"Common.h:{ln} is not the expected grid constant: {line!r}")
        common[ln - 1] = re.sub(r"^const int", "int", line)
    with open(os.path.join(OUT, "Common_rt.h"), "w", encoding="latin-1") as f:
        f.write("\n".join(common))
    with open(os.path.join(src, "FluidCuda.cu"), encoding="latin-1") as f:
        lines = f.read().split("\n")
    index = lines[INDEX_FIRST - 1:INDEX_LAST]
    body = lines[KERNEL_FIRST - 1:KERNEL_LAST]
    if not (index[0].startswith("#define GridIndex") and index[1].startswith("#define LineIndex")
            and any("__global__ void ChemPotential" in l for l in body)):
        raise RuntimeError("FluidCuda.cu layout differs from the expected one")
    body = ["#ifndef GridIndex"] + index + ["#endif"] + body
    with open(os.path.join(OUT, "ref_kernels.inc"), "w", encoding="latin-1") as f:
        f.write("\n".join(body) + "\n")
    impact = []
    for first, last, head in IMPACT_RANGES:
        part = lines[first - 1:last]
        if head not in part[0]:
            raise RuntimeError(f"FluidCuda.cu:{first} is not {head}")
        impact += part
    with open(os.path.join(OUT, "ref_impact.inc"), "w", encoding="latin-1") as f:
        f.write("\n".join(impact) + "\n")


def generate_gpu(src: str) -> None:
    """Common_gpu.h: the reference's Common.h with its grid constants taken
    from the macros REF_DX / REF_DY / REF_DZ (still compile-time constants,
    as in the reference), for oracle/ref_gpu_bench.cu."""
    os.makedirs(OUT, exist_ok=True)
    with open(os.path.join(src, "Common.h"), encoding="latin-1") as f:
        common = f.read().split("\n")
    for ln, axis in ((25, "DY"), (26, "DX"), (27, "DZ")):
        if not common[ln - 1].startswith(f"const int {axis}"):
            raise RuntimeError(f"Common.h:{ln} is not the expected grid constant: {common[ln - 1]!r}")
        common[ln - 1] = f"const int {axis} = REF_{axis};"
    with open(os.path.join(OUT, "Common_gpu.h"), "w", encoding="latin-1") as f:
        f.write("\n".join(common))


def build_gpu_bench(dx: int, dy: int, dz: int) -> str:
    """Compile oracle/ref_gpu_bench.cu for one grid (needs the generated
    oracle/_ref/Common_gpu.h and ref_kernels.inc; nvcc for sm_103a)."""
    out = os.path.join(OUT, f"ref_gpu_bench_{dx}x{dy}x{dz}")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-w",
           f"-DREF_DX={dx}", f"-DREF_DY={dy}", f"-DREF_DZ={dz}", "-I", OUT,
           os.path.join(HERE, "ref_gpu_bench.cu"), "-o", out]
    subprocess.run(cmd, check=True)
    return out


def compile_lib() -> str:
    out = os.path.join(OUT, "libref.so")
    cmd = [
        "g++", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-w",
        "-std=c++17", "-I", OUT, os.path.join(HERE, "ref_shim.cpp"), "-o", out,
    ]
    subprocess.run(cmd, check=True)
    return out


def build_tecplot(src: str = DEFAULT_SRC) -> str | None:
    """The reference's Tecplot writer (ordered_tec.cpp, compiled from the
    reference tree where it lies) behind oracle/tec_ref_driver.cpp."""
    if not src or not os.path.isfile(os.path.join(src, "ordered_tec.cpp")):
        return None
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, "libtecref.so")
    subprocess.run(["g++", "-O2", "-fPIC", "-shared", "-w", "-std=c++17", "-I", src,
                    os.path.join(HERE, "tec_ref_driver.cpp"), os.path.join(src, "ordered_tec.cpp"), "-o", out],
                   check=True)
    return out


def build(src: str = DEFAULT_SRC) -> str | None:
    """Generate (when the reference tree exists) and compile; returns the .so
    path, or None when neither the reference tree nor generated files exist."""
    if src and os.path.isfile(os.path.join(src, "FluidCuda.cu")):
        generate(src)
        generate_gpu(src)
    if not (os.path.isfile(os.path.join(OUT, "Common_rt.h"))
            and os.path.isfile(os.path.join(OUT, "ref_kernels.inc"))):
        return None
    return compile_lib()


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=DEFAULT_SRC)
    a = ap.parse_args()
    p = build(a.src)
    t = build_tecplot(a.src)
    print(p if p else "reference sources unavailable; nothing built", t or "")
    sys.exit(0)
