"""CPU: the C-ABI library loads, exports every entry point include/cpmp.h
declares, matches the ctypes struct layouts, and its host-side logic
(defaults, validation, EOS constants, coexistence) works without a GPU."""
import ctypes as C
import json
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADER = os.path.join(ROOT, "include", "cpmp.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cpmp_\w+)\s*\(", src)))


def test_every_declared_symbol_is_exported(cpmp):
    lib = cpmp.lib()
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", cpmp._abi.LIB_PATH], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r" T (cpmp_\w+)", out))
    assert set(names) <= exported
    assert set(cpmp._abi.SIGNATURES) <= exported


def test_struct_layout_matches_header(cpmp):
    prog = r'''
#include <stdio.h>
#include <stddef.h>
#include "cpmp.h"
int main(void){
 printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(cpmp_params), offsetof(cpmp_params, ts),
        offsetof(cpmp_params, cocurve_dir), offsetof(cpmp_params, device), sizeof(cpmp_droplet),
        sizeof(cpmp_diag), offsetof(cpmp_diag, step), sizeof(cpmp_impact), offsetof(cpmp_impact, drop_velocity));
 return 0;}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(prog)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.dirname(HEADER), c, "-o", exe], check=True)
        vals = [int(v) for v in subprocess.run([exe], capture_output=True, text=True).stdout.split()]
    P, D, G = cpmp.Params, cpmp.Droplet, cpmp.Diag
    assert vals == [C.sizeof(P), P.ts.offset, P.cocurve_dir.offset, P.device.offset, C.sizeof(D),
                    C.sizeof(G), G.step.offset, C.sizeof(cpmp.Impact), cpmp.Impact.drop_velocity.offset]


def test_defaults_are_the_reference_initialize(cpmp):
    p = cpmp.default_params()
    # FluidCuda.cu:121-131 and the compile-time switches at :1-7
    assert (p.model, p.tr, p.k, p.ka, p.k1, p.k2, p.tau) == (202, 0.7, 0.2, 0.001, 0.0, 0.0, 0.8)
    assert (p.base_pt, p.wall_mode, p.lap_order, p.complex_bc, p.ts_from_tau) == (-0.08, 1, 5, 1, 1)


def test_parameter_validation_without_gpu(cpmp):
    for kw in (dict(lap_order=6), dict(dx=0), dict(model=101), dict(tau=0.5),
               dict(scheme=0, storage=2), dict(scheme=1, storage=0), dict(wall_mode=3),
               dict(dz=5)):
        with pytest.raises(cpmp.CpmpError) as e:
            cpmp.Solver(**kw)
        assert e.value.status in (1, 7), kw


def test_library_coexistence_matches_maxwell_oracle(cpmp, oracle_mod):
    O = oracle_mod
    for model in (201, 202, 203, 204, 205, 206):
        for tr in (0.6, 0.7, 0.85):
            lib = cpmp.coexistence(model, tr)
            g, l = O.coexistence(model, tr)
            A, B, Tc, Rc = O.eos_constants(model, tr)
            assert abs(lib["den_g"] / g - 1) < 1e-9 and abs(lib["den_l"] / l - 1) < 1e-9
            assert (lib["A"], lib["B"], lib["Tc"], lib["Rc"]) == pytest.approx((A, B, Tc, Rc), rel=1e-15)
    # CS with a = 0.5, b = 4 (the periodic-box configuration)
    lib = cpmp.coexistence(206, 0.85, eos_a=0.5, eos_b=4.0)
    g, l = O.coexistence(206, 0.85, 0.5, 4.0)
    assert abs(lib["den_g"] / g - 1) < 1e-9 and lib["Tc"] == pytest.approx(0.09432870 / 2, rel=1e-15)


def test_library_reads_cocurve_tables_like_setmultiphase(cpmp):
    rows = json.load(open(os.path.join(GOLDEN, "cocurve_rows.json")))
    with tempfile.TemporaryDirectory() as d:
        for tag, by_tr in rows.items():
            with open(os.path.join(d, f"CoCurve_{tag}_2.txt"), "w") as f:
                f.write("T   DenGas   DenLiquid \n")
                for trs, (g, l) in by_tr.items():
                    f.write(f"{float(trs):.11f}    {g!r}    {l!r}\n")
        for tag, model in (("PRW", 202), ("VDW", 201), ("CSE", 206), ("RKS", 205)):
            g, l = rows[tag]["0.700"]
            r = cpmp.coexistence(model, 0.7, cocurve_dir=d)
            assert r["den_g"] == g * r["Rc"] and r["den_l"] == l * r["Rc"]
        with pytest.raises(cpmp.CpmpError) as e:
            cpmp.coexistence(202, 0.703, cocurve_dir=d)
        assert e.value.status == 4


def test_create_without_gpu_fails_cleanly(cpmp):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(cpmp.CpmpError) as e:
        cpmp.Solver(dx=16, dy=16, dz=16)
    assert e.value.status in (2, 3)


def test_integration_cpp_binding_compiles_and_links(cpmp, tmp_path):
    """The C++ binding a maintainer of the reference would add
    (csrc/reference_host_binding.cpp) compiles against include/cpmp.h and links
    to libcpmp.so, with the reference's compile-time grid and step counts as
    macros."""
    import shutil
    if not shutil.which("g++"):
        pytest.skip("no host C++ compiler")
    src = os.path.join(ROOT, "3dcpmpmodel_gb300", "csrc", "reference_host_binding.cpp")
    libdir = os.path.join(ROOT, "3dcpmpmodel_gb300")
    r = subprocess.run(["g++", "-O1", "-DDX=64", "-DDY=64", "-DDZ=64", "-DAllStep=100", "-DShowStep=10",
                        src, "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lcpmp",
                        f"-Wl,-rpath,{libdir}", "-o", str(tmp_path / "host")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.parametrize("kw,status,text", [
    (dict(dx=0, dy=8, dz=8), 1, "grid dimensions"),
    (dict(dx=4096, dy=4096, dz=2048), 1, "grid too large"),
    (dict(dx=16, dy=16, dz=7, wall_mode=1), 1, "dz >= 8"),
    (dict(dx=16, dy=16, dz=16, lap_order=9), 1, "lap_order"),
    (dict(dx=16, dy=16, dz=16, scheme=0, storage=2), 7, "PLAIN scheme"),
    (dict(dx=2048, dy=2048, dz=1024, scheme=1, storage=2), 7, "32 bits"),
    (dict(dx=16, dy=16, dz=16, scheme=1, storage=0), 7, "FUSED scheme stores"),
    (dict(dx=16, dy=16, dz=16, tau=0.5), 1, "tau"),
])
def test_create_rejects_invalid_parameters(cpmp, kw, status, text):
    """cpmp_create validates the parameter set before touching the device:
    the same errors on a machine without a GPU."""
    p = cpmp.default_params(**kw)  # scheme 0 PLAIN / 1 FUSED; storage 0 f64, 1 f32, 2 f16, 3 bf16
    h = C.c_void_p()
    rc = cpmp.lib().cpmp_create(C.byref(p), C.byref(h))
    assert rc == status and text.encode() in cpmp.lib().cpmp_last_error()
