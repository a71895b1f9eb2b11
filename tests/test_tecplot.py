"""Tecplot #!TDV112 output against the reference's own writer.

The golden files tests/golden/tec_*.plt were written by the reference's
TEC_FILE classes (ordered_tec.cpp) through oracle/tec_ref_driver.cpp, in the
SaveTask (FluidCuda.cu:901-927) and SaveAllByType (FluidCuda.cu:1032-1092)
layouts, from the state of the prw_walls_complex5 fixture.  The host writer
must reproduce them byte for byte from the same arrays; the device-side
cpmp_write_tecplot must reproduce their layout exactly and their values to
the PLAIN FP64 parity tolerance (1e-11 relative).
"""
import ctypes as C
import os
import struct
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, GOLDEN)
import make_golden  # noqa: E402

SAVETASK = os.path.join(GOLDEN, "tec_FlowField_40.plt")
ALLBYTYPE = os.path.join(GOLDEN, "tec_Field_3D_Nowstep=40.plt")
TEC_DTYPES = {1: np.float32, 2: np.float64, 3: np.int32, 4: np.int16, 5: np.int8}


def read_tdv112(path):
    """Parse one-zone ordered Tecplot binary; returns dict with the raw
    header bytes (everything before the min/max table), names, dims,
    min/max pairs and the variable arrays."""
    b = open(path, "rb").read()
    assert b[:8] == b"#!TDV112"
    o = 8

    def i32():
        nonlocal o
        v = struct.unpack_from("<i", b, o)[0]
        o += 4
        return v

    def f32():
        nonlocal o
        v = struct.unpack_from("<f", b, o)[0]
        o += 4
        return v

    def s():
        chars = []
        while True:
            c = i32()
            if c == 0:
                return "".join(map(chr, chars))
            chars.append(c)

    assert i32() == 1
    i32()
    title = s()
    nvar = i32()
    names = [s() for _ in range(nvar)]
    assert f32() == 299.0
    zone = s()
    o += 4 + 4 + 8 + 4  # parent, strand, time, unused
    assert i32() == 0 and i32() == 0
    o += 8
    dims = (i32(), i32(), i32())
    assert i32() == 0
    assert f32() == 357.0
    assert f32() == 299.0
    types = [i32() for _ in range(nvar)]
    assert (i32(), i32(), i32()) == (0, 0, -1)
    head = b[:o]
    mm = np.frombuffer(b, np.float64, 2 * nvar, o).reshape(nvar, 2)
    o += 16 * nvar
    n = dims[0] * dims[1] * dims[2]
    data = []
    for t in types:
        dt = np.dtype(TEC_DTYPES[t])
        data.append(np.frombuffer(b, dt, n, o))
        o += n * dt.itemsize
    assert o == len(b), "trailing bytes"
    return dict(head=head, title=title, names=names, zone=zone, dims=dims, types=types, minmax=mm, data=data)


def test_golden_files_parse():
    st = read_tdv112(SAVETASK)
    assert st["names"] == ["i", "j", "k", "Density"] and st["title"] == "Model3D"
    assert st["types"] == [4, 4, 4, 2] and st["zone"] == "tec_FlowField_40"
    ab = read_tdv112(ALLBYTYPE)
    assert ab["names"] == ["i", "j", "k", "Ux", "Uy", "Uz", "Density"] and ab["title"] == "Field_3D"
    assert ab["dims"] == (24, 6, 20)
    for v in range(7):
        assert ab["minmax"][v, 0] == ab["data"][v].min() and ab["minmax"][v, 1] == ab["data"][v].max()


def test_host_writer_is_byte_identical(cpmp, tmp_path):
    dims, st, ab = make_golden.tecplot_arrays()
    DX, DY, DZ, LX, LY, LZ, steps = dims
    p = str(tmp_path / "tec_FlowField_40.plt")
    cpmp.tecplot_write(p, "Model3D", "tec_FlowField_40", dict(zip(["i", "j", "k", "Density"], st)), (LZ, LY, LX))
    assert open(p, "rb").read() == open(SAVETASK, "rb").read()
    p = str(tmp_path / "tec_Field_3D_Nowstep=40.plt")
    cpmp.tecplot_write(p, "Field_3D", "tec_Field_3D_Nowstep=40",
                       dict(zip(["i", "j", "k", "Ux", "Uy", "Uz", "Density"], ab)), (DX, DY, DZ))
    assert open(p, "rb").read() == open(ALLBYTYPE, "rb").read()


def test_host_writer_all_types_against_live_reference(cpmp, tmp_path):
    """Every value type, against the reference writer built from its own
    sources (skipped where oracle/_ref/libtecref.so was not built)."""
    so = os.path.join(ROOT, "oracle", "_ref", "libtecref.so")
    if not os.path.exists(so):
        pytest.skip("reference Tecplot writer not built here")
    L = C.CDLL(so)
    rng = np.random.default_rng(7)
    LX, LY, LZ = 3, 4, 5
    n = LX * LY * LZ
    mi = rng.integers(-300, 300, n).astype(np.int16)
    mj = rng.integers(-300, 300, n).astype(np.int16)
    mk = rng.integers(-300, 300, n).astype(np.int16)
    d = rng.standard_normal(n)
    P = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert L.ref_tec_savetask(str(tmp_path).encode(), b"ref_st", LX, LY, LZ, P(mi), P(mj), P(mk), P(d)) == 0
    ours = str(tmp_path / "ours_st.plt")
    cpmp.tecplot_write(ours, "Model3D", "ref_st", {"i": mi, "j": mj, "k": mk, "Density": d}, (LZ, LY, LX))
    assert open(ours, "rb").read() == open(str(tmp_path / "ref_st.plt"), "rb").read()


def test_host_writer_rejects_bad_arguments(cpmp, tmp_path):
    with pytest.raises(Exception):
        cpmp.tecplot_write(str(tmp_path / "x.plt"), "t", "z", {"a": np.zeros(4)}, (0, 1, 1))
    with pytest.raises(Exception):
        cpmp.tecplot_write(str(tmp_path / "no_such_dir" / "x.plt"), "t", "z", {"a": np.zeros(4)}, (4, 1, 1))


@pytest.mark.gpu
@pytest.mark.parametrize("layout,golden", [("savetask", SAVETASK), ("allbytype", ALLBYTYPE)])
def test_device_writer_matches_reference_file(cpmp, tmp_path, layout, golden):
    from test_gpu_parity import load_case, solver_for
    z, kw = load_case("prw_walls_complex5")
    s = solver_for(cpmp, kw, den=(float(z["den_g"]), float(z["den_l"])))
    s.step(int(z["steps"]))
    s.sync()
    p = str(tmp_path / os.path.basename(golden))
    dimv = cpmp.dim_velocity(kw["radius"], make_golden.TEC_DIAMETER, kw.get("tau", 0.8))
    assert dimv == make_golden.dim_velocity(kw["radius"], make_golden.TEC_DIAMETER, kw.get("tau", 0.8))
    s.write_tecplot(p, layout, decimate=5, reference_stride=True, vel_scale=dimv)
    ours, ref = read_tdv112(p), read_tdv112(golden)
    assert ours["head"] == ref["head"]
    np.testing.assert_allclose(ours["minmax"], ref["minmax"], rtol=1e-11, atol=1e-13)
    for a, b in zip(ours["data"], ref["data"]):
        if a.dtype.kind in "iu":
            assert np.array_equal(a, b)
        else:
            # gas nodes carry the -2 marker in both; the liquid/gas split is
            # the same because no density lies within 1e-11 of the midpoint
            np.testing.assert_allclose(a, b, rtol=1e-11, atol=1e-13)
