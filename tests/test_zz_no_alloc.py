"""GPU: cpmp_mass_noalloc, the reduction entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (code embedded in a host or
framework that owns device memory, or stream-ordered pipelines where an
allocation would synchronise the device).  They pass their own device buffers;
the entry point keeps its block partials in a fixed 24 KB device array inside
the library.  This file is collected last so that a failure here comes after
every other test has run; it passes alone in a fresh process as well.

Checked: on two calls in a row (two different states) its three outputs equal
those of cpmp_reduce on the same fields, to 1e-12 relative (the reductions run
the same kernels in the same order, so they normally agree bit for bit).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_reduction_matches_cpmp_reduce(cpmp):
    torch = pytest.importorskip("torch")
    lib = cpmp.lib()
    s = cpmp.Solver(dx=40, dy=16, dz=28, scheme=cpmp.SCHEME["plain"], storage=cpmp.STORE["f32"],
                    base_pt=-0.04)
    s.set_flow_field(radius=8.0, width=4.0)
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    for call, steps in enumerate((5, 40)):
        s.step(steps)
        ref = s.reduce()
        # the caller's own device buffers (allocated by the test, not the entry point)
        typ = torch.from_numpy(s.get("type")).cuda()
        rho = torch.from_numpy(s.get("rho", np.float32)).cuda()
        mv = torch.from_numpy(s.get("mv", np.float32)).cuda()
        out.fill_(-1.0)
        torch.cuda.synchronize()
        stream = torch.cuda.current_stream().cuda_stream
        rc = lib.cpmp_mass_noalloc(C.c_void_p(typ.data_ptr()), C.c_void_p(rho.data_ptr()),
                                   C.c_void_p(mv.data_ptr()), C.c_longlong(s.n), C.c_void_p(stream),
                                   C.c_void_p(out.data_ptr()))
        assert rc == 0, lib.cpmp_last_error()
        torch.cuda.synchronize()
        mass, vmax, bad = out.cpu().tolist()
        assert mass == pytest.approx(ref["mass"], rel=1e-12), call
        assert vmax == pytest.approx(ref["max_speed"], rel=1e-12, abs=1e-30), call
        assert bad == float(ref["nonfinite"]), call
    # sizes beyond the stated maximum are rejected with a clear error
    rc = lib.cpmp_mass_noalloc(C.c_void_p(typ.data_ptr()), C.c_void_p(rho.data_ptr()), None,
                               C.c_longlong((1 << 34) + 1), None, C.c_void_p(out.data_ptr()))
    assert rc == 8 and b"CPMP_NOALLOC_MAX_NODES" in lib.cpmp_last_error()
    s.close()
