"""GPU: cpmp_mass_noalloc, the reduction entry point that allocates nothing.

It exists for callers that cannot call cudaMalloc (code embedded in a host or
framework that owns device memory, or stream-ordered pipelines where an
allocation would synchronise the device).  They pass their own device buffers;
the entry point keeps its block partials in a fixed 24 KB device array inside
the library.  This file is collected last so that a failure here comes after
every other test has run; it passes alone in a fresh process as well.

Checked, each on two calls in a row (two different states): its three
outputs equal those of cpmp_reduce on the same PLAIN-scheme fields, to 1e-12
relative (the reductions run the same kernels in the same order, so they
normally agree bit for bit), on a grid that fills whole 256-node blocks and
on one of 273 280 nodes, which is not a multiple of 256 and needs more than
one pass of the 1024 partial blocks; without an MV field the maximum speed is
0 and the mass unchanged.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(lib, typ, rho, mv, n, out, torch):
    out.fill_(-1.0)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.cpmp_mass_noalloc(C.c_void_p(typ.data_ptr()), C.c_void_p(rho.data_ptr()),
                               None if mv is None else C.c_void_p(mv.data_ptr()), C.c_longlong(n),
                               C.c_void_p(stream), C.c_void_p(out.data_ptr()))
    assert rc == 0, lib.cpmp_last_error()
    torch.cuda.synchronize()
    return out.cpu().tolist()


@pytest.mark.parametrize("dims", [(40, 16, 28), (70, 64, 61), (67, 45, 93), (128, 128, 120)],
                         ids=["whole_blocks", "ragged", "odd_n_scalar_multipass", "vector_two_group_trips"])
def test_noalloc_reduction_matches_cpmp_reduce(cpmp, dims):
    torch = pytest.importorskip("torch")
    lib = cpmp.lib()
    dx, dy, dz = dims
    s = cpmp.Solver(dx=dx, dy=dy, dz=dz, scheme=cpmp.SCHEME["plain"], storage=cpmp.STORE["f32"],
                    base_pt=-0.04)
    s.set_flow_field(radius=min(dims) / 4.0, width=4.0)
    # the reduction grid has at most 912 blocks of 256 threads; n divisible by
    # 4 takes groups of four nodes, two groups per loop trip where there are
    # more than 2 x 912 x 256 groups, and any other n one node per trip
    if dims == (70, 64, 61):  # a partial last block
        assert s.n % 256 != 0 and s.n % 4 == 0
    if dims == (67, 45, 93):  # the scalar loop, several nodes per thread
        assert s.n % 4 != 0 and s.n > 912 * 256
    if dims == (128, 128, 120):  # the group loop with two groups per trip and a remainder
        assert s.n // 4 > 2 * 912 * 256
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    for call, steps in enumerate((5, 40)):
        s.step(steps)
        ref = s.reduce()
        # the caller's own device buffers (allocated by the test, not the entry point)
        typ = torch.from_numpy(s.get("type")).cuda()
        rho = torch.from_numpy(s.get("rho", np.float32)).cuda()
        mv = torch.from_numpy(s.get("mv", np.float32)).cuda()
        mass, vmax, bad = _call(lib, typ, rho, mv, s.n, out, torch)
        assert mass == pytest.approx(ref["mass"], rel=1e-12), call
        assert vmax == pytest.approx(ref["max_speed"], rel=1e-12, abs=1e-30), call
        assert bad == float(ref["nonfinite"]), call
        mass0, vmax0, bad0 = _call(lib, typ, rho, None, s.n, out, torch)
        assert mass0 == mass and vmax0 == 0.0 and bad0 == bad, call
    # sizes beyond the stated maximum are rejected with a clear error
    rc = lib.cpmp_mass_noalloc(C.c_void_p(typ.data_ptr()), C.c_void_p(rho.data_ptr()), None,
                               C.c_longlong((1 << 34) + 1), None, C.c_void_p(out.data_ptr()))
    assert rc == 8 and b"CPMP_NOALLOC_MAX_NODES" in lib.cpmp_last_error()
    s.close()
