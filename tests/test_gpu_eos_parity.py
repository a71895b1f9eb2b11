"""GPU parity of the equations of state and physics options beyond the
golden-fixture cases: every EOS of the parameter surface (VdW, CS, PR-M, RK-E,
RK-S -- the RK-S form at T/Tc 0.75 is the physics of the 512^3 benchmark),
the seven-point Laplacian, the K1/K2 pressure-tensor term and the Laplace-law
probe, each against the FP64 oracle on identical seeded inputs.

The reference itself evaluates only the PR chemical potential
(FluidCuda.cu:453); the oracle's other mu0 forms are pinned by the CoCurve
coexistence tables (tests/test_oracle.py).

Tolerances (relative unless stated; velocities as max |du| / max |u_oracle|):
  PLAIN FP64 vs oracle                           rho 1e-11, u 1e-9, mu 1e-12 absolute
  FUSED FP32 / FP16 vs oracle after 100 steps    rho 5e-6 / 2e-3, u 20x that
  Laplace probe on the same field                1e-12
  FP32 after 1000 steps vs the reference build   see test_fp32_after_1000_steps
"""
import numpy as np
import pytest

from test_gpu_parity import oracle_run, rel_err, solver_for, vel_err

pytestmark = pytest.mark.gpu

BOX = dict(dx=40, dy=16, dz=28, radius=8.0, width=4.0, base_pt=-0.04)
EOS_CASES = {
    "vdw": dict(BOX, model=201, tr=0.75),
    "prm": dict(BOX, model=203, tr=0.7),
    "rke": dict(BOX, model=204, tr=0.75),
    "rks": dict(BOX, model=205, tr=0.75),
    "cs_walled": dict(BOX, model=206, tr=0.8, eos_a=0.5, eos_b=4.0, Ka=0.01, tau=1.0),
}
OPTION_CASES = {
    "lap7": dict(BOX, lap_order=7),
    "k1k2": dict(BOX, K1=0.002, K2=-0.002, tau=1.0),
    "k1k2_lap7_rks": dict(BOX, model=205, tr=0.75, K1=0.002, K2=-0.002, tau=1.0, lap_order=7),
    "simple_bc": dict(BOX, complex_bc=0),
}


def coex(cfg, cpmp):
    co = cpmp.coexistence(cfg.get("model", 202), cfg.get("tr", 0.7), cfg.get("eos_a", 0.0),
                          cfg.get("eos_b", 0.0))
    return co["den_g"], co["den_l"]


@pytest.mark.parametrize("case", sorted(EOS_CASES) + sorted(OPTION_CASES))
def test_plain_fp64_vs_oracle(cpmp, oracle_mod, case):
    cfg = {**EOS_CASES, **OPTION_CASES}[case]
    den = coex(cfg, cpmp)
    st = oracle_run(oracle_mod, cfg, 100, den)
    s = solver_for(cpmp, cfg, storage="f64", den=den)
    s.step(100)
    fluid = st.type == 1
    assert rel_err(s.get("rho"), st.dens, fluid) < 1e-11
    assert vel_err(s.get("u"), (st.vx, st.vy, st.vz), fluid) < 1e-9
    assert vel_err(s.get("force"), (st.fx, st.fy, st.fz), fluid) < 1e-9
    assert float(np.max(np.abs(s.get("mu")[fluid] - st.pote[fluid]))) < 1e-12
    s.close()


@pytest.mark.parametrize("storage,rtol", [("f32", 5e-6), ("f16", 2e-3)])
@pytest.mark.parametrize("case", sorted(EOS_CASES) + sorted(OPTION_CASES))
def test_fused_vs_oracle(cpmp, oracle_mod, case, storage, rtol):
    cfg = {**EOS_CASES, **OPTION_CASES}[case]
    den = coex(cfg, cpmp)
    st = oracle_run(oracle_mod, cfg, 100, den)
    s = solver_for(cpmp, cfg, scheme="fused", storage=storage, den=den)
    s.step(100)
    fluid = st.type == 1
    e = rel_err(s.get("rho"), st.dens, fluid)
    assert e < rtol, e
    assert vel_err(s.get("u"), (st.vx, st.vy, st.vz), fluid) < 20 * rtol
    s.close()


LAPLACE = dict(dx=32, dy=32, dz=32, radius=8.0, width=2.0, wall_mode=0, centre=(16, 16, 16),
               model=206, tr=0.85, eos_a=0.5, eos_b=4.0, Ka=0.01, tau=1.0)


LAPLACE_RKS = dict(dx=32, dy=32, dz=32, radius=9.0, width=3.0, wall_mode=0, centre=(16, 16, 16),
                   model=205, tr=0.75)


@pytest.mark.parametrize("cfg", [LAPLACE, LAPLACE_RKS], ids=["cs", "rks"])
def test_laplace_probe_matches_oracle(cpmp, oracle_mod, cfg):
    """cpmp_reduce's Laplace probe (radius from the mid-density crossing, EOS
    pressure jump, K^2 dp R / 2) equals the oracle's SaveDataOriDen on the
    same density field."""
    den = coex(cfg, cpmp)
    st = oracle_run(oracle_mod, cfg, 200, den)
    s = solver_for(cpmp, cfg, storage="f64", den=den)
    s.set("rho", st.dens)
    d = s.reduce()
    o = st.laplace()
    assert o["lap_r"] > 4.0 and o["lap_dp"] != 0.0
    for k in ("lap_r", "lap_dp", "sigma"):
        assert d["lap_sigma" if k == "sigma" else k] == pytest.approx(o[k], rel=1e-12, abs=1e-15), k
    s.close()


# Measured maximum relative errors of FP32 runs against the FP64 reference
# (walled CP-PRW box below; velocities relative to the largest speed):
#   steps          100      200      500      1000     2000
#   PLAIN rho    1.7e-6   2.6e-6   4.4e-6   5.2e-6   5.3e-6
#   PLAIN u      2.2e-6   1.7e-6   2.6e-6   3.8e-6   4.7e-6
#   FUSED rho    6.7e-7   1.1e-6   2.1e-6   2.3e-6   2.8e-6
#   FUSED u      1.2e-6   1.1e-6   1.9e-6   1.8e-6   1.9e-6
# Both schemes balance mass without a rounded weight (each node's rest
# population is the remainder of its mass moment after the moving
# populations), and the FUSED FP32 force divides by its stencil constants
# with correct rounding, so neither error grows: both meet the 1e-5 bound
# after 1000 steps, asserted here.
FP32_1000 = {"plain": (1e-5, 1e-5), "fused": (1e-5, 1e-5)}


@pytest.mark.parametrize("scheme", ["plain", "fused"])
def test_fp32_after_1000_steps(cpmp, oracle_mod, scheme):
    """FP32 rho and u after 1000 steps against the reference's own kernels
    (their host build, FP64; the FP64 oracle where that build is absent --
    the two are bit-identical)."""
    import os
    O = oracle_mod
    cfg = dict(BOX)
    den = coex(cfg, cpmp)
    backend = "ref" if os.path.exists(O.REF_SO) else "oracle"
    st = O.State(O.Setup(**cfg), den[0], den[1], backend).init()
    st.step(1000)
    s = solver_for(cpmp, cfg, scheme=scheme, storage="f32", den=den)
    s.step(1000)
    fluid = st.type == 1
    rtol, utol = FP32_1000[scheme]
    e = rel_err(s.get("rho"), st.dens, fluid)
    eu = vel_err(s.get("u"), (st.vx, st.vy, st.vz), fluid)
    assert e < rtol, e
    assert eu < utol, eu
    s.close()
