"""GPU: batched boxes (one persistent fused-collide launch per step) equal
individual runs of the same boxes bit for bit when the tile is the same."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOXES = [
    dict(dx=40, dy=16, dz=28, model=202, tr=0.7, base_pt=-0.04, radius=8.0),
    dict(dx=32, dy=24, dz=32, model=201, tr=0.8, base_pt=0.02, radius=9.0),
    dict(dx=48, dy=8, dz=40, model=206, tr=0.75, base_pt=0.0, radius=10.0, eos_a=0.5, eos_b=4.0),
]


def params_of(cpmp, box, storage):
    kw = {k: v for k, v in box.items() if k != "radius"}
    return cpmp.default_params(scheme=cpmp.SCHEME["fused"], storage=cpmp.STORE[storage], **kw)


@pytest.mark.parametrize("storage", ["f16", "f32"])
def test_batch_equals_individual_runs(cpmp, storage):
    tile = (4, 32, 8)
    b = cpmp.Batch([params_of(cpmp, box, storage) for box in BOXES])
    b.set_tile(*tile)
    for s, box in zip(b.boxes, BOXES):
        s.set_flow_field(radius=box["radius"], width=4.0)
    b.step(1)   # a single step
    b.step(10)  # graph replays of step pairs
    b.step(3)   # odd remainder
    b.sync()
    for s, box in zip(b.boxes, BOXES):
        ref = cpmp.Solver(params=params_of(cpmp, box, storage))
        ref.set_flow_field(radius=box["radius"], width=4.0)
        ref.set_tile(*tile)
        ref.step(14)
        assert np.array_equal(s.get("rho"), ref.get("rho"))
        assert np.array_equal(s.get("dist"), ref.get("dist"))
        d, dr = s.reduce(), ref.reduce()
        assert d["step"] == 14 and not d["nonfinite"]
        # the collide's per-box max |MV| (the batch keeps one slot per box and parity)
        assert d["max_speed"] > 0 and d["max_speed"] == dr["max_speed"]
        assert d["mass"] == dr["mass"]
        ref.close()
    b.close()


def test_batch_one_persistent_collide_launch_per_step(cpmp):
    b = cpmp.Batch([params_of(cpmp, box, "f16") for box in BOXES])
    for s, box in zip(b.boxes, BOXES):
        s.set_flow_field(radius=box["radius"], width=4.0)
    b.kernel_timing(True)
    b.step(4)
    b.sync()
    kt = b.kernel_times()
    b.kernel_timing(False)
    assert kt["fused_collide"][0] == 4 and kt["density"][0] == 4
    with pytest.raises(cpmp.CpmpError):
        b.boxes[0].step(1)  # boxes are stepped through the batch only
    b.close()


def test_batch_autotune_keeps_the_state(cpmp):
    b = cpmp.Batch([params_of(cpmp, box, "f16") for box in BOXES])
    for s, box in zip(b.boxes, BOXES):
        s.set_flow_field(radius=box["radius"], width=4.0)
    b.step(3)
    before = [s.get("dist") for s in b.boxes]
    speeds = [s.reduce()["max_speed"] for s in b.boxes]
    t = b.autotune()
    assert t["tile_y"] > 0 and t["step_ms"] > 0
    for s, d, v in zip(b.boxes, before, speeds):
        assert np.array_equal(s.get("dist"), d)
        assert s.reduce()["max_speed"] == v  # the scratch steps leave the diagnostics alone
    b.step(2)
    b.close()
