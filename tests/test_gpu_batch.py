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


def test_batch_reduce_equals_each_box_reduce(cpmp):
    """cpmp_batch_reduce (four launches for all boxes) returns each box's
    cpmp_reduce bit for bit: boxes whose node count is a multiple of 4 or not,
    one too small for the contact-angle slice (dx < 8), one larger than the
    mass pass's 912 x 256 threads."""
    boxes = BOXES + [
        dict(dx=33, dy=17, dz=27, model=202, tr=0.7, base_pt=0.02, radius=7.0),  # N odd
        dict(dx=6, dy=12, dz=20, model=201, tr=0.8, base_pt=0.0, radius=4.0),    # no contact angle
        dict(dx=96, dy=64, dz=44, model=202, tr=0.75, base_pt=-0.04, radius=16.0),
    ]
    b = cpmp.Batch([params_of(cpmp, box, "f16") for box in boxes])
    for s, box in zip(b.boxes, boxes):
        s.set_flow_field(radius=box["radius"], width=4.0)
    assert b.boxes[-1].n > 912 * 256 and b.boxes[3].n % 4 != 0
    done = 0
    for steps in (0, 5, 2):  # before any step, then odd and even step counts
        b.step(steps)
        done += steps
        got = b.reduce()
        for s, g in zip(b.boxes, got):
            assert g == s.reduce()
        assert got[0]["step"] == done
    assert got[0]["max_speed"] > 0 and got[5]["mass"] > 0
    b.close()


def test_batch_reduce_reports_the_nonfinite_box(cpmp):
    """A NaN density planted (from the host) on a fluid node of box 1 makes
    cpmp_batch_reduce return CPMP_ERR_NONFINITE naming box 1, with every
    box's diagnostics filled."""
    b = cpmp.Batch([params_of(cpmp, box, "f32") for box in BOXES])
    for s, box in zip(b.boxes, BOXES):
        s.set_flow_field(radius=box["radius"], width=4.0)
    b.step(2)
    rho = b.boxes[1].get("rho")
    rho[len(rho) // 2 + 5] = np.nan
    b.boxes[1].set("rho", rho)
    with pytest.raises(cpmp.CpmpError) as e:
        b.reduce()
    assert e.value.status == 5 and "box 1" in str(e.value)
    got = b.reduce(allow_nonfinite=True)
    assert [g["nonfinite"] for g in got] == [0, 1, 0]
    assert got[0] == b.boxes[0].reduce() and got[2]["mass"] > 0
    b.close()
