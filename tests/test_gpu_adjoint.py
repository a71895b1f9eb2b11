"""GPU: the adjoint step.  Gradients of J = sum_fluid (rho^T - target)^2 with
respect to the bottom wall field and kappa, checked against central finite
differences (h = 1e-3, FP64, relative error <= 1e-3) and between FP32 and
FP64 adjoints; the checkpoint interval must not change the result."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def smooth_field(nx, ny, seed, amp, mean):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.fftfreq(ny)[None, :]
    filt = np.exp(-(kx ** 2 + ky ** 2) * (2 * np.pi * 3.0) ** 2 / 2)
    w = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    w = (w - w.mean()) / (w.std() + 1e-30)
    return mean + amp * w


def setup(cpmp, storage):
    p = cpmp.default_params(dx=24, dy=16, dz=20, model=206, tr=0.8, eos_a=0.5, eos_b=4.0, ka=0.01, tau=1.0,
                            base_pt=0.0, scheme=cpmp.SCHEME["plain"], storage=cpmp.STORE[storage])
    return {"params": p, "droplet": dict(radius=6.0, width=3.0, centre=(12.0, 8.0, 3.0))}


STEPS = 60


@pytest.fixture(scope="module")
def problem(cpmp):
    ag = importlib.import_module("3dcpmpmodel_gb300.autograd")
    st = setup(cpmp, "f64")
    w_target = smooth_field(24, 16, 1, 0.02, 0.0)
    w0 = smooth_field(24, 16, 2, 0.02, 0.0)
    target = ag.final_density(st, w_target, 0.01, STEPS)
    return ag, st, w0, target


def test_adjoint_matches_central_differences_fp64(cpmp, problem):
    ag, st, w0, target = problem
    s = ag._solver(st, w0, 0.01)
    loss, gw, gk = s.adjoint(STEPS, target)
    s.close()
    assert loss == pytest.approx(ag.run_loss(st, w0, 0.01, STEPS, target), rel=1e-12)
    h = 1e-3
    # kappa
    fd = (ag.run_loss(st, w0, 0.01 + h, STEPS, target) - ag.run_loss(st, w0, 0.01 - h, STEPS, target)) / (2 * h)
    assert gk == pytest.approx(fd, rel=1e-3)
    # the wall columns with the largest gradient (under the contact line)
    g2 = gw[: 24 * 16].reshape(24, 16)
    idx = np.argsort(np.abs(g2).ravel())[::-1][:4]
    for c in idx:
        i, j = divmod(int(c), 16)
        wp, wm = w0.copy(), w0.copy()
        wp[i, j] += h
        wm[i, j] -= h
        fd = (ag.run_loss(st, wp, 0.01, STEPS, target) - ag.run_loss(st, wm, 0.01, STEPS, target)) / (2 * h)
        assert g2[i, j] == pytest.approx(fd, rel=1e-3), (i, j)


def test_fp32_adjoint_agrees_with_fp64(cpmp, problem):
    ag, st64, w0, target = problem
    s = ag._solver(st64, w0, 0.01)
    _, g64, k64 = s.adjoint(STEPS, target)
    s.close()
    st32 = setup(cpmp, "f32")
    s = ag._solver(st32, w0, 0.01)
    _, g32, k32 = s.adjoint(STEPS, target)
    s.close()
    assert np.linalg.norm(g32 - g64) <= 1e-3 * np.linalg.norm(g64)
    assert k32 == pytest.approx(k64, rel=1e-3)


def test_checkpoint_interval_does_not_change_gradients(cpmp, problem):
    ag, st, w0, target = problem
    out = []
    for every in (1, 0, 7, STEPS):
        s = ag._solver(st, w0, 0.01)
        out.append(s.adjoint(STEPS, target, every))
        s.close()
    for loss, gw, gk in out[1:]:
        assert loss == out[0][0] and gk == out[0][2]
        assert np.array_equal(gw, out[0][1])


def test_autograd_function(cpmp, problem):
    torch = pytest.importorskip("torch")
    ag, st, w0, target = problem
    w = torch.tensor(w0, dtype=torch.float64, requires_grad=True)
    k = torch.tensor(0.01, dtype=torch.float64, requires_grad=True)
    J = ag.WallKappaLoss.apply(w, k, st, STEPS, target)
    (2.0 * J).backward()
    s = ag._solver(st, w0, 0.01)
    loss, gw, gk = s.adjoint(STEPS, target)
    s.close()
    assert float(J.detach()) == pytest.approx(loss, rel=1e-14)
    assert np.allclose(w.grad.numpy(), 2.0 * gw[: 24 * 16].reshape(24, 16), rtol=0, atol=0)
    assert float(k.grad) == pytest.approx(2.0 * gk, rel=1e-14)
