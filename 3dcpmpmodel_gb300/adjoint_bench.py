"""Adjoint benchmark on the 96^3 wall-field inversion set-up.

    python -m 3dcpmpmodel_gb300.adjoint_bench [--steps 2000] [--fd]

96^3 box, z walls, CS EOS (a = 0.5, b = 4) at T/Tc = 0.8, droplet radius 24
on the bottom wall, FP32 PLAIN scheme; J = sum_fluid (rho^T - target)^2 with
the target from a different seeded smooth 96 x 96 wall field.  Prints one
JSON line: forward time (the PLAIN FP32 forward the adjoint differentiates,
and the FUSED FP32 forward of the same box), adjoint time (its own
checkpointed forward, the segment replays and the reverse sweep), the ratios, the per-kernel device time
of a separately timed adjoint pass, and with --fd the FP64
adjoint against central differences (h = 1e-3) for kappa and the two largest
wall-gradient entries, plus the FP32-vs-FP64 gradient difference.
"""
import argparse
import importlib
import json
import time

import numpy as np

cp = importlib.import_module("3dcpmpmodel_gb300")
ag = importlib.import_module("3dcpmpmodel_gb300.autograd")


def smooth_field(nx, ny, seed, amp, mean=0.0, corr=8.0):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal((nx, ny))
    kx = np.fft.fftfreq(nx)[:, None]
    ky = np.fft.fftfreq(ny)[None, :]
    filt = np.exp(-(kx ** 2 + ky ** 2) * (2 * np.pi * corr) ** 2 / 2)
    w = np.real(np.fft.ifft2(np.fft.fft2(w) * filt))
    w = (w - w.mean()) / (w.std() + 1e-30)
    return mean + amp * w


def setup(storage, L=96, radius=24.0, scheme="plain"):
    p = cp.default_params(dx=L, dy=L, dz=L, model=206, tr=0.8, eos_a=0.5, eos_b=4.0, ka=0.01, tau=1.0,
                          base_pt=0.0, scheme=cp.SCHEME[scheme], storage=cp.STORE[storage])
    return {"params": p, "droplet": dict(radius=radius, width=4.0, centre=(L / 2, L / 2, 3.0))}


def measure(steps: int = 2000, size: int = 96, fd: bool = False) -> dict:
    """The adjoint-versus-forward record of the wall-field inversion set-up
    (see the module docstring) as a dict."""
    import torch
    a = argparse.Namespace(steps=steps, size=size, fd=fd)
    L = a.size
    st = setup("f32", L, L / 4)
    w_t = smooth_field(L, L, 1, 0.02)
    w0 = smooth_field(L, L, 2, 0.02)
    target = ag.final_density(st, w_t, 0.01, a.steps)

    s = ag._solver(st, w0, 0.01)
    s.step(2)
    s.sync()
    s = ag._solver(st, w0, 0.01)
    ev = torch.cuda.Event
    stream = torch.cuda.ExternalStream(s.stream)
    e0, e1 = ev(enable_timing=True), ev(enable_timing=True)
    e0.record(stream)
    s.step(a.steps)
    e1.record(stream)
    e1.synchronize()
    t_fwd = e0.elapsed_time(e1) / 1e3
    s.close()

    # the fastest forward the library has for this box: the FUSED scheme with
    # FP32 storage (tile picked by the autotuner), same wall field and kappa
    stf = setup("f32", L, L / 4, scheme="fused")
    s = ag._solver(stf, w0, 0.01)
    s.autotune()
    s.step(2)
    s.sync()
    stream = torch.cuda.ExternalStream(s.stream)
    e0, e1 = ev(enable_timing=True), ev(enable_timing=True)
    e0.record(stream)
    s.step(a.steps)
    e1.record(stream)
    e1.synchronize()
    t_fwd_fused = e0.elapsed_time(e1) / 1e3
    s.close()

    s = ag._solver(st, w0, 0.01)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    loss, gw, gk = s.adjoint(a.steps, target)
    t_adj = time.perf_counter() - t0
    s.close()
    # per-kernel device time of one more adjoint pass (events around every launch)
    s = ag._solver(st, w0, 0.01)
    s.kernel_timing(True)
    s.adjoint(a.steps, target)
    kt = {k: {"launches": int(v[0]), "ms": round(v[1], 3)} for k, v in s.kernel_times().items()}
    s.close()
    out = {"metric": "adjoint time / forward time", "value": round(t_adj / t_fwd, 3),
           "forward_s": round(t_fwd, 4), "adjoint_s": round(t_adj, 4),
           "forward_fused_f32_s": round(t_fwd_fused, 4),
           "adjoint_over_fused_forward": round(t_adj / t_fwd_fused, 3),
           "backward_over_forward": round((t_adj - t_fwd) / t_fwd, 3),
           "config": {"grid": [L, L, L], "steps": a.steps, "storage": "f32", "checkpoint_every": "ceil(sqrt(T))"},
           "loss": loss, "grad_kappa": gk, "grad_wall_norm": float(np.linalg.norm(gw)),
           "kernel_ms_timed_pass": kt}
    if a.fd:
        st64 = setup("f64", L, L / 4)
        target64 = target
        s = ag._solver(st64, w0, 0.01)
        loss64, gw64, gk64 = s.adjoint(a.steps, target64)
        s.close()
        h = 1e-3
        fd_k = (ag.run_loss(st64, w0, 0.01 + h, a.steps, target64) -
                ag.run_loss(st64, w0, 0.01 - h, a.steps, target64)) / (2 * h)
        g2 = gw64[: L * L].reshape(L, L)
        checks = {"kappa": {"adjoint": gk64, "fd": fd_k, "rel_err": abs(gk64 - fd_k) / abs(fd_k)}}
        for c in np.argsort(np.abs(g2).ravel())[::-1][:2]:
            i, j = divmod(int(c), L)
            wp, wm = w0.copy(), w0.copy()
            wp[i, j] += h
            wm[i, j] -= h
            fd = (ag.run_loss(st64, wp, 0.01, a.steps, target64) - ag.run_loss(st64, wm, 0.01, a.steps, target64)) / (2 * h)
            checks[f"wall[{i},{j}]"] = {"adjoint": g2[i, j], "fd": fd, "rel_err": abs(g2[i, j] - fd) / abs(fd)}
        out["fd_fp64"] = checks
        out["fp32_vs_fp64_grad_rel_l2"] = float(np.linalg.norm(gw - gw64) / np.linalg.norm(gw64))
        out["fp32_vs_fp64_kappa_rel"] = abs(gk - gk64) / abs(gk64)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--size", type=int, default=96)
    ap.add_argument("--fd", action="store_true")
    a = ap.parse_args()
    print(json.dumps(measure(a.steps, a.size, a.fd)))


if __name__ == "__main__":
    main()
