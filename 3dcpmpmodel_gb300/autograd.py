"""torch.autograd.Function over the library's adjoint step.

``WallKappaLoss.apply(wall, kappa, setup, steps, target)`` returns the loss
J = sum over fluid nodes of (rho^T - target)^2 after ``steps`` steps from a
freshly initialised droplet, as a function of the bottom-wall chemical
potential field ``wall`` (DX x DY) and the interface parameter ``kappa``.
Its backward pass returns dJ/dwall and dJ/dkappa from one adjoint sweep
(sqrt(T) checkpoint-and-recompute) instead of re-running the simulation.

``setup`` is a dict: ``params`` (a Params, PLAIN scheme) and ``droplet``
(keyword arguments of Solver.set_flow_field).  The top wall keeps the
parameters' base_pt.
"""
from __future__ import annotations

import importlib

import numpy as np
import torch

cp = importlib.import_module("3dcpmpmodel_gb300")


def _solver(setup, wall: np.ndarray, kappa: float):
    s = cp.Solver(params=setup["params"])
    full = np.full(2 * s.dx * s.dy, setup["params"].base_pt, dtype=np.float64)
    full[: s.dx * s.dy] = wall.reshape(-1)
    s.set_wall_field(full)
    s.set_kappa(kappa)
    s.set_flow_field(**setup["droplet"])
    return s


def run_loss(setup, wall: np.ndarray, kappa: float, steps: int, target: np.ndarray) -> float:
    """Forward only: the loss of one run (used for finite differences)."""
    s = _solver(setup, wall, kappa)
    s.step(steps)
    rho = s.get("rho")
    fluid = s.get("type") == 1
    d = rho[fluid] - target.reshape(-1)[fluid]
    s.close()
    return float(np.dot(d, d))


def final_density(setup, wall: np.ndarray, kappa: float, steps: int) -> np.ndarray:
    s = _solver(setup, wall, kappa)
    s.step(steps)
    rho = s.get("rho")
    s.close()
    return rho


class WallKappaLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, wall, kappa, setup, steps, target, checkpoint_every=0):
        w = wall.detach().cpu().double().numpy()
        s = _solver(setup, w, float(kappa))
        loss, gw, gk = s.adjoint(int(steps), np.asarray(target, dtype=np.float64), int(checkpoint_every))
        s.close()
        n2 = w.size
        ctx.save_for_backward(torch.from_numpy(gw[:n2].reshape(w.shape)).to(wall.dtype),
                              torch.tensor(gk, dtype=kappa.dtype))
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad_out):
        gw, gk = ctx.saved_tensors
        return grad_out.to(gw.dtype) * gw, grad_out.to(gk.dtype) * gk, None, None, None, None
