"""Test harness of the differentiation form (test infrastructure only; the
library's entry points are ph_derivs and ph_adjoint).

* Derivs: a torch.autograd.Function around one derivs evaluation on the GPU
  (forward: upload + ph_derivs, backward: ph_adjoint at the same state).
* Rollout: global-timestep leapfrog steps (step_leapfrog.f90:91-760 with one
  velocity iteration, the reference's tolv > 1e2 setting) driven from Python
  with GPU derivs, and their reverse pass with checkpoints: states are kept
  every `ckpt` steps, each segment is recomputed forward and then reversed
  step by step, one ph_adjoint per force evaluation (neighbour lists and pair
  terms are recomputed inside it, nothing else is stored).
"""
from __future__ import annotations

import numpy as np
import torch

from phantom_gb300 import capi


def evaluate(dev: capi.Context, xyzh: np.ndarray, vxyzu: np.ndarray, want_divv: bool = False):
    """One derivs at (xyzh, vxyzu): fxyzu (N,4) and the wrapped positions
    with the converged smoothing lengths (N,4) (and div v, float32)."""
    n = xyzh.shape[0]
    dev.upload(xyzh, vxyzu)
    dev.derivs(1, 0.0)
    xo = np.empty((n, 4)); vo = np.empty((n, 4)); fo = np.empty((n, 4))
    dv = np.empty(n, np.float32)
    dev.download_state(xo, vo, None, fo, None, dv)
    return (fo, xo, dv) if want_divv else (fo, xo)


class Derivs(torch.autograd.Function):
    """fxyzu = derivs(xyzh, vxyzu) with its vector-Jacobian product from
    ph_adjoint (gradient slot of h is zero: h follows from the positions)."""

    @staticmethod
    def forward(ctx, xyzh, vxyzu, dev):
        f, _ = evaluate(dev, xyzh.detach().numpy(), vxyzu.detach().numpy())
        ctx.dev = dev
        ctx.save_for_backward(xyzh, vxyzu)
        return torch.from_numpy(f)

    @staticmethod
    def backward(ctx, gf):
        xyzh, vxyzu = ctx.saved_tensors
        dev = ctx.dev
        dev.upload(xyzh.detach().numpy(), vxyzu.detach().numpy())
        gx, gv = dev.adjoint(gf.detach().numpy())
        return torch.from_numpy(gx), torch.from_numpy(gv), None


class Rollout:
    """K leapfrog steps with fixed timesteps dts from (x0, v0) and the
    gradient of L = sum w . a_K (the accelerations of the last evaluation)."""

    def __init__(self, dev: capi.Context, cfg: dict, dts, ckpt: int = 4):
        if cfg.get("nalpha", 0):
            # alpha evolves with d(div v)/dt of the positions and velocities;
            # the adjoint holds it fixed within one evaluation only
            raise NotImplementedError("rollout gradients through the Cullen-Dehnen switch are not built")
        self.dev, self.dts, self.ckpt = dev, list(dts), ckpt
        self.nv = 3 if cfg.get("isothermal") else 4
        self.m, self.hfact = cfg["massoftype"], cfg["hfact"]
        self.grav = bool(cfg.get("gravity"))

    def _step(self, x, v, f, dv, dt):
        nv = self.nv
        vs = v.copy(); vs[:, :nv] += 0.5 * dt * f[:, :nv]       # kick
        x1 = x.copy(); x1[:, :3] += dt * vs[:, :3]              # drift
        # h predicted from div v (step_leapfrog.f90 predict_sph): it seeds the
        # h-rho solve and builds the tree, whose node hmax decides the
        # self-gravity walk, so with self-gravity the reverse pass uploads
        # this point again (without, the converged h)
        h = x[:, 3]
        t = self.hfact / np.abs(h)
        rho = self.m * (t * t * t)
        x1[:, 3] = h - dt * (-h / (3.0 * rho)) * rho * dv.astype(np.float64)
        vp = vs.copy(); vp[:, :nv] += 0.5 * dt * f[:, :nv]      # predicted v
        f1, x1w, dv1 = evaluate(self.dev, x1, vp, True)          # derivs at the new positions
        v1 = vs.copy(); v1[:, :nv] += 0.5 * dt * f1[:, :nv]     # kick
        return x1w, v1, f1, dv1, (x1 if self.grav else x1w, vp)

    def forward(self, x0, v0):
        f0, xw, dv0 = evaluate(self.dev, x0, v0, True)
        x, v, f, dv = xw, v0.copy(), f0, dv0
        self.checkpoints = {}
        for n, dt in enumerate(self.dts):
            if n % self.ckpt == 0:
                self.checkpoints[n] = (x.copy(), v.copy(), f.copy(), dv.copy())
            x, v, f, dv, _ = self._step(x, v, f, dv, dt)
        self.x0 = x0.copy() if self.grav else xw
        return f

    def loss_and_grad(self, x0, v0, w):
        fK = self.forward(x0, v0)
        L = float(np.sum(w * fK[:, :3]))
        n = x0.shape[0]
        nv = self.nv
        xb = np.zeros((n, 4)); vb = np.zeros((n, 4)); fb = np.zeros((n, 4)); fb[:, :3] = w
        K = len(self.dts)
        for c0 in sorted(self.checkpoints, reverse=True):
            # recompute the segment forward from its checkpoint
            x, v, f, dv = (a.copy() for a in self.checkpoints[c0])
            seg = []
            for m in range(c0, min(c0 + self.ckpt, K)):
                x1, v1, f1, dv1, ev = self._step(x, v, f, dv, self.dts[m])
                seg.append((self.dts[m], ev))
                x, v, f, dv = x1, v1, f1, dv1
            for dt, (x1, vp) in reversed(seg):
                vsb = vb.copy()
                f1b = fb.copy(); f1b[:, :nv] += 0.5 * dt * vb[:, :nv]
                self.dev.upload(x1, vp)
                gx, gv = self.dev.adjoint(f1b)
                x1b = xb + gx
                vsb += gv
                fnb = np.zeros((n, 4)); fnb[:, :nv] += 0.5 * dt * gv[:, :nv]
                vsb[:, :3] += dt * x1b[:, :3]
                fnb[:, :nv] += 0.5 * dt * vsb[:, :nv]
                xb, vb, fb = x1b, vsb, fnb
        # initial evaluation f0 = F(x0, v0)
        self.dev.upload(self.x0, v0)
        gx, gv = self.dev.adjoint(fb)
        xb = xb + gx
        vb = vb + gv
        xb[:, 3] = 0.0
        return L, xb, vb
