"""Differentiable SDM potential: ``torch.autograd.Function`` over the CUDA path.

For every replica r the potential is U_r = U0 + W(u'(u)) (the reference's
PotEnergy without the group-1 term, platforms/reference/src/ReferenceSDMKernels.cpp:283).
With s = W'(u') du'/du:

* d U / d theta_k = (1 - s) dU0/dtheta_k + s dU1/dtheta_k for the charge,
  sigma and epsilon of every displaced (ligand) particle k -- the sums
  dU_state/dtheta_k come from the hand-written adjoint kernel (sdm_adjoint);
* d U / d d_i = -s F1_i for the displacement map (F1: forces at x + d);
* d U / d x_i = -F_i (the mixed force);
* d U / d {lambda1, lambda2, alpha, u0, w0} = partial derivatives of W at
  fixed u' (FP64, below), from which dU/dlambda of a thermodynamic-
  integration schedule follows by the chain rule.

The reference's only derivative is the non-equilibrium dW/dlambda
(ReferenceSDMKernels.cpp:289-302, which sets dW/dalpha to 0); here dW/dalpha
is the exact derivative of the integrated logistic bias.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import capi
from .systems import ILOGISTIC, QUADRATIC, SDMParams, SDMSystem


def bias_partials(p: SDMParams, be: float) -> dict:
    """Partial derivatives of W(u') at fixed u' = be with respect to the bias
    parameters (ILogistic: lambda1, lambda2, alpha, u0, w0; Quadratic: gamma,
    wb, w0; Linear: lambdac)."""
    out = dict(lambda1=0.0, lambda2=0.0, alpha=0.0, u0=0.0, w0=0.0, gamma=0.0, wb=0.0, lambdac=0.0)
    if p.bias_method == ILOGISTIC:
        a, l1, l2 = p.alpha, p.lambda1, p.lambda2
        out["w0"] = 1.0
        if a > 0:
            x = -a * (be - p.u0)
            e = math.exp(x)
            ee = 1.0 + e
            L = math.log(ee)
            out["lambda1"] = -L / a
            out["lambda2"] = L / a + be
            out["u0"] = (l2 - l1) * e / ee
            out["alpha"] = (l2 - l1) * (-L / (a * a) - (be - p.u0) * e / (a * ee))
        else:
            out["lambda2"] = be
    elif p.bias_method == QUADRATIC:
        out["gamma"] = 0.5 * be * be
        out["wb"] = be
        out["w0"] = 1.0
    else:
        out["lambdac"] = be
    return out


class SDMEngine:
    """One system with R replicas on the GPU, prepared for differentiation.

    The displaced set D (particles with a nonzero displacement at creation)
    is fixed; its charges/sigmas/epsilons and the displacement values are
    the differentiable inputs."""

    def __init__(self, system: SDMSystem, device: int = 0):
        self.system = system
        self.h = capi.Handle([system], device=device)
        self.R = system.replicas
        self.n = system.n
        d = np.asarray(system.displacement, np.float64).reshape(-1, 3)
        self.D = np.nonzero(np.any(d != 0.0, axis=1))[0].astype(np.int32)
        self.base = [dataclass_copy(p) for p in system.params]
        self._q = np.asarray(system.charge, np.float64).copy()
        self._s = np.asarray(system.sigma, np.float64).copy()
        self._e = np.asarray(system.epsilon, np.float64).copy()
        self._d = d.copy()

    def close(self):
        self.h.close()

    def run(self, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
        """Forward + everything the backward needs (FP64 numpy arrays)."""
        if not (np.array_equal(qD, self._q[self.D]) and np.array_equal(sD, self._s[self.D])
                and np.array_equal(eD, self._e[self.D])):
            self._q[self.D], self._s[self.D], self._e[self.D] = qD, sD, eD
            self.h.set_particle_params(0, self.D, qD, sD, eD)
        d = np.asarray(d, np.float64).reshape(-1, 3)
        if not np.array_equal(d, self._d):
            nz = np.nonzero(np.any(d != 0.0, axis=1))[0]
            if not np.array_equal(nz, self.D):
                raise ValueError("the set of displaced particles must not change")
            self._d = d.copy()
            self.h.set_displacement(0, d)
        params = []
        for r in range(self.R):
            p = dataclass_copy(self.base[r])
            p.lambda1, p.lambda2, p.alpha, p.u0, p.w0 = (float(lam1[r]), float(lam2[r]), float(alpha[r]),
                                                        float(u0[r]), float(w0[r]))
            p.noneq = 0
            self.h.set_params(r, p.as_array())
            params.append(p)
        res, F = self.h.evaluate(np.asarray(x, np.float64).reshape(-1, 3))
        F0, F1 = self.h.state_forces()
        G = self.h.adjoint(self.R * len(self.D)).reshape(self.R, len(self.D), 2, 3)
        return res, F.reshape(self.R, self.n, 3), F1.reshape(self.R, self.n, 3), G, params


def dataclass_copy(p):
    import dataclasses
    return dataclasses.replace(p)


class SDMPotential(torch.autograd.Function):
    """U (R,) = SDMPotential.apply(engine, x, qD, sD, eD, d, lambda1, lambda2, alpha, u0, w0)

    x: (R, N, 3); qD, sD, eD: (nD,); d: (N, 3); lambda1..w0: (R,).  All FP64.
    Differentiable in every tensor input."""

    @staticmethod
    def forward(ctx, engine: SDMEngine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
        cpu = lambda t: t.detach().to("cpu", torch.float64).numpy()
        res, F, F1, G, params = engine.run(cpu(x), cpu(qD), cpu(sD), cpu(eD), cpu(d), cpu(lam1), cpu(lam2),
                                           cpu(alpha), cpu(u0), cpu(w0))
        s = res[:, capi.R_S]
        part = [bias_partials(p, res[r, capi.R_BINDE]) for r, p in enumerate(params)]
        ctx.save_for_backward(*(torch.from_numpy(np.ascontiguousarray(v)) for v in
                                (s, F, F1, G, cpu(eD))))
        ctx.partials = part
        ctx.dev = x.device
        return torch.from_numpy(res[:, capi.R_EPOT].copy()).to(x.device)

    @staticmethod
    def backward(ctx, gU):
        s, F, F1, G, eD = ctx.saved_tensors
        g = gU.detach().to("cpu", torch.float64)
        w = torch.stack([(1.0 - s), s], dim=1)                   # (R, 2) state weights
        gD = torch.einsum("r,rs,rksc->kc", g, w, G)              # (nD, 3)
        grad_q = gD[:, 0]
        grad_s = gD[:, 1]
        grad_e = torch.where(eD > 0, gD[:, 2] / (2.0 * eD.clamp_min(1e-300)), torch.zeros_like(eD))
        grad_d = -torch.einsum("r,r,rnc->nc", g, s, F1)
        grad_x = -g[:, None, None] * F
        pl = lambda key: g * torch.tensor([p[key] for p in ctx.partials], dtype=torch.float64)
        dev = ctx.dev
        to = lambda t: t.to(dev)
        return (None, to(grad_x), to(grad_q), to(grad_s), to(grad_e), to(grad_d), to(pl("lambda1")),
                to(pl("lambda2")), to(pl("alpha")), to(pl("u0")), to(pl("w0")))


def sdm_potential(engine: SDMEngine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
    return SDMPotential.apply(engine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0)
