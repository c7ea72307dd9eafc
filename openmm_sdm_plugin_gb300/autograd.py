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
  fixed u' (FP64), from which dU/dlambda of a thermodynamic-integration
  schedule follows by the chain rule.

The backward is one library call (sdm_backward_device: one kernel, fixed-
order FP64 sums); ``bias_partials`` and ``bias_partials_device`` below are
the same partial derivatives in plain Python and torch, kept as references.

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


def bias_partials_device(methods, be, l1, l2, alpha, u0):
    """bias_partials for every replica at once, on the device: (R,) tensors
    d W / d {lambda1, lambda2, alpha, u0, w0} at fixed u' = be.  methods: (R,)
    bias method ids."""
    zero = torch.zeros_like(be)
    ilog = methods == ILOGISTIC
    pos = ilog & (alpha > 0)
    a = torch.where(pos, alpha, torch.ones_like(alpha))
    x = -a * (be - u0)
    e = torch.where(pos, torch.exp(x), zero)
    ee = 1.0 + e
    L = torch.log(ee)
    dl = l2 - l1
    d_l1 = torch.where(pos, -L / a, zero)
    d_l2 = torch.where(pos, L / a + be, torch.where(ilog, be, zero))
    d_u0 = torch.where(pos, dl * e / ee, zero)
    d_al = torch.where(pos, dl * (-L / (a * a) - (be - u0) * e / (a * ee)), zero)
    d_w0 = torch.where(ilog | (methods == QUADRATIC), torch.ones_like(be), zero)
    return d_l1, d_l2, d_al, d_u0, d_w0


class SDMEngine:
    """One system with R replicas on the GPU, prepared for differentiation.

    The displaced set D (particles with a nonzero displacement at creation)
    is fixed; its charges/sigmas/epsilons and the displacement values are
    the differentiable inputs.  Everything after the parameter pushes stays
    on the device and on the caller's current CUDA stream: the evaluation
    (a captured graph), the state-1 forces, the adjoint sums and the
    backward contractions.  Parameters are pushed to the library (a host
    call that synchronises) only when an input tensor changed: a different
    tensor object or a new in-place version."""

    def __init__(self, system: SDMSystem, device: int = 0):
        self.system = system
        self.h = capi.Handle([system], device=device)
        self.dev = torch.device("cuda", device)
        self.R = system.replicas
        self.n = system.n
        d = np.asarray(system.displacement, np.float64).reshape(-1, 3)
        self.D = np.nonzero(np.any(d != 0.0, axis=1))[0].astype(np.int32)
        self.base = [dataclass_copy(p) for p in system.params]
        self._q = np.asarray(system.charge, np.float64).copy()
        self._s = np.asarray(system.sigma, np.float64).copy()
        self._e = np.asarray(system.epsilon, np.float64).copy()
        self._d = d.copy()
        f64 = dict(dtype=torch.float64, device=self.dev)
        self.methods = torch.tensor([p.bias_method for p in self.base], dtype=torch.int64, device=self.dev)
        # persistent device buffers: the captured evaluation graph keys on their addresses
        self.x = torch.zeros((self.R * self.n, 3), **f64)
        self.res = torch.zeros((self.R, capi.NRESULTS), **f64)
        self.F = torch.zeros((self.R * self.n, 3), **f64)
        self.F1 = torch.zeros((self.R * self.n, 3), **f64)
        self.G = torch.zeros((6 * self.h.num_perturbed(),), **f64)
        self._seen = {}

    def close(self):
        self.h.close()

    def _changed(self, name, t) -> bool:
        last = self._seen.get(name)
        if last is not None and last[0] is t and last[1] == t._version:
            return False
        self._seen[name] = (t, t._version)
        return True

    def _push(self, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
        host = lambda t: t.detach().to("cpu", torch.float64).numpy()
        if self._changed("qD", qD) | self._changed("sD", sD) | self._changed("eD", eD):
            q, sg, ep = host(qD), host(sD), host(eD)
            if not (np.array_equal(q, self._q[self.D]) and np.array_equal(sg, self._s[self.D])
                    and np.array_equal(ep, self._e[self.D])):
                self._q[self.D], self._s[self.D], self._e[self.D] = q, sg, ep
                self.h.set_particle_params(0, self.D, q, sg, ep)
        if self._changed("d", d):
            dd = host(d).reshape(-1, 3)
            if not np.array_equal(dd, self._d):
                nz = np.nonzero(np.any(dd != 0.0, axis=1))[0]
                if not np.array_equal(nz, self.D):
                    raise ValueError("the set of displaced particles must not change")
                self._d = dd.copy()
                self.h.set_displacement(0, dd)
        names = ("lambda1", "lambda2", "alpha", "u0", "w0")
        vals = (lam1, lam2, alpha, u0, w0)
        if any([self._changed(k, v) for k, v in zip(names, vals)]):
            hv = [host(v).reshape(-1) for v in vals]
            for r in range(self.R):
                p = dataclass_copy(self.base[r])
                p.lambda1, p.lambda2, p.alpha, p.u0, p.w0 = (float(v[r]) for v in hv)
                p.noneq = 0
                self.h.set_params(r, p.as_array())

    def run(self, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
        """Forward on the device: (U, s, F, F1, G, results) as device tensors
        (views of the engine's buffers: copy what must outlive the next call)."""
        self._push(qD, sD, eD, d, lam1, lam2, alpha, u0, w0)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        self.x.copy_(x.detach().reshape(-1, 3))
        self.h.evaluate_device(self.x.data_ptr(), self.res.data_ptr(), self.F.data_ptr(), stream)
        self.h.state_forces_device(0, self.F1.data_ptr(), stream)
        self.h.adjoint_device(self.G.data_ptr(), stream)
        res = self.res
        return (res[:, capi.R_EPOT], res[:, capi.R_S], self.F.view(self.R, self.n, 3),
                self.F1.view(self.R, self.n, 3), self.G.view(self.R, -1, 2, 3), res)

    def backward(self, g, res, F, F1, G, eD, prm, need):
        """All gradients from dL/dU = g (R,) in one library call
        (sdm_backward_device) on the current stream: grad_x (R, N, 3),
        grad_d (N, 3), grad_p (nD, 3: charge, sigma, epsilon) and the bias
        rows (5, R: lambda1, lambda2, alpha, u0, w0).  `need` = which of
        (x, parameters, displacement, bias) to compute; the others are None."""
        f64 = dict(dtype=torch.float64, device=self.dev)
        gx = torch.empty((self.R, self.n, 3), **f64) if need[0] else None
        gp = torch.empty((len(self.D), 3), **f64) if need[1] else None
        gd = torch.empty((self.n, 3), **f64) if need[2] else None
        gb = torch.empty((5, self.R), **f64) if need[3] else None
        ptr = lambda t: t.data_ptr() if t is not None else 0
        self.h.backward_device(g.data_ptr(), res.data_ptr(), F.data_ptr(), F1.data_ptr(), G.data_ptr(),
                               eD.data_ptr(), prm.data_ptr(), ptr(gx), ptr(gd), ptr(gp), ptr(gb),
                               torch.cuda.current_stream(self.dev).cuda_stream)
        return gx, gp, gd, gb


def dataclass_copy(p):
    import dataclasses
    return dataclasses.replace(p)


class SDMPotential(torch.autograd.Function):
    """U (R,) = SDMPotential.apply(engine, x, qD, sD, eD, d, lambda1, lambda2, alpha, u0, w0)

    x: (R, N, 3); qD, sD, eD: (nD,); d: (N, 3); lambda1..w0: (R,).  All FP64,
    on any device (the result and the gradients come back on x's device).
    Differentiable in every tensor input."""

    @staticmethod
    def forward(ctx, engine: SDMEngine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
        U, s, F, F1, G, res = engine.run(x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0)
        on = lambda t: t.detach().to(engine.dev, torch.float64).reshape(-1)
        prm = torch.stack([on(lam1), on(lam2), on(alpha), on(u0)])   # (4, R) of this evaluation
        ctx.save_for_backward(res.clone(), F.clone(), F1.clone(), G.clone(),
                              on(eD).contiguous(), prm)
        ctx.engine = engine
        ctx.devs = (x.device, qD.device, d.device, lam1.device)
        return U.clone().to(x.device)

    @staticmethod
    def backward(ctx, gU):
        res, F, F1, G, eD, prm = ctx.saved_tensors
        xdev, pdev, ddev, ldev = ctx.devs
        n = ctx.needs_input_grad
        need = (n[1], n[2] or n[3] or n[4], n[5], any(n[6:]))
        g = gU.detach().to(res.device, torch.float64).contiguous()
        gx, gp, gd, gb = ctx.engine.backward(g, res, F, F1, G, eD, prm, need)
        col = lambda t, k, dev: t[:, k].to(dev) if t is not None else None
        row = lambda k: gb[k].to(ldev) if gb is not None else None
        return (None, gx.to(xdev) if gx is not None else None, col(gp, 0, pdev), col(gp, 1, pdev),
                col(gp, 2, pdev), gd.to(ddev) if gd is not None else None,
                row(0), row(1), row(2), row(3), row(4))


def sdm_potential(engine: SDMEngine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0):
    return SDMPotential.apply(engine, x, qD, sD, eD, d, lam1, lam2, alpha, u0, w0)
