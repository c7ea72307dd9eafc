"""Dense FP64 PyTorch restatement of U_lambda = U0 + W(u'(U1 - U0)) (test
infrastructure: the gradient reference of the autograd tests).

Pair candidates come from a k-d tree at x and x+d (cutoff + margin); the
energy applies the exact FP64 rule r < rc.  Same physics as oracle/sdm_oracle.c.
"""
import numpy as np
import torch
from scipy.spatial import cKDTree

K = 138.935456


def candidate_pairs(s, x, d):
    box = np.asarray(s.box)
    out = set()
    for y in (x, x + d):
        t = cKDTree(np.mod(y, box), boxsize=box)
        p = t.query_pairs(s.cutoff + 0.05, output_type="ndarray")
        out.update(map(tuple, np.sort(p, axis=1)))
    ex = set(map(tuple, np.sort(np.asarray(s.exclusions).reshape(-1, 2), axis=1)))
    pairs = np.array(sorted(out - ex), dtype=np.int64).reshape(-1, 2)
    return torch.from_numpy(pairs[:, 0]), torch.from_numpy(pairs[:, 1])


def softcore(u, method, umax, a, ub):
    if method == 0:
        return u
    if method == 1:
        t = torch.tanh((u - ub) / umax)
        return torch.where(u <= ub, u, umax * t + ub)
    gu = (u - ub) / (a * (umax - ub))
    z = 1 + 2 * gu * (gu + 1)
    za = z.clamp_min(1e-300) ** a
    return torch.where(u <= ub, u, (umax - ub) * (za - 1) / (za + 1) + ub)


def potential(s, x, q, sig, eps, d, lam1, lam2, alpha, u0, w0, prm, pairs=None):
    """x (N,3) float64 tensor; q/sig/eps (N,) tensors; d (N,3); scalars as tensors."""
    box = torch.tensor(np.asarray(s.box), dtype=torch.float64)
    if pairs is None:
        pairs = candidate_pairs(s, x.detach().numpy(), d.detach().numpy())
    i, j = pairs
    rc = s.cutoff
    er = s.eps_rf
    krf = (er - 1) / ((2 * er + 1) * rc ** 3)
    crf = 3 * er / ((2 * er + 1) * rc)
    se = torch.sqrt(eps)

    def energy(pos):
        dv = pos[j] - pos[i]
        dv = dv - box * torch.round(dv.detach() / box)
        r2 = (dv * dv).sum(1)
        m = r2 < rc * rc
        r2 = torch.where(m, r2, torch.ones_like(r2))
        r = torch.sqrt(r2)
        sg = 0.5 * (sig[i] + sig[j])
        ep = se[i] * se[j]
        s6 = (sg * sg / r2) ** 3
        e = 4 * ep * (s6 * s6 - s6) + K * q[i] * q[j] * (1 / r + krf * r2 - crf)
        return torch.where(m, e, torch.zeros_like(e)).sum()

    U0 = energy(x)
    U1 = energy(x + d)
    u = U1 - U0
    be = softcore(u, prm.softcore_method, prm.umax, prm.acore, prm.ubcore)
    ee = 1 + torch.exp(-alpha * (be - u0))
    W = ((lam2 - lam1) / alpha) * torch.log(ee) + lam2 * be + w0
    return U0 + W, u
