"""Helpers shared by the GPU parity tests."""
import numpy as np

EPS = np.finfo(np.float64).eps


def to_dev(a, dtype=None):
    import torch
    a = np.asarray(a)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    t = torch.from_numpy(np.ascontiguousarray(a.T)).cuda()
    if dtype is not None:
        t = t.to(dtype)
    return t.t()            # column-major view, strides (1, m)


def to_host(t):
    return np.asfortranarray(t.t().contiguous().cpu().numpy().T)


def berr(orc, A, X, B, sym=False):
    return orc.backward_error(np.asfortranarray(A), np.asfortranarray(X), np.asfortranarray(B), sym_lower=sym)


def spd(orc, n, seed):
    """A = G G^T / n + I with G ~ N(0,1) from SLATE's Philox normal stream."""
    G = orc.generate(3, seed, n, n)
    return np.asfortranarray(G @ G.T / n + np.eye(n))
