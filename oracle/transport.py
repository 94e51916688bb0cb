"""FP64 restatement of the cache transport over a frozen ray set — TEST INFRASTRUCTURE ONLY.

For K kept rays per point (``pyoracle.Scene.frozen_hits``: the rays of one iteration of the
reference's k_ref, prep_mesh.cuh:182-200) the cache's fixed point is linear:

    L_l = T (E_l G_l + L_l),   T[i, j] = A_j / K x (rays of point i that reach point j),

G_l the direct light of light l at unit emission (k_build, poc_gpu.cu:369-391).  This module
solves it in FP64 and differentiates J = sum_i w_i sum_l L_l[i] with respect
to the emissions E_l two ways: central finite differences (h = 1e-3 E_l) and the adjoint
u = (I - T^T)^{-1} w, dJ/dE_l = (u - w) . G_l.  Solves are FP64 Jacobi sweeps run to a relative
change of 1e-15.  Only the tests import it.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def transport_matrix(hits: np.ndarray, albedo: np.ndarray) -> sp.csr_matrix:
    Np, K = hits.shape
    src = np.repeat(np.arange(Np), K)
    dst = hits.reshape(-1)
    keep = dst >= 0
    vals = albedo.astype(np.float64)[dst[keep]] / K
    return sp.csr_matrix((vals, (src[keep], dst[keep])), shape=(Np, Np))   # repeated rays add up


def _fixed_point(M: sp.csr_matrix, b: np.ndarray, tol: float = 1e-15, max_iter: int = 5000) -> np.ndarray:
    """x = b + M x by Jacobi sweeps in FP64 (M's rows sum to at most max(albedo) < 1, so the
    iteration contracts), until a sweep changes x by less than tol x max |x|."""
    x = b.copy()
    for _ in range(max_iter):
        nx = b + M @ x
        if np.max(np.abs(nx - x)) <= tol * max(np.max(np.abs(nx)), 1e-300):
            return nx
        x = nx
    raise RuntimeError("transport fixed point did not converge")


class Transport:
    def __init__(self, hits: np.ndarray, albedo: np.ndarray, G: np.ndarray):
        self.T = transport_matrix(hits, albedo)
        self.Tt = self.T.T.tocsr()
        self.G = G.astype(np.float64)                       # (Np, NL)

    def radiance(self, E: np.ndarray) -> np.ndarray:
        """L summed over lights: (I - T)^{-1} T (G E)."""
        return _fixed_point(self.T, self.T @ (self.G @ np.asarray(E, np.float64)))

    def objective(self, E: np.ndarray, w: np.ndarray) -> float:
        return float(np.dot(w.astype(np.float64), self.radiance(E)))

    def importance(self, w: np.ndarray) -> np.ndarray:
        """u = (I - T^T)^{-1} w."""
        return _fixed_point(self.Tt, w.astype(np.float64))

    def adjoint_gradient(self, w: np.ndarray) -> np.ndarray:
        u = self.importance(w)
        return (u - w.astype(np.float64)) @ self.G

    def fd_gradient(self, E: np.ndarray, w: np.ndarray, rel: float = 1e-3) -> np.ndarray:
        E = np.asarray(E, np.float64)
        g = np.empty(len(E))
        for l in range(len(E)):
            h = rel * E[l] if E[l] > 0 else rel
            ep, em = E.copy(), E.copy()
            ep[l] += h
            em[l] -= h
            g[l] = (self.objective(ep, w) - self.objective(em, w)) / (2 * h)
        return g
