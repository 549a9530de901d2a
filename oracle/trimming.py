"""Manifold trimming of one PD (test infrastructure only).

CPU restatement of the embedding-and-trimming loop of ``manifoldTrimmingAuto.op`` (reference
``modules/manifoldTrimmingAuto.py:44-77``) over the FP64 diffusion map of ``dm_embedding``:
embed D (k = nS), keep the points whose first three diffusion coordinates lie within ``rad`` of
the origin (``get_psiPath``, :18-28), and while that drops points, embed the kept points'
distances again and keep the positive eigenvalues only (:61-70).  ``np.random`` is seeded once
before the first embedding; later embeddings continue its stream, as the reference's do.
Parity is pinned by ``tests/golden/trim_*.npz``, made by running the reference's own op.
"""
from __future__ import annotations

import numpy as np

from .dm_embedding import dm_embedding


def psi_path(psi: np.ndarray, rad: float) -> np.ndarray:
    """get_psiPath(psi, rad, 0) (manifoldTrimmingAuto.py:18-28)."""
    return np.nonzero(np.sqrt(psi[:, 0] ** 2 + psi[:, 1] ** 2 + psi[:, 2] ** 2) < rad)[0]


def trim(D: np.ndarray, tune: float = 3, rad: float = 5, seed: int = 0):
    """Returns (lamb, psi, sigma, mu, posPath, n_embeddings) of the last embedding."""
    np.random.seed(seed)
    D = np.asarray(D, dtype=np.float64)
    nS = D.shape[0]
    lamb, psi, sigma, mu = dm_embedding(D, tune=tune, seed=None, full=True)
    keep = psi_path(psi, rad)
    runs = 1
    while len(keep) < nS:
        nS = len(keep)
        lamb, psi, sigma, mu = dm_embedding(D[keep][:, keep], tune=tune, seed=None, full=True)
        lamb = lamb[lamb > 0]
        keep = keep[psi_path(psi, rad)]
        runs += 1
    return lamb, psi, sigma, mu, keep, runs
