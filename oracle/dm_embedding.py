"""Diffusion-map embedding of a PD's distance matrix (test infrastructure only).

CPU restatement of ``DMembeddingII.op(D, k, tune, prefsigma)`` (reference
``modules/DMembeddingII.py:43-185``) with the helpers it calls: ``fergusonE.op``
(``modules/fergusonE.py:21-58``), ``sembeddingonFly.op`` (``modules/sembeddingonFly.py:14-36``)
and ``slaplacianonFly.op`` (``modules/slaplacianonFly.py:42-81``), for the k = nS neighbourhood
the manifold stage uses (``manifoldTrimmingAuto.py:51-54``).  It is the downstream validation
metric of the distance stage: the subspace angles between the top-8 eigenvector coordinates psi
of a GPU D and of the FP64 D.  The reference draws from ``np.random`` (``DMembeddingII.py:142``,
``fergusonE.py:52``); ``dm_embedding`` seeds it first.
"""
from __future__ import annotations

import numpy as np
from scipy.linalg import subspace_angles
from scipy.optimize import OptimizeWarning, curve_fit
from scipy.sparse import csc_matrix, csr_matrix
from scipy.sparse.linalg import ArpackNoConvergence, eigsh

NUM_EIGS = 15          # p.num_eigs (p.py:69-70)


def _tanh_model(x, a0, a1, a2, a3):
    return a3 + a2 * np.tanh(a0 * x + a1)


def ferguson(Dv: np.ndarray, log_eps: np.ndarray, a0: np.ndarray):
    """Kernel-bandwidth fit (fergusonE.py:25-58): log sum_ij W_ij(eps) over a log eps grid,
    fitted by a3 + a2 tanh(a0 x + a1), refitted from random starts until the parameter error
    sum is <= 100."""
    D2 = Dv * Dv
    eps_max = np.exp(log_eps).max()
    sg = np.sort(D2 / (2.0 * eps_max))
    thr = max(-np.log(0.01 * np.sum(np.exp(-sg)) / len(D2)), 10)
    log_sum = np.empty(len(log_eps))
    for k, le in enumerate(log_eps):
        d = D2 / (2.0 * np.exp(le))
        log_sum[k] = np.log(np.sum(np.exp(-d[d < thr])))
    import warnings
    resnorm = np.inf
    popt = None
    while resnorm > 100:
        with warnings.catch_warnings():
            warnings.simplefilter('ignore', OptimizeWarning)
            popt, pcov = curve_fit(_tanh_model, log_eps, log_sum, p0=a0.ravel())
        resnorm = np.sum(np.sqrt(np.fabs(np.diag(pcov))))
        a0 = np.random.rand(4, 1) - .5
    return popt, log_sum


def neighbour_lists(D: np.ndarray, k: int):
    """Sorted neighbour lists (DMembeddingII.py:43-57, :97-110): for each point (column of D,
    self first with distance 0) its k nearest entries; flattened rank-major."""
    nS = D.shape[0]
    Dm = np.array(D, dtype=np.float64, copy=True)
    Dm[np.arange(nS), np.arange(nS)] = -np.inf
    order = np.argsort(Dm, axis=0, kind='quicksort')[:k, :]
    vals = np.take_along_axis(Dm, order, axis=0)
    vals[0, :] = 0
    rows = np.broadcast_to(np.arange(nS)[None, :], (k, nS))
    return rows.reshape(-1), order.reshape(-1), vals.reshape(-1)


def dm_embedding(D: np.ndarray, k: int = None, tune: float = 3, seed: int = 0,
                 full: bool = False):
    """Returns (lambda, psi, sigma) as DMembeddingII.op does (psi = v[:,1:]/v[:,0]); with
    ``full`` also the Riemannian measure mu = v[:,0]^2 (DMembeddingII.py:178-181).  ``seed`` None
    draws from np.random as it stands (a caller that seeded it once for several embeddings)."""
    if seed is not None:
        np.random.seed(seed)
    nS = D.shape[0]
    k = nS if k is None else k
    rows, cols, vals = neighbour_lists(D, k)
    nz = ~(vals < 1e-6)
    y = csr_matrix((np.sqrt(vals[nz]), (rows[nz], cols[nz])), shape=(nS, nS)).toarray()
    y = y ** 2 + (y ** 2).T - y * y.T                   # symmetrised squared distances
    r_nz, c_nz = y.nonzero()
    v_nz = y[r_nz, c_nz]
    z = csr_matrix((np.ones(int((~nz).sum())), (rows[~nz], cols[~nz])), shape=(nS, nS)).toarray()
    r_z, c_z = z.nonzero()
    yRow = np.concatenate((r_z, r_nz)).astype(int)
    yCol = np.concatenate((c_z, c_nz)).astype(int)
    yVal = np.concatenate((np.zeros(len(r_z)), v_nz))
    a0 = np.random.rand(4, 1) - .5
    popt, _ = ferguson(np.sqrt(yVal), np.arange(-150, 150.2, 0.2), a0)
    sigma = tune * np.sqrt(2 * np.exp(-popt[1] / popt[0]))
    n_eigs = min(NUM_EIGS, nS - 3)
    # sparse normalised graph Laplacian (slaplacianonFly.py:42-81), alpha = 1
    w = np.exp(-(yVal / sigma ** 2))
    L = csc_matrix((w, (yRow, yCol)), shape=(nS, nS))
    d = np.asarray(L.sum(axis=0)).ravel()
    w = w / (d[yRow] * d[yCol])
    L = csc_matrix((w, (yRow, yCol)), shape=(nS, nS))
    d = np.sqrt(np.asarray(L.sum(axis=0)).ravel())
    w = w / (d[yRow] * d[yCol])
    L = csc_matrix((w, (yRow, yCol)), shape=(nS, nS))
    L = abs(L + L.T) / 2.0
    try:
        vals_e, vecs = eigsh(L, k=n_eigs + 1, maxiter=300)
    except ArpackNoConvergence as e:
        vals_e, vecs = e.eigenvalues, e.eigenvectors
    ix = np.argsort(vals_e)[::-1]
    vals_e = vals_e[ix]
    vecs = vecs[:, ix]
    psi = np.zeros((nS, n_eigs))
    m = vecs.shape[1] - 1
    psi[:, :m] = vecs[:, 1:] / vecs[:, :1]
    if full:
        return vals_e, psi, sigma, vecs[:, 0] * vecs[:, 0]
    return vals_e, psi, sigma


def top8_subspace_angle(D_a: np.ndarray, D_b: np.ndarray, seed: int = 0) -> float:
    """Largest principal angle (radians) between the spans of the top-8 diffusion-map
    coordinates of two distance matrices of the same PD."""
    _, pa, _ = dm_embedding(D_a, seed=seed)
    _, pb, _ = dm_embedding(D_b, seed=seed)
    return float(np.max(subspace_angles(pa[:, :8], pb[:, :8])))
