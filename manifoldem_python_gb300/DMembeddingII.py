"""Diffusion-map embedding of a PD's distance matrix on the GPU.

Drop-in for the reference's ``DMembeddingII.op(D, k, tune, prefsigma)``
(``modules/DMembeddingII.py:86-185``), the direct consumer of the distance stage's D
(``manifoldTrimmingAuto.py:51-67``, ``embedd.py:43``, ``NLSA.py:45,146``).  Same arguments, same
8-tuple ``(lamb, psi, sigma, mu, logEps, logSumWij, popt, R_squared)``.

Split of the work:

* GPU (``csrc/dmap.cu`` through the C ABI): the symmetrised squared-distance matrix
  (``DMembeddingII.py:112-139``), the bandwidth sweep of ``fergusonE.op`` (1501 sums of
  n^2 exponentials, ``fergusonE.py:36-44``) and the normalised kernel of ``slaplacianonFly.op``
  (alpha = 1, ``slaplacianonFly.py:55-80``);
* GPU library calls: the k-nearest lists (``torch.topk`` per column, the point itself first as
  the reference's ``D[iS, iS] = -inf`` makes it) and the eigen-decomposition of the dense
  normalised kernel (``torch.linalg.eigh``), from which the ``nEigs + 1`` eigenpairs of largest
  magnitude are kept and sorted by decreasing value, as ``eigsh(..., which='LM')`` followed by
  the sort in ``sembeddingonFly.py:29-31`` gives;
* host: the tanh fit of the sweep with ``scipy.optimize.curve_fit`` and its random restarts
  drawn from ``np.random`` in the reference's order (``DMembeddingII.py:142``,
  ``fergusonE.py:46-56``), so a seeded caller gets the reference's starting points.

The sweep evaluates the exponentials in float32 and accumulates in float64; everything else is
float64.
"""
from __future__ import annotations

import ctypes
import math
import warnings
from typing import Optional

import numpy as np

from . import _lib

NUM_EIGS = 15                                       # p.num_eigs (p.py:69-70)
LOG_EPS = np.arange(-150, 150.2, 0.2)               # DMembeddingII.py:146


def _tanh_model(x, a0, a1, a2, a3):
    return a3 + a2 * np.tanh(a0 * x + a1)


def ferguson_fit(log_eps: np.ndarray, log_sum: np.ndarray, a0: np.ndarray):
    """The tanh fit of fergusonE.op (fergusonE.py:46-56): refit from random starts until the sum
    of the parameters' standard errors is <= 100.  Returns (popt, resnorm, R_squared)."""
    from scipy.optimize import OptimizeWarning, curve_fit
    resnorm = np.inf
    popt = r2 = None
    while resnorm > 100:
        with warnings.catch_warnings():
            warnings.simplefilter('ignore', OptimizeWarning)
            popt, pcov = curve_fit(_tanh_model, log_eps, log_sum, p0=np.ravel(a0))
        resnorm = np.sum(np.sqrt(np.fabs(np.diag(pcov))))
        a0 = np.random.rand(4, 1) - .5
        resid = log_sum - _tanh_model(log_eps, *popt)
        r2 = 1 - np.sum(resid ** 2) / np.sum((log_sum - np.mean(log_sum)) ** 2)
    return popt, resnorm, r2


class _Device:
    """Device buffers of one embedding."""

    def __init__(self, D, device):
        import torch
        self.torch = torch
        self.dev = torch.device(device or 'cuda')
        if isinstance(D, torch.Tensor):
            self.D = D.to(device=self.dev, dtype=torch.float64).contiguous()
        else:
            self.D = torch.from_numpy(np.ascontiguousarray(D, dtype=np.float64)).to(self.dev)
        self.n = int(self.D.shape[0])
        self.stream = torch.cuda.current_stream(self.dev)
        self.lib = _lib.load()

    def listed(self, k: int):
        """uint8 (n, n): listed[i, j] = 1 if j is among the k nearest of point i (column i of D,
        the point itself first), or None when k >= n."""
        torch = self.torch
        if k >= self.n:
            return None
        Dm = self.D.clone()
        Dm.fill_diagonal_(-math.inf)
        idx = torch.topk(Dm, k, dim=0, largest=False, sorted=True).indices      # (k, n)
        out = torch.zeros((self.n, self.n), dtype=torch.uint8, device=self.dev)
        cols = torch.arange(self.n, device=self.dev).expand(k, self.n)
        out[cols.reshape(-1), idx.reshape(-1)] = 1
        return out

    def call(self, name, *args):
        _lib.check(getattr(self.lib, name)(*args, ctypes.c_void_p(self.stream.cuda_stream)),
                   name)


def op(D, k: int, tune: float, prefsigma: float, num_eigs: int = NUM_EIGS,
       device: Optional[str] = None):
    """DMembeddingII.op on the GPU: returns (lamb, psi, sigma, mu, logEps, logSumWij, popt,
    R_squared) with the reference's shapes (host numpy arrays)."""
    g = _Device(D, device)
    torch, n = g.torch, g.n
    listed = g.listed(int(k))
    Y = torch.empty((n, n), dtype=torch.float64, device=g.dev)
    g.call('mem_dm_symmetrise', g.D.data_ptr(), n,
           listed.data_ptr() if listed is not None else None, Y.data_ptr())
    n_edges = int((Y >= 0).sum().item())
    a0 = np.random.rand(4, 1) - .5                   # DMembeddingII.py:142
    log_eps = LOG_EPS
    log2e = 1.0 / math.log(2.0)
    # threshold of fergusonE.find_thres (fergusonE.py:27-32): 1% of the mean kernel value at the
    # largest eps, at least 10
    scale = torch.tensor([log2e / (2.0 * float(np.max(np.exp(log_eps))))], dtype=torch.float32,
                         device=g.dev)
    s0 = torch.empty(1, dtype=torch.float64, device=g.dev)
    g.call('mem_dm_sweep', Y.data_ptr(), n, scale.data_ptr(), 1, math.inf, s0.data_ptr())
    thr = max(-math.log(0.01 * float(s0.item()) / n_edges), 10.0)
    with np.errstate(over='ignore'):     # +inf for the smallest eps: only d = 0 terms survive
        scale = torch.from_numpy((log2e / (2.0 * np.exp(log_eps))).astype(np.float32)).to(g.dev)
    sums = torch.empty(len(log_eps), dtype=torch.float64, device=g.dev)
    g.call('mem_dm_sweep', Y.data_ptr(), n, scale.data_ptr(), len(log_eps), thr, sums.data_ptr())
    log_sum = np.log(sums.cpu().numpy())
    popt, _, r2 = ferguson_fit(log_eps, log_sum, a0)
    sigma = tune * np.sqrt(2 * np.exp(-popt[1] / popt[0]))    # DMembeddingII.py:156
    n_eigs = min(num_eigs, n - 3)
    scratch = torch.empty(2 * n, dtype=torch.float64, device=g.dev)
    g.call('mem_dm_laplacian', Y.data_ptr(), n, float(sigma), scratch.data_ptr())
    vals, vecs = torch.linalg.eigh(Y)
    sel = torch.argsort(vals.abs(), descending=True)[:n_eigs + 1]     # eigsh(which='LM')
    vals, vecs = vals[sel], vecs[:, sel]
    order = torch.argsort(vals, descending=True)
    lamb = vals[order].cpu().numpy()
    v = vecs[:, order].cpu().numpy()
    psi = np.zeros((n, n_eigs))
    m = v.shape[1] - 1
    psi[:, :m] = v[:, 1:] / v[:, :1]
    mu = v[:, 0] * v[:, 0]
    return lamb, psi, sigma, mu, log_eps, log_sum, popt, r2
