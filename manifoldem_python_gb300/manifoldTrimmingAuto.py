"""Manifold trimming of one PD on the GPU diffusion map.

Drop-in for the reference's ``manifoldTrimmingAuto.op(input_data, posPath, tune, rad, visual,
doSave)`` (``modules/manifoldTrimmingAuto.py:38-95``), which ``manifoldAnalysis.op`` calls for
every PD (``manifoldAnalysis.py:94-102``): the diffusion-map embedding of the PD's distance
matrix, then, while points lie outside the radius ``rad`` in the first three diffusion
coordinates, their removal and a new embedding of the rest; the result goes to the psi pickle
(``myio.fout1`` with the reference's ten keys), its progress marker and the eigenvalue file.
The embeddings run on the GPU (``manifoldem_python_gb300.DMembeddingII``), drawing from
``np.random`` in the reference's order; the D pickle written by the distance stage is read
with ``myio.fin1``.  ``visual`` would draw matplotlib figures in the reference; no figure is
drawn here.
"""
from __future__ import annotations

import os

import numpy as np

from . import DMembeddingII, myio
from .p import params_module

PREFSIGMA_FIRST = 60000      # manifoldTrimmingAuto.py:54
PREFSIGMA_LOOP = 600000      # manifoldTrimmingAuto.py:67


def get_psiPath(psi: np.ndarray, rad: float, plotNum: int) -> np.ndarray:
    """Indices of the points within ``rad`` of the origin in diffusion coordinates plotNum ..
    plotNum + 2 (manifoldTrimmingAuto.py:18-28)."""
    dist = np.sqrt(psi[:, plotNum] ** 2 + psi[:, plotNum + 1] ** 2 + psi[:, plotNum + 2] ** 2)
    return (dist < rad).nonzero()[0]


def trim(D: np.ndarray, posPath, tune: float, rad: float, device=None):
    """The embedding-and-trimming loop (manifoldTrimmingAuto.py:44-77): returns the last
    embedding's 8-tuple (lamb with only its positive values when the loop ran, as the
    reference leaves it) and the kept indices posPath."""
    nS = D.shape[1]
    if np.isscalar(posPath) and posPath == 0:
        posPath = np.arange(nS)
    posPath = np.asarray(posPath)
    D = np.asarray(D)[posPath][:, posPath]
    nS = D.shape[1]
    res = DMembeddingII.op(D, nS, tune, PREFSIGMA_FIRST, device=device)
    posPath1 = get_psiPath(res[1], rad, 0)
    while len(posPath1) < nS:
        nS = len(posPath1)
        D1 = D[posPath1][:, posPath1]
        res = DMembeddingII.op(D1, D1.shape[0], tune, PREFSIGMA_LOOP, device=device)
        lamb = res[0]
        res = (lamb[lamb > 0],) + tuple(res[1:])
        posPath1 = posPath1[get_psiPath(res[1], rad, 0)]
    return res, posPath[posPath1]


def op(input_data, posPath, tune, rad, visual, doSave, device=None):
    """manifoldTrimmingAuto.op: input_data = [dist_file, psi_file, eig_file, prD]."""
    dist_file, psi_file, eig_file, prD = input_data[:4]
    data = myio.fin1(dist_file)
    (lamb, psi, sigma, mu, logEps, logSumWij, popt, R_squared), posPath = trim(
        data['D'], posPath, tune, rad, device)
    if doSave['Is']:
        myio.fout1(psi_file, ['lamb', 'psi', 'sigma', 'mu', 'posPath', 'ind', 'logEps',
                              'logSumWij', 'popt', 'R_squared'],
                   [lamb, psi, sigma, mu, posPath, data['ind'], logEps, logSumWij, popt,
                    R_squared])
        p = params_module()
        open(os.path.join(p.psi_prog, '%s' % (prD)), 'a').close()
    if os.path.exists(eig_file):
        os.remove(eig_file)
    for i in range(len(lamb) - 1):
        with open(eig_file, 'a') as f:
            f.write('%d\t%.5f\n' % (i + 1, lamb[i + 1]))
    return None
