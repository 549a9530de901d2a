"""NLSA stage of one projection direction (test infrastructure only).

CPU restatement in float64 of the reference's ``NLSA.op`` (``modules/NLSA.py:23-158``) and the
helpers it calls: ``get_wiener.op`` (``modules/get_wiener.py:9-21``), ``svdRF.op``
(``modules/svdRF.py:9-36``), ``L2_distance.op`` (``modules/L2_distance.py:43-76``),
``fit_1D_open_manifold_3D.op`` (``modules/fit_1D_open_manifold_3D.py:64-161``) with
``get_fit_1D_open_manifold_3D_param.op`` (``:12-92``), ``solve_d_R_d_tau_p_3D.op`` (``:35-60``)
and ``R_p.op`` (``:41-49``), and the two diffusion-map embeddings through
``oracle.dm_embedding``.  The Wiener-filtered snapshots are formed image by image with
``scipy.fftpack`` exactly as the reference loops (``NLSA.py:66-86``), so this module is the slow,
literal form that the GPU stage's frequency-domain contraction is checked against.  It draws from
``np.random`` in the reference's order (two embeddings, each ``DMembeddingII.py:142`` plus the
restarts of ``fergusonE.py:52``); seed it once before calling ``nlsa``.
"""
from __future__ import annotations

import numpy as np
from scipy.fftpack import fft2, ifft2

from .dm_embedding import dm_embedding


def con_distances(DD: np.ndarray, con_order: int) -> np.ndarray:
    """ConD = sum_{i < ConOrder} DD[i:i+m, i:i+m], m = num - ConOrder, added in order i = 0, 1, ..
    (NLSA.py:31-34)."""
    num = DD.shape[1]
    m = num - con_order
    ConD = np.zeros((m, m))
    for i in range(con_order):
        ConD += DD[i:i + m, i:i + m]
    return ConD


def get_wiener(CTF1: np.ndarray, con_order: int, num: int) -> np.ndarray:
    """wiener_dom[i] = sum_{ii < ConOrder} CTF1[ConOrder - ii + i]^2 + 1/5 (get_wiener.py:9-21),
    the ii = 0 term first."""
    dim = CTF1.shape[1]
    wd = np.zeros((num - con_order, dim, dim))
    for i in range(num - con_order):
        for ii in range(con_order):
            wd[i] = wd[i] + CTF1[con_order - ii + i] ** 2
    return wd + 1. / 5


def snapshot_matrix(IMG1, CTF1, wd, msk2, mu_psi, con_order, num, wiener=True):
    """A (ConOrder N^2, psiTrunc): block ii = tmp_ii @ mu_psi, column i of tmp_ii the snapshot
    ind3 = ConOrder - ii + i - 1 transposed and flattened, Wiener-filtered by
    CTF1[ind3] / wiener_dom[i] and masked when ``wiener`` (NLSA.py:63-86)."""
    dim = IMG1.shape[1]
    m = num - con_order
    A = np.zeros((con_order * dim * dim, mu_psi.shape[1]))
    tmp = np.zeros((dim * dim, m))
    for ii in range(con_order):
        for i in range(m):
            ind3 = con_order - ii + i - 1
            img = IMG1[ind3]
            if wiener:
                img = ifft2(fft2(img) * (CTF1[ind3] / wd[i])).real
                img = img * msk2
            tmp[:, i] = img.T.reshape(-1)
        A[ii * dim * dim:(ii + 1) * dim * dim] = tmp @ mu_psi
    return A


def svd_rf(A: np.ndarray):
    """Thin SVD through the eigen-decomposition of the smaller Gram matrix, eigenpairs sorted by
    decreasing value (svdRF.py:9-36)."""
    D1, D2 = A.shape

    def tidy(D, EV):
        order = np.argsort(D)[::-1]
        D = np.sort(D)[::-1]
        EV = EV[:, order]
        sq = np.sqrt(D)
        return D, EV, np.diag(sq), np.diag(1. / sq)

    if D1 > D2:
        D, V = np.linalg.eigh(A.T @ A)
        D, V, S, invS = tidy(D, V)
        U = A @ (V @ invS)
    else:
        D, U = np.linalg.eigh(A @ A.T)
        D, U, S, invS = tidy(D, U)
        V = A.T @ (U @ invS)
    return U, S, V


def l2_distance(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Euclidean distances between the columns of a and b, squared values below 1e-8 set to 0
    (L2_distance.py:43-76)."""
    aa = np.sum(a ** 2, axis=0)
    bb = np.sum(b ** 2, axis=0)
    ab = a.T @ b
    t = aa[:, None] + bb[None, :] - 2 * ab
    t[t < 1e-8] = 0
    return np.sqrt(t)


# ---- 1D open-manifold fit x_ij = a_j cos(j pi tau_i) + b_j, j = 1..3 -------------------------

def _residual(x_p, a, b, tau):
    """R_p at the candidates tau (R_p.py:41-49)."""
    jj = np.arange(1, 4)
    err = x_p - b - a * np.cos(tau * jj * np.pi)
    return np.sum(err ** 2, axis=1)


def _solve_tau_p(x_p, a, b):
    """tau of one point: the real roots in [-1, 1] of dR/d(beta), beta = cos(pi tau), then 0 and
    1, the candidate of least residual (solve_d_R_d_tau_p_3D.py:35-60)."""
    coef = np.array([48 * a[2] ** 2, 0, 8 * a[1] ** 2 - 48 * a[2] ** 2,
                     -12 * a[2] * (x_p[2] - b[2]),
                     a[0] ** 2 - 4 * a[1] ** 2 + 9 * a[2] ** 2 - 4 * a[1] * (x_p[1] - b[1]),
                     -a[0] * (x_p[0] - b[0]) + 3 * a[2] * (x_p[2] - b[2])])
    beta = np.roots(coef)
    beta = beta[~(np.abs(np.imag(beta)) > 0)]
    beta = np.real(beta[~(np.abs(beta) > 1)])
    cand = np.vstack((np.arccos(beta.reshape(-1, 1)) / np.pi, 0, 1))
    return cand[np.argmin(_residual(x_p, a, b, cand))]


def _initial_fit(psi):
    """Initial a, b from cubic / quadratic least-squares fits in the (x1, x3) and (x1, x2) planes
    (get_fit_1D_open_manifold_3D_param.py:24-86)."""
    nS = psi.shape[0]
    X, Y, Z = psi[:, 0], psi[:, 1], psi[:, 2]
    X2 = X * X
    X3 = X2 * X
    X4 = X2 * X2
    X5 = X3 * X2
    X6 = X3 * X3
    sX, sX2, sX3, sX4, sX5, sX6 = (np.sum(v) for v in (X, X2, X3, X4, X5, X6))
    A = np.array([[sX6, sX5, sX4, sX3], [sX5, sX4, sX3, sX2], [sX4, sX3, sX2, sX],
                  [sX3, sX2, sX, nS]])
    rhs = np.array([np.dot(X3, Z), np.dot(X2, Z), np.dot(X, Z), np.sum(Z)])
    D, E, F, G = np.linalg.lstsq(A, rhs)[0]
    disc = E * E - 3 * D * F
    if disc < 0:
        disc = 0.
    if np.absolute(D) < 1e-8:
        D = 1e-8
    a1 = (2. * np.sqrt(disc)) / (3. * D)
    a3 = (2. * disc ** (3 / 2.)) / (27. * D * D)
    b1 = -E / (3 * D)
    b3 = (2. * E * E * E) / (27. * D * D) - (E * F) / (3 * D) + G
    XXb = X * (X - 2 * b1)
    A = np.array([[np.sum(XXb * XXb), np.sum(XXb)], [np.sum(XXb), nS]])
    Ac, C = np.linalg.lstsq(A, np.array([np.dot(XXb, Y), np.sum(Y)]))[0]
    a2 = 2. * Ac * disc / (9. * D * D)
    b2 = C + (Ac * E * E) / (9. * D * D) - (2. * Ac * F) / (3. * D)
    return np.array([a1, a2, a3]), np.array([b1, b2, b3])


def fit_1d_open_manifold_3d(psi: np.ndarray, max_iter: int = 100):
    """Alternating fit of {a, b} (three 2x2 least-squares problems) and {tau} (per point) until
    the amplitude and offset changes fall below 1 % (fit_1D_open_manifold_3D.py:64-161).  Returns
    (a, b, tau) with tau of shape (nS, 1)."""
    x = psi[:, 0:3]
    nS = x.shape[0]
    a, b = _initial_fit(psi)
    tau = np.zeros((nS, 1))
    for p in range(nS):
        tau[p] = _solve_tau_p(x[p], a, b)
    eps = 1e-4
    for _ in range(1, max_iter + 1):
        a_old, b_old = a, b
        cj = np.cos(tau @ (np.pi * np.array([[1, 2, 3]])))
        A11 = np.sum(cj ** 2, axis=0)
        A12 = np.sum(cj, axis=0)
        b1 = np.sum(x * cj, axis=0)
        b2 = np.sum(x, axis=0)
        coeff = np.zeros((2, 3))
        for q in range(3):
            coeff[:, q] = np.linalg.lstsq(np.array([[A11[q], A12[q]], [A12[q], nS]]),
                                          np.array([b1[q], b2[q]]))[0]
        a, b = coeff[0, :], coeff[1, :]
        # the reference keeps tau_old = tau, the same array that is then updated in place, so
        # its change in tau is always 0 and only the a / b changes end the iteration
        tau_old = tau
        for p in range(nS):
            tau[p] = _solve_tau_p(x[p], a, b)
        da = np.max(np.fabs(a - a_old) / (np.fabs(a) + eps)) * 100
        db = np.max(np.fabs(b - b_old) / (np.fabs(b) + eps)) * 100
        dt = np.max(np.fabs(tau - tau_old))
        if da < 1 and db < 1 and dt < 0.01:
            break
    return a, b, tau


def nlsa(NLSAPar: dict, DD, posPath, posPsi1, imgAll, msk2, CTF, ExtPar: dict):
    """NLSA.op: returns (IMGT, Topo_mean, psirec, psiC1, sdiag, VX, mu, tau) (NLSA.py:23-158)."""
    num = NLSAPar['num']
    c = NLSAPar['ConOrder']
    k = NLSAPar['k']
    tune = NLSAPar['tune']
    nS = NLSAPar['nS']
    psiTrunc = NLSAPar['psiTrunc']
    ConD = con_distances(np.asarray(DD, dtype=np.float64), c)
    _, psiC, _, mu = dm_embedding(ConD, k=k, tune=tune, seed=None, full=True)
    psiC1 = np.copy(psiC)
    wiener = 'prD' in ExtPar
    if wiener:
        sel = np.asarray(posPath)[np.asarray(posPsi1)]
        IMG1 = np.asarray(imgAll, dtype=np.float64)[sel]
        CTF1 = np.asarray(CTF, dtype=np.float64)[sel]
        wd = get_wiener(CTF1, c, num)
    elif 'cuti' in ExtPar:
        IMG1 = np.asarray(imgAll, dtype=np.float64)[np.asarray(posPsi1)]
        CTF1 = wd = None
    else:
        raise ValueError("ExtPar names neither 'prD' nor 'cuti'")
    dim = CTF.shape[1]
    ell = psiTrunc - 1
    psiX = np.hstack((np.ones((psiC.shape[0], 1)), psiC[:, 0:ell]))
    mu_psi = mu.reshape((-1, 1)) * psiX
    A = snapshot_matrix(IMG1, CTF1, wd, np.asarray(msk2), mu_psi, c, num, wiener)
    U, S, V = svd_rf(A)
    VX = V.T @ psiX.T
    sdiag = np.diag(S)
    npix = dim * dim
    Topo_mean = np.zeros((npix, psiTrunc))
    for ii in range(psiTrunc):
        Topo_mean[:, ii] = np.mean(np.stack([U[q * npix:(q + 1) * npix, ii] for q in range(c)],
                                            axis=1), axis=1)
    ConImgT = np.zeros((U.shape[0], ell + 1))
    for i in range(0, 2):
        ConImgT = ConImgT + U[:, i].reshape(-1, 1) @ (sdiag[i] * V[:, i].reshape(1, -1))
    IMGT = np.zeros((npix, nS - 2 * c))
    for i in range(c):
        t = ConImgT[i * npix:(i + 1) * npix] @ psiX.T
        for ii in range(num - 2 * c):
            IMGT[:, ii] = IMGT[:, ii] + t[:, i + ii]
    with np.errstate(divide='ignore', invalid='ignore'):
        IMGT = (IMGT - IMGT.mean(axis=0)) / IMGT.std(axis=0)
    Drecon = l2_distance(IMGT, IMGT)
    _, psirec, _, mu = dm_embedding(Drecon ** 2, k=min(IMGT.shape), tune=tune, seed=None,
                                    full=True)
    _, _, tau = fit_1d_open_manifold_3d(psirec)
    return IMGT, Topo_mean, psirec, psiC1, sdiag, VX, mu, tau
