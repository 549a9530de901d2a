"""1D open-manifold fit of the NLSA reconstruction coordinates (host, numpy).

Drop-in for the reference's ``fit_1D_open_manifold_3D.op(psi)``
(``modules/fit_1D_open_manifold_3D.py:64-161``) with ``get_fit_1D_open_manifold_3D_param.op``
(``:12-92``), ``solve_d_R_d_tau_p_3D.op`` (``:35-60``) and ``R_p.op`` (``:41-49``): the model
x_ij = a_j cos(j pi tau_i) + b_j, j = 1..3, fitted by alternating three 2x2 least-squares problems
for (a_j, b_j) and a per-point minimisation over tau_i.  Returns (a, b, tau), tau of shape (nS, 1).

The per-point step finds the real roots in [-1, 1] of the quintic dR/d(beta), beta = cos(pi tau),
as eigenvalues of its companion matrix -- the construction of ``np.roots`` -- for all points in
one batched ``np.linalg.eigvals`` call, keeps the candidates the reference keeps (roots with a
zero imaginary part and modulus <= 1, then tau = 0 and tau = 1) and takes the first candidate of
least residual.  Points whose polynomial has a zero leading or trailing coefficient go through
``np.roots`` itself, which strips those zeros.  The reference stops when the amplitude and offset
changes are below 1 %: its change in tau is always 0, because it keeps ``tau_old = tau``, the
array it then updates in place; the same rule is kept here.
"""
from __future__ import annotations

import numpy as np

MAX_ITER = 100              # get_fit_1D_open_manifold_3D_param.py:17
DELTA_A_MAX = 1             # percent (:19)
DELTA_B_MAX = 1             # percent (:20)
DELTA_TAU_MAX = 0.01        # (:21)
_EPS = 1e-4                 # fit_1D_open_manifold_3D.py:59
_JJ = np.arange(1, 4)


def _coefficients(x: np.ndarray, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """(nS, 6) coefficients of dR/d(beta), highest power first (solve_d_R_d_tau_p_3D.py:37-42)."""
    n = x.shape[0]
    coef = np.empty((n, 6))
    coef[:, 0] = 48 * a[2] ** 2
    coef[:, 1] = 0
    coef[:, 2] = 8 * a[1] ** 2 - 48 * a[2] ** 2
    coef[:, 3] = -12 * a[2] * (x[:, 2] - b[2])
    coef[:, 4] = a[0] ** 2 - 4 * a[1] ** 2 + 9 * a[2] ** 2 - 4 * a[1] * (x[:, 1] - b[1])
    coef[:, 5] = -a[0] * (x[:, 0] - b[0]) + 3 * a[2] * (x[:, 2] - b[2])
    return coef


def _candidates(coef: np.ndarray):
    """Candidate betas (nS, 5) complex and a validity mask: the roots the reference keeps."""
    n = coef.shape[0]
    roots = np.zeros((n, 5), dtype=np.complex128)
    have = np.zeros((n, 5), dtype=bool)
    full = (coef[:, 0] != 0) & (coef[:, 5] != 0)
    idx = np.nonzero(full)[0]
    if idx.size:
        comp = np.zeros((idx.size, 5, 5))
        comp[:, 0, :] = -coef[idx, 1:] / coef[idx, :1]
        comp[:, np.arange(1, 5), np.arange(0, 4)] = 1
        roots[idx] = np.linalg.eigvals(comp)
        have[idx] = True
    for p in np.nonzero(~full)[0]:
        r = np.roots(coef[p])
        roots[p, :r.size] = r
        have[p, :r.size] = True
    keep = have & ~(np.abs(np.imag(roots)) > 0)
    keep &= ~(np.abs(roots) > 1)
    return np.real(roots), keep


def solve_tau(x: np.ndarray, a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """tau of every point (solve_d_R_d_tau_p_3D.op for p = 0 .. nS-1), shape (nS, 1)."""
    beta, keep = _candidates(_coefficients(x, a, b))
    n = x.shape[0]
    with np.errstate(invalid='ignore'):
        cand = np.concatenate((np.arccos(np.where(keep, beta, 0.0)) / np.pi,
                               np.zeros((n, 1)), np.ones((n, 1))), axis=1)       # (n, 7)
    err = x[:, None, :] - b - a * np.cos(cand[:, :, None] * _JJ * np.pi)
    R = np.sum(err ** 2, axis=2)
    R[:, :5][~keep] = np.inf
    pick = np.argmin(R, axis=1)
    return cand[np.arange(n), pick].reshape(n, 1)


def initial_parameters(psi: np.ndarray):
    """a, b from a cubic fit of x3 against x1 and a quadratic fit of x2 against x1
    (get_fit_1D_open_manifold_3D_param.py:24-86)."""
    nS = psi.shape[0]
    X, Y, Z = psi[:, 0], psi[:, 1], psi[:, 2]
    X2 = X * X
    X3 = X2 * X
    X4 = X2 * X2
    X5 = X3 * X2
    X6 = X3 * X3
    sX, sX2, sX3 = np.sum(X), np.sum(X2), np.sum(X3)
    sX4, sX5, sX6 = np.sum(X4), np.sum(X5), np.sum(X6)
    M = np.array([[sX6, sX5, sX4, sX3], [sX5, sX4, sX3, sX2], [sX4, sX3, sX2, sX],
                  [sX3, sX2, sX, nS]])
    rhs = np.array([np.dot(X3, Z), np.dot(X2, Z), np.dot(X, Z), np.sum(Z)])
    D, E, F, G = np.linalg.lstsq(M, rhs)[0]
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
    M2 = np.array([[np.sum(XXb * XXb), np.sum(XXb)], [np.sum(XXb), nS]])
    Aq, C = np.linalg.lstsq(M2, np.array([np.dot(XXb, Y), np.sum(Y)]))[0]
    a2 = 2. * Aq * disc / (9. * D * D)
    b2 = C + (Aq * E * E) / (9. * D * D) - (2. * Aq * F) / (3. * D)
    return np.array([a1, a2, a3]), np.array([b1, b2, b3])


def op(psi: np.ndarray):
    """fit_1D_open_manifold_3D.op: (a, b, tau)."""
    psi = np.asarray(psi, dtype=np.float64)
    x = psi[:, 0:3]
    nS = x.shape[0]
    a, b = initial_parameters(psi)
    tau = solve_tau(x, a, b)
    for _ in range(1, MAX_ITER + 1):
        a_old, b_old = a, b
        cj = np.cos(np.dot(tau, np.pi * np.array([[1, 2, 3]])))
        A11 = np.sum(cj ** 2, axis=0)
        A12 = np.sum(cj, axis=0)
        b1 = np.sum(x * cj, axis=0)
        b2 = np.sum(x, axis=0)
        coeff = np.zeros((2, 3))
        for q in range(3):
            coeff[:, q] = np.linalg.lstsq(np.array([[A11[q], A12[q]], [A12[q], nS]]),
                                          np.array([b1[q], b2[q]]))[0]
        a, b = coeff[0, :], coeff[1, :]
        tau = solve_tau(x, a, b)
        delta_a = np.max(np.fabs(a - a_old) / (np.fabs(a) + _EPS)) * 100
        delta_b = np.max(np.fabs(b - b_old) / (np.fabs(b) + _EPS)) * 100
        delta_tau = 0.0          # tau_old is tau itself in the reference
        if delta_a < DELTA_A_MAX and delta_b < DELTA_B_MAX and delta_tau < DELTA_TAU_MAX:
            break
    return a, b, tau
