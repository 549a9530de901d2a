"""Host-side per-PD bookkeeping of the distance stage, in float64 numpy as the reference does it.

These are O(n) per PD and stay on the host exactly like the reference keeps them in numpy:
image index/conjugate bookkeeping (``getDistanceCTF_local_Conj9combinedS2.py:245-252``), the
projection direction of the bin (``:169-185``, ``:297-301``), the per-image in-plane angles
(``:187-202``, ``:315-323``) and psi_p (``:206-213`` via ``q2Spider.op``, ``q2Spider.py:19-60``).
psi_p is a least-squares fit that stops at ftol=1e-12 before full convergence; the branch and the
last digits it lands on depend on the optimiser's path, so it is computed with the same
``scipy.optimize.least_squares`` call and residual arithmetic order as the reference.
"""
from __future__ import annotations

import dataclasses

import numpy as np
from scipy import optimize


@dataclasses.dataclass
class PdGeometry:
    ind: np.ndarray           # as given (the PD's indices into the augmented set)
    stack_index: np.ndarray   # int64 image of the stack read for each entry
    flip: np.ndarray          # uint8, 1 for conjugate views
    imgLabels: np.ndarray     # int, +1 plain / -1 conjugate
    PDs: np.ndarray           # (3, nS)
    PD: np.ndarray            # (3,)
    psi_p: float              # degrees
    Psis: np.ndarray          # (nS, 1)
    Nom: np.ndarray           # (nS, 1)
    Dnom: np.ndarray          # (nS, 1)
    psi_rad: np.ndarray       # (nS,) Psis with NaN replaced by 0, contiguous


def index_bookkeeping(ind: np.ndarray, nStot: int):
    """Stack index, flip flag and label of every entry (reference :246-252, :271): entries with
    ind >= nStot/2 (compared in floating point) are conjugate views of image ind - nStot/2."""
    ind = np.asarray(ind)
    half = nStot / 2
    conj = ind >= half
    stack_index = np.where(conj, (ind - half), ind).astype(np.int64)
    labels = np.where(conj, -1, 1).astype(int)
    return stack_index, conj.astype(np.uint8), labels


def calc_avg_pd(q: np.ndarray, nS: int) -> np.ndarray:
    return 2 * np.vstack((q[1, :] * q[3, :] - q[0, :] * q[2, :],
                          q[0, :] * q[1, :] + q[2, :] * q[3, :],
                          q[0, :] ** 2 + q[3, :] ** 2 - np.ones((1, nS)) / 2.0))


def _hamilton(q: np.ndarray, s: np.ndarray) -> np.ndarray:
    # same operation order as the reference's qMult_bsx so the optimiser sees identical values
    q0, qv = q[0:1, :][0], q[1:4, :]
    s0, sv = s[0:1, :][0], s[1:4, :]
    cr = np.vstack((qv[1, :] * sv[2, :] - qv[2, :] * sv[1, :],
                    qv[2, :] * sv[0, :] - qv[0, :] * sv[2, :],
                    qv[0, :] * sv[1, :] - qv[1, :] * sv[0, :]))
    return np.vstack((q0 * s0 - np.sum(qv * sv, axis=0), q0 * sv + s0 * qv + cr))


def spider_psi(qr: np.ndarray) -> float:
    """Spider psi (radians) of a unit quaternion by the reference's least-squares fit."""
    return spider_euler(qr)[2]


def spider_euler(qr: np.ndarray):
    """Spider (phi, theta, psi) in radians of a unit quaternion: the least-squares fit of
    q2Spider.op (modules/q2Spider.py:19-60), same start, bounds and tolerance."""
    qr = qr / np.sqrt(sum(qr ** 2))

    def residual(a):
        c0, s0 = np.cos(a[0] / 2.), np.sin(a[0] / 2.)
        c1, s1 = np.cos(a[1] / 2.), np.sin(a[1] / 2.)
        c2, s2 = np.cos(a[2] / 2.), np.sin(a[2] / 2)
        qa = np.array([c0, 0., 0., -s0]).reshape(-1, 1)
        qb = np.array([c1, 0, -s1, 0.]).reshape(-1, 1)
        qc = np.array([c2, 0., 0., -s2]).reshape(-1, 1)
        return qr - _hamilton(qc, _hamilton(qb, qa)).flatten()

    res = optimize.least_squares(residual, np.array([0, 0, 0]), bounds=(-np.inf, np.inf),
                                 ftol=1e-12)
    return res.x[0], res.x[1], res.x[2]


def spider_rotation(phi: float, theta: float, psi: float) -> np.ndarray:
    """Rotation matrix of Spider Euler angles (radians), projectMask.eulerRotMatrix3DSpider
    (modules/projectMask.py:48-58)."""
    cf, sf = np.cos(phi), np.sin(phi)
    ct, st = np.cos(theta), np.sin(theta)
    cp, sp = np.cos(psi), np.sin(psi)
    return np.array([[cf * cp * ct - sf * sp, cp * ct * sf + cf * sp, -cp * st],
                     [-cp * sf - cf * ct * sp, cf * cp - ct * sf * sp, sp * st],
                     [cf * st, sf * st, ct]])


def mask_transform(PD: np.ndarray, N: int):
    """The affine map of projectMask.op (modules/projectMask.py:120-131) for projection
    direction PD: output voxel o of the (axis-0/2 swapped) mask volume samples the input at
    R o + offset.  Returns (R (3, 3), offset (3,))."""
    Qr = np.array([1 + PD[2], PD[1], -PD[0], 0]).T
    q1 = Qr / np.sqrt(sum(Qr ** 2))
    phi, theta, psi = spider_euler(q1)
    sym = np.array([phi, theta, psi])
    sym[2] = 0
    sym = sym * (-1.)
    R = spider_rotation(sym[2], sym[1], sym[0])
    c = 0.5 * np.array([N, N, N], dtype=np.float64)
    return R, c - np.dot(R, c)


def psi_ang(PD: np.ndarray) -> float:
    Qr = np.array([1 + PD[2], PD[1], -PD[0], 0])
    Qr = Qr / np.sqrt(np.sum(Qr ** 2))
    psi = spider_psi(Qr)
    return float(np.mod(psi, 2 * np.pi) * (180 / np.pi))


def pd_geometry(ind: np.ndarray, q: np.ndarray, nStot: int, psi_p: float = None) -> PdGeometry:
    nS = ind.shape[0]
    stack_index, flip, labels = index_bookkeeping(ind, nStot)
    PDs = calc_avg_pd(q, nS)
    PD = np.sum(PDs, 1)
    PD = PD / np.linalg.norm(PD)
    if psi_p is None:
        psi_p = psi_ang(PD)
    s = -(1 + PD[2]) * q[3, :] - PD[0] * q[1, :] - PD[1] * q[2, :]
    c = (1 + PD[2]) * q[0, :] + PD[1] * q[1, :] - PD[0] * q[2, :]
    with np.errstate(divide='ignore', invalid='ignore'):
        Psi = 2 * np.arctan(s / c)
    Psi = np.where(np.isnan(Psi), 0.0, Psi)
    return PdGeometry(ind=ind, stack_index=stack_index, flip=flip, imgLabels=labels, PDs=PDs,
                      PD=PD, psi_p=psi_p, Psis=Psi.reshape(nS, 1).astype(np.float64),
                      Nom=s.reshape(nS, 1).astype(np.float64),
                      Dnom=c.reshape(nS, 1).astype(np.float64),
                      psi_rad=np.ascontiguousarray(Psi, dtype=np.float64))
