"""FP64 CPU oracle of ManifoldEM's per-PD CTF-distance stage (test infrastructure only).

A numpy/scipy restatement of ``getDistanceCTF_local_Conj9combinedS2.op`` (reference
``modules/getDistanceCTF_local_Conj9combinedS2.py:216-420``) and of the helpers it calls.  Every
function cites the reference lines it follows.  Arithmetic is float64 throughout, as in the
reference.  Two deliberate restatements:

* ``rotatefill.op`` (``modules/rotatefill.py:21-25``) tiles the image 3x3 and calls
  ``scipy.ndimage.rotate(order=3)``.  Because the tile is three periods wide and the spline
  prefilter pole (sqrt(3)-2) decays to nothing over one period, that equals a *periodic* cubic
  B-spline rotation about ((N-1)/2, (N-1)/2); the oracle evaluates it directly with
  ``map_coordinates(order=3, mode='grid-wrap')`` (agreement <= 1.4e-13 relative, checked in
  ``tests/test_oracle.py``).
* ``q2Spider.op`` (``modules/q2Spider.py:19-60``) is restated with the same
  ``scipy.optimize.least_squares`` call and the same residual arithmetic order: the optimiser stops
  at ftol=1e-12 before full convergence, so the branch it lands on and its last digits depend on
  that path, and the distance stage inherits them through psi_p.
"""
from __future__ import annotations

import math
import os
from typing import Dict, Optional, Sequence

import numpy as np
from scipy import ndimage, optimize
from scipy.fftpack import fft2, ifft2, ifftshift

VERSION = 'getDistanceCTF_local9, V 1.0'     # value of the module-level ``version`` string (:40)
WIENER_SNR = 5                               # get_wiener1 (:423)

OUTPUT_KEYS = ['D', 'ind', 'q', 'df', 'CTF', 'imgAll', 'msk2', 'PD', 'PDs', 'Psis', 'imgAvg',
               'imgAvgFlip', 'imgAllFlip', 'imgLabels', 'Dnom', 'Nom', 'imgAllIntensity',
               'version', 'options']        # myio.fout1 key list (:409-412)


# ----------------------------------------------------------------------------- small helpers
def annular_mask(a: float, b: float, N: int, M: int) -> np.ndarray:
    """``annularMask.op`` (``modules/annularMask.py:19-32``): 1 where a^2 <= r^2 < b^2 about
    (N/2-1, M/2)."""
    x = np.arange(N, dtype=np.float64)[:, None] - N / 2 + 1
    y = np.arange(M, dtype=np.float64)[None, :] - M / 2
    r2 = x * x + y * y
    return ((r2 >= a * a) & (r2 < b * b)).astype(np.float64)


def create_grid(N: int) -> np.ndarray:
    """Radial frequency grid Q in units of Nyquist (``:139-154``)."""
    if N % 2 == 1:
        a = np.arange(-(N - 1) / 2, (N - 1) / 2 + 1)
    else:
        a = np.arange(-N / 2., N / 2)
    X, Y = np.meshgrid(a, a)
    return (1. / (N / 2.)) * np.sqrt(X ** 2 + Y ** 2)


def create_filter(filter_type: str, order: float, Qc: float, Q: np.ndarray) -> np.ndarray:
    """Butterworth / Gaussian low-pass (``:156-167``)."""
    if filter_type == 'Gauss':
        return np.exp(-(np.log(2) / 2.) * (Q / Qc) ** 2)
    if filter_type == 'Butter':
        return np.sqrt(1. / (1 + (Q / Qc) ** (2 * order)))
    raise ValueError('%s filter is unsupported' % filter_type)


def ctf_cryo_frank(k: np.ndarray, Cs: float, df: float, kev: float, B: float, ampc: float) -> np.ndarray:
    """``ctemh_cryoFrank.op`` (``modules/ctemh_cryoFrank.py:24-44``).  k in 1/A, Cs in mm, df in A,
    B the Gaussian envelope half-width (inf = no envelope)."""
    Cs = Cs * 1.0e7
    wav = 12.3986 / np.sqrt((2 * 511.0 + kev) * kev)
    w1 = np.pi * Cs * wav * wav * wav
    w2 = np.pi * wav * df
    k2 = k * k
    sigm = B / math.sqrt(2 * math.log(2))
    wi = np.exp(-k2 / (2 * sigm ** 2))
    wr = (0.5 * w1 * k2 - w2) * k2
    return (np.sin(wr) - ampc * np.cos(wr)) * wi


def rotate_periodic(img: np.ndarray, angle_deg: float) -> np.ndarray:
    """``rotatefill.op`` (``modules/rotatefill.py:21-25``) as a periodic cubic B-spline rotation.

    out[r, c] = spline(cos t (r-c0) + sin t (c-c0) + c0, -sin t (r-c0) + cos t (c-c0) + c0),
    t = radians(angle_deg), c0 = (N-1)/2, indices wrapped modulo N."""
    N = img.shape[0]
    c0 = (N - 1) / 2.0
    t = np.deg2rad(angle_deg)
    r, c = np.meshgrid(np.arange(N, dtype=np.float64), np.arange(N, dtype=np.float64), indexing='ij')
    x = np.cos(t) * (r - c0) + np.sin(t) * (c - c0) + c0
    y = -np.sin(t) * (r - c0) + np.cos(t) * (c - c0) + c0
    return ndimage.map_coordinates(img, [x, y], order=3, mode='grid-wrap')


def calc_avg_pd(q: np.ndarray, nS: int) -> np.ndarray:
    """Per-image projection directions from quaternions (``:169-185``)."""
    return 2 * np.vstack((q[1, :] * q[3, :] - q[0, :] * q[2, :],
                          q[0, :] * q[1, :] + q[2, :] * q[3, :],
                          q[0, :] ** 2 + q[3, :] ** 2 - np.ones((1, nS)) / 2.0))


def get_psi(q: np.ndarray, PD: np.ndarray, iS: int):
    """In-plane angle of image iS relative to PD (``:187-202``)."""
    s = -(1 + PD[2]) * q[3, iS] - PD[0] * q[1, iS] - PD[1] * q[2, iS]
    c = (1 + PD[2]) * q[0, iS] + PD[1] * q[1, iS] - PD[0] * q[2, iS]
    with np.errstate(divide='ignore', invalid='ignore'):
        Psi = 2 * np.arctan(s / c)
    return Psi, s, c


def _qmult(q: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Quaternion product in the operation order of ``qMult_bsx.op`` (``modules/qMult_bsx.py:14-34``),
    kept alike so the least-squares path below sees identical residuals."""
    q = q.reshape(-1, 1) if q.ndim < 2 else q
    s = s.reshape(-1, 1) if s.ndim < 2 else s
    q0, qv = q[0, :], q[1:4, :]
    s0, sv = s[0, :], s[1:4, :]
    cr = np.vstack((qv[1, :] * sv[2, :] - qv[2, :] * sv[1, :],
                    qv[2, :] * sv[0, :] - qv[0, :] * sv[2, :],
                    qv[0, :] * sv[1, :] - qv[1, :] * sv[0, :]))
    return np.vstack((q0 * s0 - np.sum(qv * sv, axis=0), q0 * sv + s0 * qv + cr))


def spider_angles(q: np.ndarray):
    """``q2Spider.op`` (``modules/q2Spider.py:19-60``): Spider (phi, theta, psi) of a unit
    quaternion by least squares from (0, 0, 0)."""
    q = q / np.sqrt(sum(q ** 2))

    def resid(a):
        q1 = np.array([np.cos(a[0] / 2.), 0., 0., -np.sin(a[0] / 2.)])
        q2 = np.array([np.cos(a[1] / 2.), 0, -np.sin(a[1] / 2.), 0.])
        q3 = np.array([np.cos(a[2] / 2.), 0., 0., -np.sin(a[2] / 2)])
        return q - _qmult(q3, _qmult(q2, q1)).flatten()

    res = optimize.least_squares(resid, np.array([0, 0, 0]), bounds=(-np.inf, np.inf), ftol=1e-12)
    return res.x[0], res.x[1], res.x[2]


def psi_ang(PD: np.ndarray) -> float:
    """In-plane angle (degrees, [0, 360)) that brings PD to the Spider frame (``:206-213``)."""
    Qr = np.array([1 + PD[2], PD[1], -PD[0], 0])
    Qr = Qr / np.sqrt(np.sum(Qr ** 2))
    _, _, psi = spider_angles(Qr)
    return np.mod(psi, 2 * np.pi) * (180 / np.pi)


def get_wiener1(CTF1: np.ndarray) -> np.ndarray:
    """Wiener denominator sum_i CTF_i^2 + 1/SNR (``:422-430``)."""
    wiener_dom = 0.
    for i in range(CTF1.shape[0]):
        wiener_dom = wiener_dom + CTF1[i, :, :] ** 2
    return wiener_dom + 1. / WIENER_SNR


# ----------------------------------------------------------------------------- image reading
def read_image(stack, idx: int, N: int) -> np.ndarray:
    """SPIDER raw stack image ``idx`` as the stage sees it (``:254-258``): elements
    [idx*N*N, (idx+1)*N*N) as an (N, N) array, transposed.  ``stack`` is a file name or an array
    of shape (num_part, N, N) / (num_part*N*N,)."""
    if isinstance(stack, (str, os.PathLike)):
        tmp = np.memmap(stack, dtype='float32', offset=N * N * idx * 4, mode='r', shape=(N, N))
    else:
        tmp = np.asarray(stack).reshape(-1, N, N)[idx]
    return np.array(tmp.T, dtype=np.float32)


def read_image_relion(stack, idx: int, sh) -> np.ndarray:
    """RELION image ``idx`` as the stage sees it (``:259-264``): the MRC stack's image as stored
    (no transpose), shifted by (sh[1][idx] - 0.5, sh[0][idx] - 0.5) with
    ``scipy.ndimage.shift(order=3, mode='wrap')``.  ``stack``: array (num_part, N, N)."""
    from scipy.ndimage import shift
    tmp = np.asarray(stack)[idx]
    return shift(tmp, (sh[1][idx] - 0.5, sh[0][idx] - 0.5), order=3, mode='wrap')


def load_pd_images(stack, ind: np.ndarray, nStot: int, N: int, msk: np.ndarray, sh=None):
    """Images of one PD with conjugates flipped and background-normalised (``:245-283``);
    ``sh`` = (shx, shy) selects the RELION branch (``read_image_relion``).

    Returns (images (nS, N, N) float64, imgLabels (nS,) int)."""
    nS = ind.shape[0]
    out = np.zeros((nS, N, N))
    labels = np.zeros(nS, dtype=int)
    for iS in range(nS):
        if ind[iS] < nStot / 2:
            idx = int(ind[iS])
            labels[iS] = 1
        else:
            idx = int(ind[iS] - nStot / 2)
            labels[iS] = -1
        tmp = read_image(stack, idx, N) if sh is None else read_image_relion(stack, idx, sh)
        if ind[iS] >= nStot / 2:
            tmp = np.flipud(tmp)
        backg = tmp * (1 - msk)
        with np.errstate(divide='ignore', invalid='ignore'):
            tmp = (tmp - backg.mean()) / backg.std()
        out[iS] = tmp
    return out, labels


def project_mask(vol: np.ndarray, PD: np.ndarray) -> np.ndarray:
    """projectMask.op (modules/projectMask.py:118-135): the mask volume rotated to the
    projection direction (scipy affine_transform, order 3, mode 'nearest'), summed along z,
    thresholded at 1; (N, N) bool."""
    from scipy.ndimage import affine_transform
    from scipy import optimize
    vol = np.swapaxes(vol, 0, 2)
    N = vol.shape[0]
    # getEuler_from_PD (:93-108) with q2Spider.op's least-squares fit (q2Spider.py:19-60)
    Qr = np.array([1 + PD[2], PD[1], -PD[0], 0]).T
    q1 = Qr / np.sqrt(sum(Qr ** 2))

    def qmul(q, s):
        return np.array([q[0] * s[0] - q[1] * s[1] - q[2] * s[2] - q[3] * s[3],
                         q[0] * s[1] + q[1] * s[0] + q[2] * s[3] - q[3] * s[2],
                         q[0] * s[2] - q[1] * s[3] + q[2] * s[0] + q[3] * s[1],
                         q[0] * s[3] + q[1] * s[2] - q[2] * s[1] + q[3] * s[0]])

    def dev(a):
        qa = np.array([np.cos(a[0] / 2.), 0., 0., -np.sin(a[0] / 2.)])
        qb = np.array([np.cos(a[1] / 2.), 0, -np.sin(a[1] / 2.), 0.])
        qc = np.array([np.cos(a[2] / 2.), 0., 0., -np.sin(a[2] / 2)])
        return q1 - qmul(qc, qmul(qb, qa))

    a = optimize.least_squares(dev, np.array([0, 0, 0]), bounds=(-np.inf, np.inf),
                               ftol=1e-12).x
    Phi, Theta, Psi = -0.0, -a[1], -a[0]            # sym = -[phi, theta, 0], (sym[2], sym[1], sym[0])
    R = np.array([[np.cos(Phi) * np.cos(Psi) * np.cos(Theta) - np.sin(Phi) * np.sin(Psi),
                   np.cos(Psi) * np.cos(Theta) * np.sin(Phi) + np.cos(Phi) * np.sin(Psi),
                   -np.cos(Psi) * np.sin(Theta)],
                  [-np.cos(Psi) * np.sin(Phi) - np.cos(Phi) * np.cos(Theta) * np.sin(Psi),
                   np.cos(Phi) * np.cos(Psi) - np.cos(Theta) * np.sin(Phi) * np.sin(Psi),
                   np.sin(Psi) * np.sin(Theta)],
                  [np.cos(Phi) * np.sin(Theta), np.sin(Phi) * np.sin(Theta), np.cos(Theta)]])
    c = 0.5 * np.array(vol.shape, dtype=np.float64)
    offset = c - np.dot(R, c)
    rho = affine_transform(input=vol, matrix=R, offset=offset, output_shape=vol.shape,
                           mode='nearest')
    msk = np.sum(rho, axis=2).reshape(N, N).T
    return msk > 1


# ----------------------------------------------------------------------------- the stage
def pd_op(ind: np.ndarray, q: np.ndarray, df: np.ndarray, stack, nStot: int, *, N: int,
          pix_size: float, Cs: float, EkV: float, AmpContrast: float, gaussEnv: float = np.inf,
          filterPar: Optional[dict] = None, options: Optional[dict] = None,
          psi_p: Optional[float] = None, msk2=1, sh=None,
          mask_volume=None) -> Dict[str, object]:
    """The 19 outputs of one PD (``getDistanceCTF_local_Conj9combinedS2.op`` ``:216-412``).

    ``psi_p`` may be passed in to skip the least-squares fit (it is then used as given);
    ``sh`` = (shx, shy) per stack image selects the RELION branch (``stack`` is then the MRC
    stack's (num_part, N, N) array); ``mask_volume`` (the volume of p.mask_vol_file) gives the
    projected mask msk2 of the PD."""
    filterPar = filterPar or dict(type='Butter', Qc=0.5, N=8)
    options = options if options is not None else dict(verbose=False, avgOnly=False, visual=False,
                                                        parallel=False, relion_data=False,
                                                        thres=None)
    nS = ind.shape[0]
    msk = annular_mask(0, N / 2., N, N)
    imgs, imgLabels = load_pd_images(stack, ind, nStot, N, msk, sh)

    # Butterworth low-pass of every image (:286-293)
    Q = create_grid(N)
    G = ifftshift(create_filter(filterPar['type'], filterPar['N'], filterPar['Qc'], Q))
    for iS in range(nS):
        imgs[iS] = ifft2(fft2(imgs[iS]) * G).real

    # projection direction of the bin and its in-plane angle (:297-313)
    PDs = calc_avg_pd(q, nS)
    PD = np.sum(PDs, 1)
    PD = PD / np.linalg.norm(PD)
    if psi_p is None:
        psi_p = psi_ang(PD)
    if mask_volume is not None:                          # (:303-310)
        msk2 = project_mask(mask_volume, PD)

    Psis = np.nan * np.ones((nS, 1))
    Nom = np.nan * np.ones((nS, 1))
    Dnom = np.nan * np.ones((nS, 1))
    imgAll = np.zeros((nS, N, N))
    imgAllFlip = np.zeros((nS, N, N))
    imgAvgFlip = np.zeros((N, N))
    CTF = np.zeros((nS, N, N))
    fy = np.zeros((nS, N, N), dtype=np.complex128)
    kgrid = Q / (2 * pix_size)
    for iS in range(nS):                                  # (:315-349)
        Psi, s, c = get_psi(q, PD, iS)
        if np.isnan(Psi):
            Psi = 0
        Psis[iS] = Psi
        Dnom[iS] = c
        Nom[iS] = s
        img = imgs[iS] * msk
        img = rotate_periodic(img, -(180 / math.pi) * Psi)
        img = rotate_periodic(img, -psi_p)
        CTF[iS] = ifftshift(ctf_cryo_frank(kgrid, Cs, df[iS], EkV, gaussEnv, AmpContrast))
        fy[iS] = fft2(img * msk2)
        imgFlip = ifft2(np.sign(CTF[iS]) * fy[iS])
        imgAllFlip[iS] = imgFlip.real
        imgAvgFlip = imgAvgFlip + imgFlip.real
        imgAll[iS] = img

    wiener_dom = -get_wiener1(CTF)                         # (:353-361)
    imgAvg = 0
    for iS in range(nS):
        imgAvg = imgAvg + ifft2(fft2(imgAll[iS]) * (CTF[iS] / wiener_dom)).real
    imgAvg = imgAvg * msk2 / nS                            # (:366-367)
    imgAvgFlip = imgAvgFlip.real * msk2 / nS

    D = np.zeros((nS, nS))
    CTF_out = CTF
    if not options['avgOnly']:                             # (:376-397)
        CTF_out = CTF.reshape(nS, N ** 2)
        D = distances_fp64(CTF_out, fy.reshape(nS, N ** 2))
    imgAllIntensity = np.mean(imgAllFlip ** 2, axis=0)     # (:400)

    vals = [D, ind, q, df, CTF_out, imgAll, msk2, PD, PDs, Psis, imgAvg, imgAvgFlip, imgAllFlip,
            imgLabels, Dnom, Nom, imgAllIntensity, VERSION, options]
    return dict(zip(OUTPUT_KEYS, vals))


def distances_fp64(CTF: np.ndarray, fy: np.ndarray) -> np.ndarray:
    """All-pairs D_ij = sum_k |CTF_j F_i - CTF_i F_j|^2 in the reference's GEMM form (``:391-397``):
    A = CTF^2 (|fy|^2)^T, D = A + A^T - 2 Re(H H^H), H = CTF * fy."""
    H = CTF.conj() * fy
    A = np.dot(np.abs(CTF) ** 2, (np.abs(fy) ** 2).T)
    return A + A.T - 2 * np.real(np.dot(H, H.conj().T))


def distances_direct(CTF: np.ndarray, fy: np.ndarray) -> np.ndarray:
    """Cancellation-free D_ij = sum_k |CTF_j F_i - CTF_i F_j|^2, one pair at a time (the blockwise
    variant ``conquer`` ``:106-122``).  O(n^2 K); small n only."""
    n = CTF.shape[0]
    D = np.zeros((n, n))
    for i in range(n):
        diff = CTF[i][None, :] * fy - CTF * fy[i][None, :]
        D[i] = np.sum(np.abs(diff) ** 2, axis=1)
    return D


# ----------------------------------------------------------------------------- half-plane features
def half_plane_weights(N: int) -> np.ndarray:
    """Weights of the last-axis half spectrum kx in [0, N//2]: 1 for kx = 0 and (even N) kx = N/2,
    else 2, so that sum_full f = sum_half w f for any f with f(-k) = conj-symmetric magnitude."""
    w = np.full(N // 2 + 1, 2.0)
    w[0] = 1.0
    if N % 2 == 0:
        w[-1] = 1.0
    return w


def distances_from_half_plane(C: np.ndarray, F: np.ndarray, N: int) -> np.ndarray:
    """D from half-plane spectra C (n, N, N//2+1) real and F (n, N, N//2+1) complex, in FP64 with the
    same algebra as the full-plane reference (the CTF is even in k, |F| is Hermitian-even)."""
    n = C.shape[0]
    w = half_plane_weights(N)[None, None, :]
    Cf = np.broadcast_to(C, F.shape).reshape(n, -1)
    Ff = (F * np.sqrt(w)).reshape(n, -1)
    return distances_fp64(Cf, Ff)
