"""NLSA stage of one projection direction on the GPU.

Drop-in for the reference's ``NLSA.op(NLSAPar, DD, posPath, posPsi1, imgAll, msk2, CTF, ExtPar)``
(``modules/NLSA.py:23-158``), which ``psiAnalysisParS2.op`` calls once per reaction coordinate
(``psiAnalysisParS2.py:94-96``) with the distance stage's ``D``, ``imgAll``, ``CTF`` and ``msk2``.
Same arguments, same 8-tuple ``(IMGT, Topo_mean, psirec, psiC1, sdiag, VX, mu, tau)`` of host
numpy arrays.

Split of the work:

* GPU, own kernels (``csrc/nlsa.cu`` through the C ABI): the concatenated distances ConD
  (``NLSA.py:31-34``, bit-identical) and the snapshot matrix A (``:63-86``): the Wiener
  denominators of ``get_wiener.op`` (``get_wiener.py:9-21``), the images' half-plane spectra (the
  shared-memory FFT of the distance stage), one banded frequency-domain correlation instead of the
  reference's c (num - c) transform pairs, c x psiTrunc inverse transforms, mask and transposed
  scatter;
* GPU, the diffusion maps of ``ConD`` and of the reconstructed frames' squared distances
  (``:45``, ``:146``) through ``manifoldem_python_gb300.DMembeddingII``;
* GPU library calls: the tall-skinny products of ``svdRF.op`` (``svdRF.py:18-36``), the
  reconstruction ``IMGT`` (``NLSA.py:112-128``) as one GEMM over the rank-2 ``ConImgT``, the frame
  normalisation and the frames' Gram matrix through the centred rank-2c basis (``L2_distance.op``,
  ``L2_distance.py:43-76``);
* host: the psiTrunc x psiTrunc eigen-decomposition of ``svdRF`` and the curve fit
  ``fit_1D_open_manifold_3D.op`` (vectorised, same results as the reference's per-point loop).

Eigenvector signs are arbitrary in the reference (ARPACK's start vector, LAPACK): ``psiC1`` and
``psirec`` columns, ``Topo_mean`` columns and ``VX`` rows agree with it up to sign; ``IMGT``,
``sdiag`` and ``mu`` do not depend on them; ``tau`` becomes ``1 - tau`` when the third column of
``psirec`` changes sign.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import DMembeddingII, _lib
from . import fit_1D_open_manifold_3D as _fit

PREFSIGMA_CON = 600000      # NLSA.py:45
PREFSIGMA_REC = 30          # NLSA.py:146


class _Gpu:
    def __init__(self, device):
        import torch
        self.torch = torch
        self.dev = torch.device(device or 'cuda')
        self.stream = torch.cuda.current_stream(self.dev)
        self.lib = _lib.load()

    def call(self, name, *args):
        _lib.check(getattr(self.lib, name)(*args, ctypes.c_void_p(self.stream.cuda_stream)),
                   name)

    def tensor(self, a, dtype, index=None):
        """a (numpy array or torch tensor), rows `index` taken first, on the device as dtype."""
        torch = self.torch
        if isinstance(a, torch.Tensor):
            t = a.to(self.dev)
            if index is not None:
                t = t.index_select(0, torch.as_tensor(index, device=self.dev))
        else:
            a = np.asarray(a)
            if index is not None:
                a = a[np.asarray(index)]
            t = torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)
        return t.to(dtype).contiguous()


def _check_even(ctf, torch):
    """The CTFs must be even in frequency (C(-k) = C(k) on the ifftshifted grid), as the
    distance stage's are, for the half-plane Wiener sum to equal the reference's full plane."""
    N = ctf.shape[-1]
    neg = (-torch.arange(N, device=ctf.device)) % N
    mirrored = ctf.index_select(1, neg).index_select(2, neg)
    scale = float(ctf.abs().max()) if ctf.numel() else 0.0
    if float((ctf - mirrored).abs().max()) > 1e-6 * max(scale, 1e-30):
        raise ValueError('NLSA.op: CTF is not even in frequency; the GPU Wiener sum needs '
                         'C(-k) = C(k) (every CTF of the distance stage is)')


def snapshots(g: _Gpu, images, ctf, mu_psi: np.ndarray, msk2, c: int):
    """A (c N^2, T) float64 on the device (NLSA.py:63-86); ctf None for the 'cuti' branch."""
    torch = g.torch
    num, N = int(images.shape[0]), int(images.shape[1])
    T = int(mu_psi.shape[1])
    mu_d = torch.from_numpy(np.ascontiguousarray(mu_psi, dtype=np.float64)).to(g.dev)
    msk_d = None
    if ctf is not None:
        m2 = np.asarray(msk2, dtype=np.float64)
        if m2.ndim == 0:
            if float(m2) != 1.0:
                msk_d = torch.full((N, N), float(m2), dtype=torch.float64, device=g.dev)
        else:
            msk_d = torch.from_numpy(np.ascontiguousarray(m2.reshape(N, N))).to(g.dev)
    nbytes = ctypes.c_size_t(0)
    _lib.check(g.lib.mem_nlsa_workspace_size(N, num, c, T, int(ctf is not None),
                                             ctypes.byref(nbytes)), 'mem_nlsa_workspace_size')
    ws = torch.empty(max(int(nbytes.value), 1), dtype=torch.uint8, device=g.dev)
    A = torch.empty((c * N * N, T), dtype=torch.float64, device=g.dev)
    g.call('mem_nlsa_snapshots', N, num, c, T, images.data_ptr(),
           ctf.data_ptr() if ctf is not None else None, mu_d.data_ptr(),
           msk_d.data_ptr() if msk_d is not None else None, ws.data_ptr(), nbytes.value,
           A.data_ptr())
    return A


def svd_rf(g: _Gpu, A):
    """svdRF.op for a tall A (svdRF.py:18-28): eigh of A^T A on the host, eigenpairs by decreasing
    value, U = A V S^-1 on the device.  Returns (U device, S, V host)."""
    D, V = np.linalg.eigh((A.T @ A).cpu().numpy())
    order = np.argsort(D)[::-1]
    D = np.sort(D)[::-1]
    V = V[:, order]
    with np.errstate(invalid='ignore', divide='ignore'):
        sq = np.sqrt(D)
        invS = np.diag(1. / sq)
    U = A @ g.torch.from_numpy(V @ invS).to(g.dev)
    return U, np.diag(sq), V


def op(NLSAPar: dict, DD, posPath, posPsi1, imgAll, msk2, CTF, ExtPar: dict,
       device: Optional[str] = None):
    """NLSA.op on the GPU: (IMGT, Topo_mean, psirec, psiC1, sdiag, VX, mu, tau)."""
    g = _Gpu(device)
    torch = g.torch
    num = int(NLSAPar['num'])
    c = int(NLSAPar['ConOrder'])
    k = NLSAPar['k']
    tune = NLSAPar['tune']
    nS = int(NLSAPar['nS'])
    psiTrunc = int(NLSAPar['psiTrunc'])
    if not 1 <= c < num:
        raise ValueError('NLSA.op: ConOrder must be in [1, num)')
    m = num - c
    DDt = g.tensor(DD, torch.float64)
    if DDt.shape[0] < num or DDt.shape[1] != num:
        raise ValueError('NLSA.op: DD must be num x num')
    ConD = torch.empty((m, m), dtype=torch.float64, device=g.dev)
    g.call('mem_nlsa_con_distances', DDt.data_ptr(), num, c, ConD.data_ptr())
    _, psiC, _, mu, _, _, _, _ = DMembeddingII.op(ConD, k, tune, PREFSIGMA_CON, device=g.dev)
    psiC1 = np.copy(psiC)
    if 'prD' in ExtPar:
        sel = np.asarray(posPath)[np.asarray(posPsi1)]
    elif 'cuti' in ExtPar:
        sel = np.asarray(posPsi1)
    else:
        raise ValueError("NLSA.op: ExtPar names neither 'prD' nor 'cuti'")
    sel = sel[:num]
    dim = int(CTF.shape[1])
    ell = psiTrunc - 1
    psiX = np.hstack((np.ones((psiC.shape[0], 1)), psiC[:, 0:ell]))
    mu_psi = mu.reshape((-1, 1)) * psiX
    images = g.tensor(imgAll, torch.float32, sel).reshape(num, dim, dim)
    ctf = None
    if 'prD' in ExtPar:
        ctf = g.tensor(CTF, torch.float32, sel).reshape(num, dim, dim)
        _check_even(ctf, torch)
    A = snapshots(g, images, ctf, mu_psi, msk2, c)
    del images, ctf
    U, S, V = svd_rf(g, A)
    del A
    VX = V.T @ psiX.T
    sdiag = np.diag(S)
    npix = dim * dim
    T = ell + 1
    U3 = U.view(c, npix, T)
    Topo_mean = U3[:, :, :psiTrunc].mean(dim=0).cpu().numpy()
    # IMGT[:, ii] = sum_{i < c} ConImgT_i psiX[i + ii]^T with ConImgT = sum_{r < 2} U_r s_r V_r^T
    # (NLSA.py:112-128): U_i[:, :2] w[i + ii], w = (psiX V[:, :2]) s[:2], as one GEMM
    n_loop = num - 2 * c
    n_out = nS - 2 * c
    w = torch.from_numpy((psiX @ V[:, :2]) * sdiag[:2]).to(g.dev)                   # (m, 2)
    Ucat = U3[:, :, :2].permute(1, 0, 2).reshape(npix, 2 * c)
    idx = (torch.arange(c, device=g.dev)[:, None] + torch.arange(n_loop, device=g.dev)[None, :])
    Wcat = w[idx].permute(0, 2, 1).reshape(2 * c, n_loop)
    IMGT = torch.zeros((npix, n_out), dtype=torch.float64, device=g.dev)
    IMGT[:, :n_loop] = Ucat @ Wcat
    mean = IMGT.mean(dim=0)
    std = IMGT.std(dim=0, unbiased=False)
    IMGT = (IMGT - mean) / std                                                       # :131-138
    # squared distances of the frames (L2_distance.py:71-76): the centred frame a is
    # Bc Wcat[:, a] with Bc = Ucat minus its column means, so the Gram matrix is
    # (Wcat/std)^T (Bc^T Bc) (Wcat/std)
    if n_out == n_loop:
        Bc = Ucat - Ucat.mean(dim=0, keepdim=True)
        Z = Wcat / std[None, :]
        G = Z.T @ ((Bc.T @ Bc) @ Z)
    else:
        G = IMGT.T @ IMGT
    aa = torch.diagonal(G)
    t = aa[:, None] + aa[None, :] - 2 * G
    t[t < 1e-8] = 0
    Drecon = torch.sqrt(t)
    lamb, psirec, _, mu_rec, _, _, _, _ = DMembeddingII.op(Drecon ** 2, min(npix, n_out), tune,
                                                           PREFSIGMA_REC, device=g.dev)
    _, _, tau = _fit.op(psirec)
    return (IMGT.cpu().numpy(), Topo_mean, psirec, psiC1, sdiag, VX, mu_rec, tau)
