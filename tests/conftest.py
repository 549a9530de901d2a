import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, 'tests', 'golden')
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN_CASES = ['even32_conj', 'odd33_env', 'even32_avgonly', 'even48_neardup', 'config1',
                'relion32', 'volmask32']


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (sm_103) and the built library')


def load_golden(case):
    z = np.load(os.path.join(GOLDEN, case + '.npz'))
    return {k: z[k] for k in z.files}


def golden_options(g):
    return dict(verbose=False, avgOnly=bool(g['avgOnly']), visual=False, parallel=False,
                relion_data=golden_relion(g), thres=6000)


def golden_relion(g):
    return bool(g['relion']) if 'relion' in g else False


def golden_mask_volume(g):
    """The mask volume of a case run with p.mask_vol_file, else None."""
    v = g.get('mask_volume')
    return v.astype(np.float32) if v is not None and v.size else None


def golden_shifts(g):
    """(shx, shy) of a RELION case, else None."""
    return (g['shx'], g['shy']) if golden_relion(g) else None


def golden_micro(g):
    return dict(N=int(g['N']), pix_size=float(g['pix_size']), Cs=float(g['Cs']),
                EkV=float(g['EkV']), AmpContrast=float(g['AmpContrast']),
                gaussEnv=float(g['gaussEnv']))


def golden_ref(g, key):
    """Reference output `key`, restricted to the stored image slices when the case keeps only
    slices; returns (array, slice index or None)."""
    if 'ref_' + key in g:
        return g['ref_' + key], None
    return g['ref_%s_slices' % key], g['slice_idx']


@pytest.fixture(scope='session')
def cuda_ready():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from manifoldem_python_gb300 import _lib
    _lib.build()
    _lib.load()
    return torch


# ---- NLSA fixtures (tests/golden/nlsa32.npz, made by make_golden.py from the reference) -------

NLSA_RUNS = {'a': 'prD', 'b': 'prD-mask', 'c': 'cuti'}


def nlsa_golden_args(g, tag):
    """Arguments of NLSA.op for run `tag` of an NLSA fixture, as psiAnalysisParS2.op builds them
    (psiAnalysisParS2.py:57-96): all images on the path, ordered along diffusion coordinate 0."""
    D = g['D']
    nS = D.shape[0]
    c = int(g['ConOrder'])
    P = g['PosPsi1']
    par = dict(num=nS, ConOrder=c, k=nS - c, tune=3, nS=nS, save=False, psiTrunc=8)
    msk2 = g['msk_disc'] if tag == 'b' else np.array(1)
    ext = dict(cuti=0) if tag == 'c' else dict(outDir='', prD=0)
    return (par, D[P][:, P], np.arange(nS), P, g['imgAll'].astype(np.float64), msk2,
            g['CTF'].astype(np.float64), ext)


def _sign_align(x, ref, axis):
    s = np.sign(np.sum(x * ref, axis=axis, keepdims=True))
    s[s == 0] = 1
    return x * s


def nlsa_errors(out, ref):
    """Differences of an NLSA.op result from a reference result, each eigenvector-derived array
    aligned in sign first (IMGT, sdiag and mu do not depend on eigenvector signs; tau is compared
    with 1 - tau_ref when the third psirec column has the opposite sign)."""
    from scipy.linalg import subspace_angles
    IMGT, Topo, psirec, psiC1, sdiag, VX, mu, tau = out
    r_IMGT, r_Topo, r_psirec, r_psiC1, r_sdiag, r_VX, r_mu, r_tau = ref
    flip = np.sum(psirec[:, 2] * r_psirec[:, 2]) < 0
    return dict(
        IMGT=float(np.abs(IMGT - r_IMGT).max()),
        sdiag=float((np.abs(sdiag - r_sdiag) / r_sdiag).max()),
        Topo=float(np.abs(_sign_align(Topo, r_Topo, 0) - r_Topo).max() / np.abs(r_Topo).max()),
        VX=float(np.abs(_sign_align(VX, r_VX, 1) - r_VX).max() / np.abs(r_VX).max()),
        psiC1=float(np.abs(_sign_align(psiC1, r_psiC1, 0) - r_psiC1)[:, :3].max()),
        psirec=float(np.abs(_sign_align(psirec, r_psirec, 0) - r_psirec)[:, :3].max()),
        psirec8=float(np.max(subspace_angles(psirec[:, :8], r_psirec[:, :8]))),
        mu=float(np.abs(mu - r_mu).max()),
        tau=float(np.abs(tau - ((1 - r_tau) if flip else r_tau)).max()),
    )


def nlsa_golden_ref(g, tag):
    return tuple(g['%s_%s' % (tag, k)].astype(np.float64) for k in
                 ('IMGT', 'Topo_mean', 'psirec', 'psiC1', 'sdiag', 'VX', 'mu', 'tau'))
