"""The manifold-trimming drop-in (manifoldem_python_gb300.manifoldTrimmingAuto.op) on the GPU
diffusion map, against the reference's own manifoldTrimmingAuto.op (golden fixtures made by
tests/golden/make_golden.py): config1's D (300 images, 70 px) at rad 5 (no point trimmed, one
embedding) and rad 3 (9 embeddings, 260 kept), and the 160-image PD of nlsa32 at rad 3.

Tolerances (those of the GPU embedding): the kept points exactly (the nearest radius to ``rad``
is at least 3.7e-4 away from it in every iteration of these cases, the embedding's coordinates
agree to about 1e-6); sigma 1e-5 relative; eigenvalues 1e-6; mu 1e-5 relative; top-8 diffusion
coordinates 1e-4 rad; log sum_ij W_ij 1e-6; the eigenvalue file line by line, values to 1e-5
(the file rounds to 5 decimals).
"""
import os
import pickle

import numpy as np
import pytest
from scipy.linalg import subspace_angles

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _eig_lines(text):
    rows = [line.split('\t') for line in text.strip().split('\n')]
    return np.array([int(a) for a, _ in rows]), np.array([float(b) for _, b in rows])


@pytest.mark.parametrize('name,r', [('trim_config1', 0), ('trim_config1', 1), ('trim_nlsa32', 0)])
def test_trimming_matches_reference(cuda_ready, tmp_path, monkeypatch, name, r):
    from manifoldem_python_gb300 import manifoldTrimmingAuto, myio, p
    g = load_golden(name)
    src = load_golden(str(g['source']))
    D = src['ref_D'] if 'ref_D' in src else src['D']
    monkeypatch.setattr(p, 'psi_prog', str(tmp_path / 'progress'), raising=False)
    os.makedirs(p.psi_prog)
    dist_file, psi_file, eig_file = (str(tmp_path / x) for x in ('dist', 'psi', 'eig.txt'))
    myio.fout1(dist_file, ['D', 'ind'], [D, g['ind']])
    np.random.seed(int(g['seed']))
    manifoldTrimmingAuto.op([dist_file, psi_file, eig_file, 3], 0, 3, float(g['rads'][r]), False,
                            dict(outputFile='', Is=True))
    with open(psi_file, 'rb') as f:
        out = pickle.load(f)
    ref = {k[len('r%d_' % r):]: v for k, v in g.items() if k.startswith('r%d_' % r)}
    np.testing.assert_array_equal(out['posPath'], ref['posPath'])
    sig_err = abs(out['sigma'] - float(ref['sigma'])) / float(ref['sigma'])
    lam_err = np.abs(out['lamb'] - ref['lamb']).max()
    ang = float(np.max(subspace_angles(out['psi'][:, :8], ref['psi'][:, :8])))
    print('%s rad %g: kept %d, sigma %.2g, lamb %.2g, psi %.2g rad'
          % (name, g['rads'][r], len(out['posPath']), sig_err, lam_err, ang))
    assert sig_err < 1e-5 and lam_err < 1e-6 and ang < 1e-4
    np.testing.assert_allclose(out['mu'], ref['mu'], rtol=1e-5, atol=0)
    np.testing.assert_allclose(out['logSumWij'], ref['logSumWij'], rtol=0, atol=1e-6)
    np.testing.assert_array_equal(out['logEps'], ref['logEps'])
    assert out['psi'].shape == ref['psi'].shape
    assert os.listdir(p.psi_prog) == ['3']
    with open(eig_file) as f:
        idx, val = _eig_lines(f.read())
    idx_r, val_r = _eig_lines(str(ref['eig_txt']))
    np.testing.assert_array_equal(idx, idx_r)
    np.testing.assert_allclose(val, val_r, rtol=0, atol=1.01e-5)
