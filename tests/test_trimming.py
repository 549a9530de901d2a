"""Manifold trimming (manifoldTrimmingAuto.op, modules/manifoldTrimmingAuto.py:38-95): the FP64
restatement in oracle/trimming.py against the reference's own op (golden fixtures
tests/golden/trim_*.npz), and the drop-in module's host side (the loop, the psi pickle, the
progress marker and the eigenvalue file) with the oracle's embedding standing in for the GPU
one, which the GPU tests cover.

Tolerances of the oracle against the reference: the kept points exactly; sigma 1e-6 relative,
eigenvalues 1e-8, mu 1e-7 relative, top-8 diffusion coordinates 1e-7 rad.  The tanh fit of the
bandwidth sweep stops at curve_fit's own tolerance, so a re-embedding's sigma can land a little
away from the reference's (1.9e-7 relative on the 150-point re-embedding of trim_nlsa32; about
1e-10 elsewhere)."""
import os
import pickle

import numpy as np
import pytest
from scipy.linalg import subspace_angles

from conftest import load_golden


def _case(name):
    g = load_golden(name)
    src = load_golden(str(g['source']))
    g['D'] = src['ref_D'] if 'ref_D' in src else src['D']
    return g


@pytest.mark.parametrize('name,r', [('trim_nlsa32', 0), ('trim_config1', 0)])
def test_oracle_trimming_matches_reference(name, r):
    from oracle.trimming import trim
    g = _case(name)
    rad = float(g['rads'][r])
    lamb, psi, sigma, mu, keep, runs = trim(g['D'], 3, rad, seed=int(g['seed']))
    print('%s rad %g: %d embeddings, kept %d of %d' % (name, rad, runs, len(keep), len(g['D'])))
    np.testing.assert_array_equal(keep, g['r%d_posPath' % r])
    assert abs(sigma - float(g['r%d_sigma' % r])) / sigma < 1e-6
    np.testing.assert_allclose(lamb, g['r%d_lamb' % r], rtol=0, atol=1e-8)
    np.testing.assert_allclose(mu, g['r%d_mu' % r], rtol=1e-7, atol=0)
    assert np.max(subspace_angles(psi[:, :8], g['r%d_psi' % r][:, :8])) < 1e-7


def _oracle_embedding(D, k, tune, prefsigma, device=None):
    from oracle.dm_embedding import dm_embedding
    lamb, psi, sigma, mu = dm_embedding(np.asarray(D), k=k, tune=tune, seed=None, full=True)
    return lamb, psi, sigma, mu, np.zeros(3), np.zeros(3), np.zeros(4), 1.0


def test_op_files_match_reference(tmp_path, monkeypatch):
    """The drop-in op on the reference's dist pickle: same posPath, psi-pickle keys, progress
    marker and eigenvalue file as the reference's op (rad 3 on the 160-image PD: 4 embeddings)."""
    from manifoldem_python_gb300 import manifoldTrimmingAuto, myio, p
    g = _case('trim_nlsa32')
    monkeypatch.setattr(manifoldTrimmingAuto.DMembeddingII, 'op', _oracle_embedding)
    monkeypatch.setattr(p, 'psi_prog', str(tmp_path / 'progress'), raising=False)
    os.makedirs(p.psi_prog)
    dist_file = str(tmp_path / 'IMGs_prD_7')
    psi_file = str(tmp_path / 'psi_prD_7')
    eig_file = str(tmp_path / 'eig_spec.txt')
    myio.fout1(dist_file, ['D', 'ind'], [g['D'], g['ind']])
    with open(eig_file, 'w') as f:
        f.write('stale\n')
    np.random.seed(int(g['seed']))
    manifoldTrimmingAuto.op([dist_file, psi_file, eig_file, 7], 0, 3, float(g['rads'][0]),
                            False, dict(outputFile='', Is=True))
    with open(psi_file, 'rb') as f:
        out = pickle.load(f)
    assert list(out) == ['lamb', 'psi', 'sigma', 'mu', 'posPath', 'ind', 'logEps', 'logSumWij',
                         'popt', 'R_squared']
    np.testing.assert_array_equal(out['posPath'], g['r0_posPath'])
    np.testing.assert_array_equal(out['ind'], g['ind'])
    assert os.listdir(p.psi_prog) == ['7']
    with open(eig_file) as f:
        assert f.read() == str(g['r0_eig_txt'])


def test_psi_path_and_subset_posPath(monkeypatch):
    """get_psiPath's strict radius, and a caller-given posPath subset (manifoldTrimmingAuto.py:48-50:
    only posPath == 0 means all points; the kept indices are returned in the full numbering)."""
    from manifoldem_python_gb300 import manifoldTrimmingAuto
    from oracle.trimming import trim
    psi = np.array([[3.0, 4.0, 0.0, 9.0], [0.0, 0.0, 4.99, 0.0], [1.0, 1.0, 1.0, 0.0]])
    np.testing.assert_array_equal(manifoldTrimmingAuto.get_psiPath(psi, 5, 0), [1, 2])
    np.testing.assert_array_equal(manifoldTrimmingAuto.get_psiPath(psi, 4.99, 1), [2])
    monkeypatch.setattr(manifoldTrimmingAuto.DMembeddingII, 'op', _oracle_embedding)
    D = _case('trim_nlsa32')['D']
    sub = np.arange(1, 160, 2)
    np.random.seed(4)
    res, kept = manifoldTrimmingAuto.trim(D, sub, 3, 2.5)
    lamb, psi, sigma, mu, keep, runs = trim(D[sub][:, sub], 3, 2.5, seed=4)
    print('subset of 80: %d embeddings, kept %d' % (runs, len(keep)))
    assert runs > 1
    np.testing.assert_array_equal(kept, sub[keep])
    np.testing.assert_allclose(res[0], lamb, rtol=0, atol=1e-12)   # ARPACK's own start vector
