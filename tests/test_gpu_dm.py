"""The GPU diffusion-map embedding (manifoldem_python_gb300.DMembeddingII.op, csrc/dmap.cu)
against the reference's own DMembeddingII.op outputs (golden fixtures made by running the
reference, tests/golden/make_golden.py) and against the FP64 restatement in oracle/.

Tolerances: the bandwidth sweep evaluates exp in float32, so log sum_ij W_ij(eps) agrees to
1e-6 absolute; sigma to 1e-5 relative; eigenvalues to 1e-6 absolute; the top-8 diffusion
coordinates span the same subspace to 1e-4 rad.
"""
import numpy as np
import pytest
from scipy.linalg import subspace_angles

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _gpu_dm(D, k=None, seed=0):
    from manifoldem_python_gb300 import DMembeddingII
    np.random.seed(seed)
    return DMembeddingII.op(np.array(D, copy=True), D.shape[0] if k is None else k, 3, 60000)


def test_dm_matches_reference_golden(cuda_ready):
    """config1 (300 images, 70 px): the reference's DMembeddingII.op on the reference's D."""
    g = load_golden('config1')
    lamb, psi, sigma, mu, log_eps, log_sum, popt, r2 = _gpu_dm(g['ref_D'])
    print('sigma %.6g vs %.6g' % (sigma, float(g['ref_dm_sigma'])))
    assert abs(sigma - float(g['ref_dm_sigma'])) / sigma < 1e-5
    assert np.abs(lamb - g['ref_dm_lambda']).max() < 1e-6
    ang = float(np.max(subspace_angles(psi[:, :8], g['ref_dm_psi8'])))
    print('top-8 subspace angle vs reference %.3g rad' % ang)
    assert ang < 1e-4
    assert psi.shape == (300, 15) and mu.shape == (300,) and len(log_sum) == len(log_eps)
    assert abs(mu.sum() - 1.0) < 1e-9 and 0.9 < r2 <= 1.0


def _sym_distances(n, seed, dup=0):
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, 6)) * np.linspace(1, 0.2, 6)
    if dup:
        X[:dup] = X[dup:2 * dup] + 1e-5 * rng.standard_normal((dup, 6))
    D = ((X[:, None, :] - X[None, :, :]) ** 2).sum(-1)
    np.fill_diagonal(D, 0)
    return D


@pytest.mark.parametrize('n,k', [(120, None), (120, 40), (257, None)])
def test_dm_matches_oracle(cuda_ready, n, k):
    """Full and k-nearest neighbourhoods, with near-duplicate points (zero-distance edges),
    against the FP64 restatement of DMembeddingII / fergusonE / slaplacianonFly."""
    from oracle.dm_embedding import dm_embedding, ferguson, neighbour_lists
    D = _sym_distances(n, seed=n + (k or 0), dup=5)
    kk = n if k is None else k
    lamb, psi, sigma, mu, log_eps, log_sum, popt, r2 = _gpu_dm(D, kk, seed=3)
    lam_o, psi_o, sigma_o = dm_embedding(D, k=kk, seed=3)
    print('n=%d k=%d sigma %.8g vs %.8g' % (n, kk, sigma, sigma_o))
    assert abs(sigma - sigma_o) / sigma_o < 1e-5
    assert np.abs(lamb - lam_o).max() < 1e-6
    assert float(np.max(subspace_angles(psi[:, :8], psi_o[:, :8]))) < 1e-4
