"""The FP64 oracle against the reference's own outputs (golden fixtures) and unit KATs."""
import numpy as np
import pytest
from scipy import ndimage

from conftest import (GOLDEN_CASES, golden_mask_volume, golden_micro, golden_options,
                      golden_ref, golden_shifts, load_golden)
from oracle import distance_oracle as O

KEYS = ['D', 'CTF', 'imgAll', 'imgAllFlip', 'PD', 'PDs', 'Psis', 'imgAvg', 'imgAvgFlip',
        'imgLabels', 'Dnom', 'Nom', 'imgAllIntensity']


@pytest.fixture(scope='module', params=GOLDEN_CASES)
def oracle_run(request):
    g = load_golden(request.param)
    res = O.pd_op(g['ind'], g['q'], g['df'], g['stack16'].astype(np.float32), int(g['nStot']),
                  options=golden_options(g), sh=golden_shifts(g),
                  mask_volume=golden_mask_volume(g), **golden_micro(g))
    return request.param, g, res


def test_oracle_matches_reference(oracle_run):
    case, g, res = oracle_run
    for k in KEYS:
        ref, sl = golden_ref(g, k)
        mine = np.asarray(res[k])
        if sl is not None:
            mine = mine[sl]
        assert mine.shape == ref.shape, (case, k)
        if k in ('imgLabels', 'PD', 'PDs', 'Psis', 'Nom', 'Dnom'):
            np.testing.assert_array_equal(mine, ref, err_msg='%s %s' % (case, k))
        else:
            den = max(np.abs(ref).max(), 1e-300)
            assert np.abs(mine - ref).max() / den < 1e-12, (case, k)
    assert tuple(g['ref_CTF_shape']) == np.shape(res['CTF'])
    assert str(g['ref_version']) == res['version']
    np.testing.assert_array_equal(np.asarray(res['msk2']), g['ref_msk2'])


def test_rotation_is_periodic_bspline():
    """rotatefill (3x3 tile + scipy rotate order 3, rotatefill.py:21-25) equals the periodic
    cubic B-spline rotation the oracle and the GPU kernel evaluate.  The tile is one period
    away from its edges, where scipy's prefilter boundary differs from periodic; that difference
    decays as |sqrt(3)-2|^N (7e-10 at N=16, below 1e-18 from N=32 on)."""
    rng = np.random.default_rng(0)
    z1 = 2 - np.sqrt(3)
    for N in (16, 32, 33, 64):
        img = rng.normal(size=(N, N))
        tol = max(1e-12, 20 * z1 ** N)
        for ang in (0.0, 17.3, -123.9, 90.0, 271.5):
            tiled = ndimage.rotate(np.tile(img, (3, 3)), ang, reshape=False)[N:2 * N, N:2 * N]
            out = O.rotate_periodic(img, ang)
            assert np.abs(out - tiled).max() / np.abs(tiled).max() < tol, (N, ang)


def test_annular_mask_centre():
    m = O.annular_mask(0, 4.0, 8, 8)
    # centre (N/2 - 1, M/2) = (3, 4), radius 4 (strict)
    assert m[3, 4] == 1 and m[3, 0] == 0 and m[3, 1] == 1 and m[7, 4] == 0 and m[0, 4] == 1


def test_ctf_no_envelope_and_phase():
    k = np.linspace(0, 0.25, 50)
    c = O.ctf_cryo_frank(k, 2.7, 15000.0, 300.0, np.inf, 0.1)
    assert abs(c[0] + 0.1) < 1e-15                      # sin 0 - A cos 0
    lam = 12.3986 / np.sqrt((2 * 511.0 + 300.0) * 300.0)
    wr = (0.5 * np.pi * 2.7e7 * lam ** 3 * k ** 2 - np.pi * lam * 15000.0) * k ** 2
    alt = np.sqrt(1.01) * np.sin(wr - np.arctan(0.1))
    assert np.abs(c - alt).max() < 1e-12


def test_half_plane_distances_equal_full_plane():
    rng = np.random.default_rng(1)
    for N in (8, 9):
        n = 5
        imgs = rng.normal(size=(n, N, N))
        F = np.fft.fft2(imgs)
        Q = O.create_grid(N)
        C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / 4.0, 2.7, df, 300., np.inf, 0.1))
                      for df in rng.uniform(1e4, 3e4, n)])
        Dfull = O.distances_fp64(C.reshape(n, -1), F.reshape(n, -1))
        Dhalf = O.distances_from_half_plane(C[:, :, :N // 2 + 1], np.fft.rfft2(imgs), N)
        assert np.abs(Dfull - Dhalf).max() / np.abs(Dfull).max() < 1e-12
        Ddir = O.distances_direct(C.reshape(n, -1), F.reshape(n, -1))
        assert np.abs(Dfull - Ddir).max() / np.abs(Dfull).max() < 1e-12


def test_centred_decomposition_is_exact():
    """D_ij = a_i + a_j + E_ij with centred features (the form both GPU contractions use)."""
    rng = np.random.default_rng(2)
    N, n = 10, 7
    F = np.fft.rfft2(rng.normal(size=(n, N, N)))
    C = rng.normal(size=(n, N, N // 2 + 1))
    w = O.half_plane_weights(N)[None, None, :]
    u = (np.sqrt(w) * np.abs(F) ** 2).reshape(n, -1)
    v = (np.sqrt(w) * C ** 2).reshape(n, -1)
    r = (np.sqrt(2 * w) * C * F.real).reshape(n, -1)
    s = (np.sqrt(2 * w) * C * F.imag).reshape(n, -1)
    mu = [x.mean(0) + rng.normal(size=x.shape[1]) for x in (u, v, r, s)]   # any centring works
    a = (mu[0] * v + mu[1] * u - mu[0] * mu[1] - mu[2] * r + mu[2] ** 2 / 2
         - mu[3] * s + mu[3] ** 2 / 2).sum(1)
    up, vp, rp, sp = (x - m for x, m in zip((u, v, r, s), mu))
    E = up @ vp.T + vp @ up.T - rp @ rp.T - sp @ sp.T
    D = a[:, None] + a[None, :] + E
    Dref = O.distances_from_half_plane(C, F, N)
    assert np.abs(D - Dref).max() / np.abs(Dref).max() < 1e-12


@pytest.mark.parametrize('case', ['config1', 'even48_neardup'])
def test_dm_embedding_matches_reference(case):
    """The diffusion-map restatement against the reference's DMembeddingII on the reference D."""
    from scipy.linalg import subspace_angles
    from oracle.dm_embedding import dm_embedding
    g = load_golden(case)
    lam, psi, sigma = dm_embedding(g['ref_D'], seed=0)
    assert abs(sigma - float(g['ref_dm_sigma'])) / sigma < 1e-8
    assert np.abs(lam - g['ref_dm_lambda']).max() < 1e-9
    assert np.max(subspace_angles(psi[:, :8], g['ref_dm_psi8'])) < 1e-8
