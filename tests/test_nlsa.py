"""NLSA stage, CPU side: the oracle (oracle/nlsa_oracle.py) against the reference's own NLSA.op
outputs (tests/golden/nlsa32.npz, made by tests/golden/make_golden.py), and the product's
vectorised curve fit (manifoldem_python_gb300/fit_1D_open_manifold_3D.py) against the reference
and the oracle's per-point loop.  The three runs: Wiener branch with msk2 = 1, Wiener branch with
a 2D mask, unfiltered 'cuti' branch."""
import numpy as np
import pytest

from conftest import NLSA_RUNS, load_golden, nlsa_errors, nlsa_golden_args, nlsa_golden_ref


@pytest.fixture(scope='module')
def nlsa_golden():
    return load_golden('nlsa32')


@pytest.mark.parametrize('tag', sorted(NLSA_RUNS))
def test_oracle_matches_reference(nlsa_golden, tag):
    from oracle.nlsa_oracle import nlsa
    g = nlsa_golden
    np.random.seed(int(g['seed']))
    out = nlsa(*nlsa_golden_args(g, tag))
    e = nlsa_errors(out, nlsa_golden_ref(g, tag))
    print(tag, NLSA_RUNS[tag], {k: '%.2e' % v for k, v in e.items()})
    assert e['IMGT'] < 1e-6                 # the fixture stores IMGT as float32
    assert e['sdiag'] < 1e-9 and e['Topo'] < 1e-8 and e['VX'] < 1e-7
    assert e['psiC1'] < 1e-7 and e['psirec'] < 1e-6 and e['psirec8'] < 1e-6
    assert e['mu'] < 1e-10 and e['tau'] < 1e-8


def test_con_distances_order():
    """ConD is the band sum in the reference's order: bit-equal to adding the shifted blocks."""
    from oracle.nlsa_oracle import con_distances
    rng = np.random.default_rng(1)
    DD = rng.standard_normal((40, 40)) * 1e3
    ConD = con_distances(DD, 5)
    ref = np.zeros((35, 35))
    for i in range(5):
        ref += DD[i:i + 35, i:i + 35]
    assert np.array_equal(ConD, ref)


@pytest.mark.parametrize('tag', sorted(NLSA_RUNS))
def test_fit_matches_reference(nlsa_golden, tag):
    """The vectorised fit on the reference's psirec gives the reference's tau bit for bit."""
    from manifoldem_python_gb300 import fit_1D_open_manifold_3D as fit
    g = nlsa_golden
    a, b, tau = fit.op(g[tag + '_psirec'])
    assert tau.shape == g[tag + '_tau'].shape
    assert np.array_equal(tau, g[tag + '_tau'])


@pytest.mark.parametrize('n,seed', [(300, 0), (1200, 1), (64, 2)])
def test_fit_matches_oracle_loop(n, seed):
    """Vectorised root finding and candidate choice against the per-point np.roots loop, on noisy
    curves of the model's shape and on a degenerate case (a_3 = 0: np.roots strips the leading
    zeros)."""
    from manifoldem_python_gb300 import fit_1D_open_manifold_3D as fit
    from oracle.nlsa_oracle import fit_1d_open_manifold_3d
    rng = np.random.default_rng(seed)
    t = np.sort(rng.uniform(0, 1, n))
    psi = np.stack([np.cos(np.pi * t), 0.7 * np.cos(2 * np.pi * t), 0.4 * np.cos(3 * np.pi * t)],
                   1) + 0.05 * rng.standard_normal((n, 3))
    a, b, tau = fit.op(psi)
    ao, bo, tauo = fit_1d_open_manifold_3d(psi.copy())
    assert np.array_equal(tau, tauo) and np.array_equal(a, ao) and np.array_equal(b, bo)
    x = psi[:, :3]
    a0 = np.array([0.9, -0.3, 0.0])
    b0 = np.array([0.01, 0.02, 0.0])
    from oracle.nlsa_oracle import _solve_tau_p
    ref = np.array([_solve_tau_p(x[p], a0, b0) for p in range(n)]).reshape(n, 1)
    assert np.array_equal(fit.solve_tau(x, a0, b0), ref)
