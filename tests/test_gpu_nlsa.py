"""GPU NLSA stage (manifoldem_python_gb300.NLSA, csrc/nlsa.cu) against the reference's own NLSA.op
outputs (tests/golden/nlsa32.npz) and against the float64 oracle (oracle/nlsa_oracle.py).

Tolerances.  ConD: bit-exact.  Snapshot matrix A (float32 spectra and banded sums, float64
Wiener denominators): 1e-5 of max |A|.  Whole stage, after sign alignment of eigenvector-derived
arrays: IMGT (unit-variance frames) 1e-5 absolute; sdiag 1e-5 relative; Topo_mean and VX 1e-4 of
their largest value; psiC1 and psirec, first three columns, 1e-4; top-8 psirec subspace 1e-4 rad;
mu 1e-6; tau 1e-4.
"""
import numpy as np
import pytest

from conftest import (NLSA_RUNS, load_golden, nlsa_errors, nlsa_golden_args, nlsa_golden_ref)

pytestmark = pytest.mark.gpu

TOL = dict(IMGT=1e-5, sdiag=1e-5, Topo=1e-4, VX=1e-4, psiC1=1e-4, psirec=1e-4, psirec8=1e-4,
           mu=1e-6, tau=1e-4)


def check(e, tol=TOL):
    bad = {k: v for k, v in e.items() if not v <= tol[k]}
    assert not bad, bad


def even_ctfs(n, N, seed):
    """CTF-like arrays even in frequency on the ifftshifted grid: sin of a defocus-dependent
    quadratic in |k|^2 (exactly C(-k) = C(k))."""
    rng = np.random.default_rng(seed)
    f = np.fft.fftfreq(N)
    k2 = f[:, None] ** 2 + f[None, :] ** 2
    df = rng.uniform(20, 60, n)
    return np.sin(-np.pi * df[:, None, None] * k2[None] + 0.3 * k2[None] ** 2 * 400 - 0.1)


@pytest.mark.parametrize('num,c', [(300, 6), (1000, 20), (37, 1)])
def test_con_distances_bit_exact(cuda_ready, num, c):
    torch = cuda_ready
    from manifoldem_python_gb300 import NLSA
    from oracle.nlsa_oracle import con_distances
    rng = np.random.default_rng(num)
    DD = rng.standard_normal((num, num)) ** 2 * 1e4
    g = NLSA._Gpu(None)
    d = torch.from_numpy(DD).cuda()
    out = torch.empty((num - c, num - c), dtype=torch.float64, device='cuda')
    g.call('mem_nlsa_con_distances', d.data_ptr(), num, c, out.data_ptr())
    assert np.array_equal(out.cpu().numpy(), con_distances(DD, c))


@pytest.mark.parametrize('N,num,c,branch', [
    (32, 90, 3, 'prD'), (64, 120, 4, 'prD'), (128, 40, 2, 'prD'),      # shared-memory FFT
    (48, 70, 3, 'prD'), (33, 60, 2, 'prD'),                             # cuFFT
    (64, 120, 4, 'prD-mask'), (48, 70, 5, 'cuti'), (33, 50, 3, 'cuti')])
def test_snapshots_match_oracle(cuda_ready, N, num, c, branch):
    """A of NLSA.py:63-86 against the reference's per-image loop (oracle), 8 modes plus a
    ninth to cover a second mode group."""
    torch = cuda_ready
    from manifoldem_python_gb300 import NLSA
    from oracle import nlsa_oracle as O
    rng = np.random.default_rng(N * 1000 + num)
    imgs = rng.standard_normal((num, N, N))
    ctf = even_ctfs(num, N, N)
    T = 9
    mu_psi = rng.standard_normal((num - c, T)) / num
    y, x = np.mgrid[0:N, 0:N]
    msk = (((x - N / 2) ** 2 + (y - N / 2 + 1) ** 2) < (0.4 * N) ** 2).astype(np.float64) \
        if branch == 'prD-mask' else np.array(1)
    wiener = branch != 'cuti'
    g = NLSA._Gpu(None)
    im_d = torch.from_numpy(imgs.astype(np.float32)).cuda()
    ctf_d = torch.from_numpy(ctf.astype(np.float32)).cuda() if wiener else None
    A = NLSA.snapshots(g, im_d, ctf_d, mu_psi, msk, c).cpu().numpy()
    imgs32 = imgs.astype(np.float32).astype(np.float64)
    ctf32 = ctf.astype(np.float32).astype(np.float64)
    wd = O.get_wiener(ctf32, c, num) if wiener else None
    ref = O.snapshot_matrix(imgs32, ctf32, wd, msk, mu_psi, c, num, wiener)
    err = np.abs(A - ref).max() / np.abs(ref).max()
    print(N, num, c, branch, 'A rel err %.2e' % err)
    assert err < 1e-5


@pytest.mark.parametrize('tag', sorted(NLSA_RUNS))
def test_nlsa_matches_reference_golden(cuda_ready, tag):
    """Whole NLSA.op on the reference's distance-stage outputs (32 px, 160 images, ConOrder 3)
    against the reference's NLSA.op run on the same inputs with the same seed."""
    from manifoldem_python_gb300 import NLSA
    g = load_golden('nlsa32')
    np.random.seed(int(g['seed']))
    out = NLSA.op(*nlsa_golden_args(g, tag))
    ref = nlsa_golden_ref(g, tag)
    assert [np.shape(a) for a in out] == [np.shape(a) for a in ref]
    e = nlsa_errors(out, ref)
    print(tag, NLSA_RUNS[tag], {k: '%.2e' % v for k, v in e.items()})
    check(e)


def _gpu_distance_outputs(torch, N, n, seed):
    """imgAll, CTF, D of one synthetic PD from the GPU distance stage."""
    import dataclasses
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config1'], name='nlsa%d' % N, N=N, n_pd=1, n_fixed=n,
                              seed=seed)
    ds = make_dataset(cfg, device='cpu')
    ind = ds.CG[0].astype(np.int64)
    params = StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                         gaussEnv=np.inf)
    res = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                    ds.stack.cuda(), ds.nStot,
                                    outputs=('D', 'img_all', 'ctf'))[0]
    return (np.asarray(res['img_all'], dtype=np.float64),
            np.asarray(res['ctf'], dtype=np.float64).reshape(n, N, N),
            np.asarray(res['D'], dtype=np.float64))


@pytest.mark.parametrize('N,n', [(64, 300), (70, 260)])
def test_nlsa_matches_oracle_on_stage_outputs(cuda_ready, N, n):
    """The distance stage's own outputs fed to NLSA.op (GPU) and to the oracle: 64 px (shared-
    memory FFT) and 70 px (cuFFT), ConOrder = floor(n / 50)."""
    torch = cuda_ready
    from manifoldem_python_gb300 import NLSA
    from oracle.dm_embedding import dm_embedding
    from oracle.nlsa_oracle import nlsa
    imgAll, CTF, D = _gpu_distance_outputs(torch, N, n, seed=200 + N)
    _, psi, _ = dm_embedding(D, seed=0)
    P = np.argsort(psi[:, 0])
    c = n // 50
    par = dict(num=n, ConOrder=c, k=n - c, tune=3, nS=n, save=False, psiTrunc=8)
    args = (par, D[P][:, P], np.arange(n), P, imgAll, np.array(1), CTF,
            dict(outDir='', prD=0))
    np.random.seed(9)
    out = NLSA.op(*args)
    np.random.seed(9)
    ref = nlsa(*args)
    e = nlsa_errors(out, ref)
    print(N, n, {k: '%.2e' % v for k, v in e.items()})
    check(e)


def test_odd_ctf_is_rejected(cuda_ready):
    from manifoldem_python_gb300 import NLSA
    g = load_golden('nlsa32')
    args = list(nlsa_golden_args(g, 'a'))
    ctf = args[6].copy()
    ctf[:, 1, 2] += 0.5                       # breaks C(-k) = C(k)
    args[6] = ctf
    with pytest.raises(ValueError):
        NLSA.op(*args)
