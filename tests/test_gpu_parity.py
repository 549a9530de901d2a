"""GPU parity of the distance stage (through the C ABI) against the reference's outputs and the
FP64 oracle.

Tolerances (max |difference| / max |reference| over the array):
* D, plain FP32 form: 1e-5 against the reference's float64 D;
* D against an FP64 contraction of the GPU's own spectra and CTFs (isolates the contraction):
  1e-6 for both the FP32 and the split-BF16 forms;
* imgAll, imgAllFlip, CTF, imgAvg, imgAvgFlip, imgAllIntensity: 2e-5 (float32 pipeline).
"""
import os
import pickle
import tempfile

import numpy as np
import pytest

from conftest import (GOLDEN_CASES, golden_mask_volume, golden_micro, golden_options,
                      golden_ref, golden_shifts, load_golden)

pytestmark = pytest.mark.gpu

PRECISIONS = ['fp32', 'bf16x3']
TOL_IMG = 2e-5


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / max(np.abs(b).max(), 1e-300))


def run_case(torch, g, precision, outputs=None):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    mic = golden_micro(g)
    params = StageParams(avg_only=bool(g['avgOnly']), precision=precision, **mic)
    stage = DistanceStage(params)
    job = PdJob(ind=g['ind'], q=g['q'], df=g['df'])
    stack = torch.from_numpy(g['stack16'].astype(np.float32)).cuda()
    outs = outputs or ('D', 'img_avg', 'img_avg_flip', 'img_all_intensity', 'img_all',
                       'img_all_flip', 'ctf', 'spectrum')
    from manifoldem_python_gb300.pipeline import VolumeMask
    vol = golden_mask_volume(g)
    mask = VolumeMask(vol) if vol is not None else None
    return stage.run([job], stack, int(g['nStot']), outputs=outs, sh=golden_shifts(g),
                     mask=mask)[0]


@pytest.mark.parametrize('precision', PRECISIONS)
@pytest.mark.parametrize('case', GOLDEN_CASES)
def test_stage_matches_reference(cuda_ready, case, precision):
    torch = cuda_ready
    g = load_golden(case)
    res = run_case(torch, g, precision)
    N = int(g['N'])
    n = g['ind'].shape[0]
    pairs = {'imgAll': 'img_all', 'imgAllFlip': 'img_all_flip', 'imgAvg': 'img_avg',
             'imgAvgFlip': 'img_avg_flip', 'imgAllIntensity': 'img_all_intensity'}
    for rk, mk in pairs.items():
        ref, sl = golden_ref(g, rk)
        mine = res[mk] if sl is None else res[mk][sl]
        assert rel(mine, ref) < TOL_IMG, (case, rk, rel(mine, ref))
    ref_ctf, sl = golden_ref(g, 'CTF')
    mine_ctf = res['ctf'] if sl is None else res['ctf'][sl]
    assert rel(mine_ctf.reshape(ref_ctf.shape), ref_ctf) < TOL_IMG
    if bool(g['avgOnly']):
        assert 'D' not in res
        return
    D = res['D']
    if golden_mask_volume(g) is not None:       # projectMask on the GPU, exact
        np.testing.assert_array_equal(res['msk2'], g['ref_msk2'])
    Dref = g['ref_D']
    assert rel(D, Dref) < 1e-5, (case, rel(D, Dref))
    np.testing.assert_array_equal(D, D.T)
    assert np.all(np.diag(D) == 0)
    # the contraction alone: FP64 D of the GPU's own half-plane spectra and exact CTFs
    from oracle import distance_oracle as O
    F = res['spectrum'][..., 0].astype(np.float64) + 1j * res['spectrum'][..., 1]
    Q = O.create_grid(N)
    C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * float(g['pix_size'])),
                                                    float(g['Cs']), d, float(g['EkV']),
                                                    float(g['gaussEnv']),
                                                    float(g['AmpContrast'])))[:, :N // 2 + 1]
                  for d in g['df']])
    D64 = O.distances_from_half_plane(C, F, N)
    np.fill_diagonal(D64, 0)
    tol = {'fp32': 1e-6, 'bf16x3': 1e-6}[precision]
    assert rel(D, D64) < tol, (case, rel(D, D64))
    assert n == D.shape[0]
    if 'ref_dm_psi8' in g:
        # downstream: top-8 diffusion-map coordinates of the GPU D vs the reference's
        from scipy.linalg import subspace_angles
        from oracle.dm_embedding import dm_embedding
        _, psi, _ = dm_embedding(D, seed=0)
        ang = float(np.max(subspace_angles(psi[:, :8], g['ref_dm_psi8'])))
        print('%s %s: D rel %.3g (vs FP64 contraction %.3g), DM top-8 angle %.3g rad'
              % (case, precision, rel(D, Dref), rel(D, D64), ang))
        assert ang < 1e-4, ang


def test_batched_equals_single(cuda_ready):
    """Two PDs in one call give the results of two separate calls."""
    torch = cuda_ready
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    g = load_golden('config1')
    stage = DistanceStage(StageParams(**golden_micro(g)))
    stack = torch.from_numpy(g['stack16'].astype(np.float32)).cuda()
    ind = g['ind']
    jobs = [PdJob(ind=ind[:170], q=g['q'][:, :170], df=g['df'][:170]),
            PdJob(ind=ind[170:], q=g['q'][:, 170:], df=g['df'][170:])]
    both = stage.run(jobs, stack, int(g['nStot']))
    for j, r in zip(jobs, both):
        single = stage.run([j], stack, int(g['nStot']))[0]
        for k in single:
            assert rel(r[k], single[k]) < 1e-6, k


def test_dropin_op_writes_reference_pickle(cuda_ready):
    """op() writes the reference's 19-key pickle (same dtypes/shapes) and the resume marker."""
    from manifoldem_python_gb300 import p as mp
    from manifoldem_python_gb300.getDistanceCTF_local_Conj9combinedS2 import op
    g = load_golden('even32_conj')
    mic = golden_micro(g)
    with tempfile.TemporaryDirectory() as tmp:
        stack_file = os.path.join(tmp, 'stack.bin')
        g['stack16'].astype(np.float32).tofile(stack_file)
        mp.init()
        mp.nPix, mp.pix_size, mp.Cs, mp.EkV = mic['N'], mic['pix_size'], mic['Cs'], mic['EkV']
        mp.AmpContrast, mp.gaussEnv = mic['AmpContrast'], mic['gaussEnv']
        mp.dist_prog = os.path.join(tmp, 'progress')
        os.makedirs(mp.dist_prog)
        out_file = os.path.join(tmp, 'IMGs_prD_3')
        options = golden_options(g)
        op([g['ind'], g['q'], g['df'], out_file, 3], dict(type='Butter', Qc=0.5, N=8),
           stack_file, None, int(g['nStot']), options)
        assert os.path.exists(os.path.join(mp.dist_prog, '3'))
        with open(out_file, 'rb') as f:
            d = pickle.load(f)
    n, N = g['ind'].shape[0], int(g['N'])
    expect = {'D': (n, n), 'CTF': (n, N * N), 'imgAll': (n, N, N), 'imgAllFlip': (n, N, N),
              'PD': (3,), 'PDs': (3, n), 'Psis': (n, 1), 'imgAvg': (N, N),
              'imgAvgFlip': (N, N), 'imgLabels': (n,), 'Dnom': (n, 1), 'Nom': (n, 1),
              'imgAllIntensity': (N, N)}
    assert len(d) == 19 and d['msk2'] == 1 and d['version'] == str(g['ref_version'])
    for k, shp in expect.items():
        assert np.shape(d[k]) == shp, k
        if k != 'imgLabels':
            assert np.asarray(d[k]).dtype == np.float64, k
    np.testing.assert_array_equal(d['imgLabels'], g['ref_imgLabels'])
    assert rel(d['D'], g['ref_D']) < 1e-5
    assert d['options'] == options


@pytest.mark.parametrize('N', [64, 96, 128, 192, 250, 300, 512])
def test_box_sizes_match_oracle(cuda_ready, N):
    """Box sizes with their own kernels, against the FP64 oracle on a small PD with conjugate
    views: 64 and 128 px (shared-memory FFTs, compile-time-size rotation), 96 and the 192 px
    workload size (cuFFT, whole-image rotation with a per-angle row stride), 250 and 300 px
    (banded rotation; 300 px with a short last prefilter segment) and 512 px, the largest box
    (per-frequency U', V' features: its half plane exceeds the ring-feature buffer)."""
    torch = cuda_ready
    import dataclasses
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    from oracle import distance_oracle as O
    cfg = dataclasses.replace(CONFIGS['config1'], N=N, n_fixed=8 if N < 512 else 5,
                              conj_pd_frac=1.0, seed=60 + N)
    ds = make_dataset(cfg, device='cpu')
    ind = ds.CG[0]
    mic = dict(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    ref = O.pd_op(ind, ds.q[:, ind], ds.df[ind], ds.stack.numpy(), ds.nStot, **mic)
    for precision in PRECISIONS:
        res = DistanceStage(StageParams(precision=precision, **mic)).run(
            [PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack.cuda(), ds.nStot)[0]
        assert rel(res['img_all'], ref['imgAll']) < TOL_IMG
        assert rel(res['img_all_flip'], ref['imgAllFlip']) < TOL_IMG
        assert rel(res['img_avg'], ref['imgAvg']) < TOL_IMG
        assert rel(res['D'], ref['D']) < 1e-5


@pytest.mark.parametrize('dma,shuffle', [('off', False), ('auto', False), ('auto', True)])
def test_streamed_stage_matches_plain(cuda_ready, dma, shuffle):
    """StreamedStage (stack in pinned host memory, PD groups on load / compute / copy streams)
    against one plain execute with the stack on the device: every group read by the load
    kernel (dma off, mem_plan_execute_split), every group staged by the copy engines (the
    synthetic stack is in PD order), and a stack in shuffled order whose groups have more runs
    than the limit (load kernel) or fewer (staged)."""
    torch = cuda_ready
    import dataclasses
    from manifoldem_python_gb300.geometry import pd_geometry
    from manifoldem_python_gb300.pipeline import (DistanceStage, PdJob, StageParams,
                                                  StreamedStage, split_outputs)
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    for N in (48, 64):
        cfg = dataclasses.replace(CONFIGS['config4'], N=N, n_pd=7, n_median=60, n_min=1,
                                  n_max=150, seed=70 + N)
        ds = make_dataset(cfg, device='cpu')
        params = StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                             precision='bf16x3')
        jobs = [PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind]) for ind in ds.CG]
        names = ('D', 'img_avg', 'img_avg_flip', 'img_all_intensity')
        ref = DistanceStage(params).run(jobs, ds.stack.cuda(), ds.nStot, outputs=names)
        geoms = [pd_geometry(np.asarray(j.ind), j.q, ds.nStot) for j in jobs]
        counts = [len(j.ind) for j in jobs]
        st = StreamedStage(params, counts, [g.psi_p for g in geoms], n_groups=3, outputs=names,
                           dma=dma, max_runs=64 if not shuffle else 40)
        sidx = np.concatenate([g.stack_index for g in geoms])
        stack_h = ds.stack.contiguous().pin_memory()
        if shuffle:
            # the same images in a permuted stack, each entry pointed at its image's new place
            num = ds.stack.shape[0]
            perm = np.random.default_rng(N).permutation(num)
            inv = np.empty_like(perm)
            inv[perm] = np.arange(num)
            stack_h = ds.stack[torch.from_numpy(perm)].contiguous().pin_memory()
            sidx = inv[sidx]
        st.set_metadata(sidx,
                        np.concatenate([g.flip for g in geoms]),
                        np.concatenate([g.psi_rad for g in geoms]),
                        np.concatenate([np.asarray(j.df, np.float64) for j in jobs]))
        if dma == 'off':
            assert st.staged_groups() == 0
        elif not shuffle:
            assert st.staged_groups() == len(st.groups)
        for _ in range(2):                      # two runs in a row reuse every buffer
            host = st.run(stack_h)
        st.device_status()
        got = []
        for gi, (g, plan) in enumerate(zip(st.groups, st.plans)):
            got += split_outputs(plan, [counts[i] for i in g], host[gi], to_host=True)
        assert len(got) == len(ref)
        for a, b in zip(got, ref):
            for k in names:
                np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]))


def _ellipsoid_mask(N):
    """A binary mask volume: an off-centre ellipsoid (float32, (N, N, N), z y x)."""
    z, y, x = np.meshgrid(*(np.arange(N, dtype=np.float64),) * 3, indexing='ij')
    c = 0.5 * N
    r = ((x - c - 2.) / (0.36 * N)) ** 2 + ((y - c + 1.) / (0.30 * N)) ** 2 + \
        ((z - c) / (0.26 * N)) ** 2
    return (r < 1).astype(np.float32)


@pytest.mark.parametrize('N,branch', [(64, 'relion'), (128, 'relion'), (64, 'mask'),
                                      (128, 'mask')])
def test_relion_and_mask_box_sizes(cuda_ready, N, branch):
    """The RELION read (order-3 'wrap' shift of the stored image) and the volume mask
    (projectMask) at the shared-memory FFT sizes, against the FP64 oracle on a PD with conjugate
    views (the golden fixtures pin both at 32 px against the reference itself)."""
    torch = cuda_ready
    import dataclasses
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams, VolumeMask
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    from oracle import distance_oracle as O
    cfg = dataclasses.replace(CONFIGS['config1'], N=N, n_fixed=12, conj_pd_frac=1.0,
                              seed=80 + N + (0 if branch == 'relion' else 1))
    ds = make_dataset(cfg, device='cpu')
    ind = ds.CG[0]
    mic = dict(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    stack = ds.stack.numpy()
    sh = vol = None
    if branch == 'relion':
        rng = np.random.default_rng(N)
        sh = (rng.uniform(-2.5, 2.5, stack.shape[0]), rng.uniform(-2.5, 2.5, stack.shape[0]))
    else:
        vol = _ellipsoid_mask(N)
    ref = O.pd_op(ind, ds.q[:, ind], ds.df[ind], stack, ds.nStot, sh=sh, mask_volume=vol, **mic)
    for precision in PRECISIONS:
        mask = VolumeMask(vol) if vol is not None else None
        res = DistanceStage(StageParams(precision=precision, **mic)).run(
            [PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack.cuda(), ds.nStot,
            sh=sh, mask=mask)[0]
        if vol is not None:
            np.testing.assert_array_equal(np.asarray(res['msk2']).reshape(N, N),
                                          np.asarray(ref['msk2']).reshape(N, N))
        for mk, rk in (('img_all', 'imgAll'), ('img_all_flip', 'imgAllFlip'),
                       ('img_avg', 'imgAvg'), ('img_avg_flip', 'imgAvgFlip')):
            assert rel(res[mk], ref[rk]) < TOL_IMG, (branch, N, mk, rel(res[mk], ref[rk]))
        assert rel(res['D'], ref['D']) < 1e-5, (branch, N, rel(res['D'], ref['D']))
