"""The split-BF16 tcgen05 contraction against the FP32 form and an FP64 contraction of the same
spectra.  Tolerance of the split form: max |D - D64| / max |D64| <= 1e-6, where D64 is the FP64
contraction of the GPU's own half-plane spectra and exact CTFs."""
import dataclasses
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dataset(N, n, near_dup=0.0, conj=0.0, seed=5):
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config1'], N=N, n_fixed=n, near_dup_frac=near_dup,
                              conj_pd_frac=conj, seed=seed)
    return cfg, make_dataset(cfg, device='cpu')


def _run(torch, cfg, ds, precision, env=None):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    old = {}
    for k, v in (env or {}).items():
        old[k] = os.environ.get(k)
        os.environ[k] = str(v)
    try:
        stage = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                          AmpContrast=cfg.ampc, precision=precision))
        ind = ds.CG[0]
        job = PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])
        return stage.run([job], ds.stack.to('cuda'), ds.nStot,
                         outputs=('D', 'spectrum', 'pair_norm'))[0]
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _d64(cfg, ds, res):
    from oracle import distance_oracle as O
    N = cfg.N
    F = res['spectrum'][..., 0].astype(np.float64) + 1j * res['spectrum'][..., 1]
    Q = O.create_grid(N)
    ind = ds.CG[0]
    C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * cfg.pix), cfg.cs, d, cfg.kv,
                                                    np.inf, cfg.ampc))[:, :N // 2 + 1]
                  for d in ds.df[ind]])
    D = O.distances_from_half_plane(C, F, N)
    np.fill_diagonal(D, 0)
    return D


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_tc_single_tile(cuda_ready):
    """One 128x128 tile (n=24, N=32): the smallest tcgen05 launch."""
    torch = cuda_ready
    cfg, ds = _dataset(32, 24, conj=1.0)
    r32 = _run(torch, cfg, ds, 'fp32')
    rtc = _run(torch, cfg, ds, 'bf16x3')
    r4 = _run(torch, cfg, ds, 'bf16x3', env={'MEM_TC_TERMS': 4})
    D64 = _d64(cfg, ds, r32)
    e32, etc, e4 = rel(r32['D'], D64), rel(rtc['D'], D64), rel(r4['D'], D64)
    print('single tile: fp32 %.3g  bf16x3 %.3g  bf16x4 %.3g' % (e32, etc, e4))
    np.testing.assert_array_equal(rtc['D'], rtc['D'].T)
    assert etc < 1e-6, etc
    assert e4 < 1e-6, e4


def test_tc_multi_tile_ragged(cuda_ready):
    """Several PDs with ragged sizes (tiles straddling n) in one call."""
    torch = cuda_ready
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    cfg = dataclasses.replace(__import__('manifoldem_python_gb300.synthetic', fromlist=['x'])
                              .CONFIGS['config4'], N=48, n_pd=5, n_median=150, n_min=1,
                              n_max=400, seed=21)
    from manifoldem_python_gb300.synthetic import make_dataset
    ds = make_dataset(cfg, device='cpu')
    jobs = [PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind]) for ind in ds.CG]
    res = {}
    for prec in ('fp32', 'bf16x3'):
        st = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                       AmpContrast=cfg.ampc, precision=prec))
        res[prec] = st.run(jobs, ds.stack.to('cuda'), ds.nStot, outputs=('D',))
    for a, b in zip(res['fp32'], res['bf16x3']):
        assert rel(b['D'], a['D']) < 2e-6


@pytest.mark.parametrize('terms', [3, 4])
@pytest.mark.parametrize('group,kahan', [(0, 0), (1, 0), (2, 0), (4, 0), (1, 1), (4, 1)])
def test_tc_accumulation_groups(cuda_ready, group, kahan, terms):
    """Near-duplicate images (cancellation) at 128 px: error of each accumulation setting."""
    torch = cuda_ready
    cfg, ds = _dataset(128, 384, near_dup=0.05, seed=9)
    rtc = _run(torch, cfg, ds, 'bf16x3', env={'MEM_TC_GROUP_CHUNKS': group, 'MEM_TC_KAHAN': kahan,
                                             'MEM_TC_TERMS': terms})
    D64 = _d64(cfg, ds, rtc)
    e = rel(rtc['D'], D64)
    nd = np.nonzero(ds.near_dup_of >= 0)[0]
    src = ds.near_dup_of[nd]
    pos = {int(v): i for i, v in enumerate(ds.CG[0])}
    pairs = [(pos[int(a)], pos[int(b)]) for a, b in zip(nd, src) if int(a) in pos and int(b) in pos]
    elem = max(abs(rtc['D'][i, j] - D64[i, j]) / D64[i, j] for i, j in pairs) if pairs else 0.0
    print('terms=%d group=%d kahan=%d: normwise %.3g, near-duplicate elementwise %.3g'
          % (terms, group, kahan, e, elem))
    if (group, kahan) == (1, 0):        # the default accumulation setting
        assert e < 1e-6


@pytest.mark.parametrize('N', [32, 64, 128])
def test_smem_fft_matches_cufft_path(cuda_ready, N):
    """The shared-memory FFT kernels (low-pass, spectrum, inverse) against the cuFFT path on the
    same inputs: every output of the stage."""
    torch = cuda_ready
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    cfg, ds = _dataset(N, 40, conj=0.5, seed=44 + N)
    names = ('D', 'img_all', 'img_all_flip', 'img_avg', 'img_avg_flip', 'img_all_intensity',
             'spectrum', 'ctf')
    outs = {}
    for smem in (0, 1):
        old = os.environ.get('MEM_SMEM_FFT')
        os.environ['MEM_SMEM_FFT'] = str(smem)
        try:
            st = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                           AmpContrast=cfg.ampc))
            ind = ds.CG[0]
            outs[smem] = st.run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                ds.stack.to('cuda'), ds.nStot, outputs=names)[0]
        finally:
            if old is None:
                os.environ.pop('MEM_SMEM_FFT', None)
            else:
                os.environ['MEM_SMEM_FFT'] = old
    for k in names:
        e = rel(np.asarray(outs[1][k]), np.asarray(outs[0][k]))
        print('N=%d %s: smem FFT vs cuFFT %.3g' % (N, k, e))
        assert e < 2e-6, (k, e)


@pytest.mark.parametrize('precision', ['fp32', 'bf16x3'])
@pytest.mark.parametrize('N', [64, 70, 128])
def test_ring_features_match_per_frequency(cuda_ready, N, precision):
    """Ring features (one U', V' column per ring of equal |k|^2) against per-frequency U', V'
    blocks (MEM_RING_FEATURES=0): the same D within the contraction's precision, and against an
    FP64 contraction of the GPU's spectra no worse than the per-frequency form."""
    torch = cuda_ready
    cfg, ds = _dataset(N, 150, near_dup=0.05, seed=90 + N)
    res = {}
    for ring in (0, 1):
        res[ring] = _run(torch, cfg, ds, precision, env={'MEM_RING_FEATURES': ring})
    e = rel(res[1]['D'], res[0]['D'])
    D64 = _d64(cfg, ds, res[1])
    e64 = rel(res[1]['D'], D64)
    e64_pf = rel(res[0]['D'], _d64(cfg, ds, res[0]))
    print('N=%d %s: ring vs per-frequency %.3g, vs FP64: ring %.3g, per-frequency %.3g'
          % (N, precision, e, e64, e64_pf))
    # no less accurate than the per-frequency layout (this PD has 5% near-duplicate images, so
    # both forms sit near 1e-6 of the FP64 contraction at 128 px)
    assert e < 2e-6 and e64 < max(1.25 * e64_pf, 1e-6)
    np.testing.assert_array_equal(res[1]['D'], res[1]['D'].T)


@pytest.mark.parametrize('N', [64, 128])
def test_fused_image_stage_matches_three_kernels(cuda_ready, N):
    """The fused per-image kernel (low-pass, both rotations and the spectrum in one CTA per
    image) against the three separate kernels on the same inputs: every output of the stage.
    The fused kernel runs the rotation with twice the samples per thread (prefilter segments of
    2x the length, start states truncated at a smaller power of the pole), so the outputs agree
    to rounding, not bit for bit."""
    torch = cuda_ready
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    cfg, ds = _dataset(N, 60, conj=0.5, seed=52 + N)
    names = ('D', 'img_all', 'img_all_flip', 'img_avg', 'img_avg_flip', 'img_all_intensity',
             'spectrum', 'ctf')
    outs = {}
    for fused in (0, 1):
        old = os.environ.get('MEM_FUSED_IMAGE')
        os.environ['MEM_FUSED_IMAGE'] = str(fused)
        try:
            st = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                           AmpContrast=cfg.ampc, precision='bf16x3'))
            ind = ds.CG[0]
            outs[fused] = st.run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                 ds.stack.to('cuda'), ds.nStot, outputs=names)[0]
        finally:
            if old is None:
                os.environ.pop('MEM_FUSED_IMAGE', None)
            else:
                os.environ['MEM_FUSED_IMAGE'] = old
    for k in names:
        e = rel(np.asarray(outs[1][k]), np.asarray(outs[0][k]))
        print('N=%d %s: fused vs three kernels %.3g' % (N, k, e))
        assert e < 1e-6, (k, e)


@pytest.mark.parametrize('N', [96, 230, 250, 300, 512])
def test_band_rotation_matches_whole_image_kernels(cuda_ready, N):
    """The banded rotation (coefficient image in bands of rows in shared memory, the column
    prefilter through global memory) against the whole-image kernels on the same inputs
    (MEM_ROT_BAND=0: the shared-memory kernel for N <= 236, the global-memory one above): imgAll
    and D agree to rounding (the two prefilters truncate their periodic start sums differently
    and filter the second rotation's axes in the other order)."""
    torch = cuda_ready
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    cfg, ds = _dataset(N, 12, conj=0.5, seed=70 + N)
    names = ('D', 'img_all', 'img_all_flip', 'img_avg')
    outs = {}
    for band, variant in ((0, 0), (2, 0), (2, 1), (2, 2), (2, 3)):
        old = {k: os.environ.get(k) for k in ('MEM_ROT_BAND', 'MEM_ROT_BAND_VARIANT')}
        os.environ['MEM_ROT_BAND'] = str(band)
        os.environ['MEM_ROT_BAND_VARIANT'] = str(variant)
        try:
            st = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                           AmpContrast=cfg.ampc, precision='bf16x3'))
            ind = ds.CG[0]
            outs[band, variant] = st.run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                         ds.stack.to('cuda'), ds.nStot, outputs=names)[0]
        finally:
            for k, v in old.items():
                if v is None:
                    os.environ.pop(k, None)
                else:
                    os.environ[k] = v
    for variant in (0, 1, 2, 3):
        for k in names:
            e = rel(np.asarray(outs[2, variant][k]), np.asarray(outs[0, 0][k]))
            print('N=%d variant %d %s: banded vs whole-image rotation %.3g' % (N, variant, k, e))
            assert e < 2e-6, (variant, k, e)
