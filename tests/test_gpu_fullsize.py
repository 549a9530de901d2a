"""The distance stage at the workload sizes (one PD each): 2000 images of 128 px (config 2),
4000 images of 192 px (config 3) and 6000 images of 250 px (the largest PD and box of config 5).
The FP64 oracle cannot run these in seconds, so the checks are size-independent properties:

* D exactly symmetric with a zero diagonal, finite, and non-negative up to rounding
  (-1e-6 of max D);
* sample rows of D against an FP64 contraction of the GPU's own half-plane spectra with exact
  FP64 CTFs (D_ij = sum_k w(k) |C_j(k) F_i(k) - C_i(k) F_j(k)|^2): 1e-6 of max D for the
  split-BF16 form (the benchmarked precision target), 2e-6 for the FP32 form;
* the Wiener and phase-flipped averages finite, and imgAllIntensity non-negative.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, N, n, seed, precision):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config1'], name='full%d' % N, N=N, n_pd=1, n_fixed=n,
                              seed=seed)
    ds = make_dataset(cfg, device='cuda')
    ind = ds.CG[0].astype(np.int64)
    params = StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                         precision=precision)
    res = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack,
                                    ds.nStot, outputs=('D', 'spectrum', 'img_avg',
                                                       'img_avg_flip', 'img_all_intensity'))[0]
    return cfg, ds.df[ind], res


def _fp64_rows(cfg, df, spec, rows):
    from oracle import distance_oracle as O
    N = cfg.N
    Nh = N // 2 + 1
    F = spec[..., 0].astype(np.float64) + 1j * spec[..., 1].astype(np.float64)
    F = F.reshape(len(df), N, Nh)
    Q = O.create_grid(N)
    w = O.half_plane_weights(N)
    C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * cfg.pix), cfg.cs, d, cfg.kv, np.inf,
                                                    cfg.ampc))[:, :Nh] for d in df])
    out = []
    for i in rows:
        row = np.empty(len(df))
        for j0 in range(0, len(df), 512):
            j = slice(j0, min(len(df), j0 + 512))
            diff = C[j] * F[i][None] - C[i][None] * F[j]
            row[j] = np.sum(w[None] * (diff.real ** 2 + diff.imag ** 2), axis=(1, 2))
        row[i] = 0.0
        out.append(row)
    return np.stack(out)


@pytest.mark.parametrize('N,n,precision', [(128, 2000, 'bf16x3'), (192, 4000, 'bf16x3'),
                                           (250, 6000, 'bf16x3'), (128, 2000, 'fp32')])
def test_full_size_pd(cuda_ready, N, n, precision):
    torch = cuda_ready
    cfg, df, res = _run(torch, N, n, seed=300 + N, precision=precision)
    D = np.asarray(res['D'])
    assert D.shape == (n, n) and np.all(np.isfinite(D))
    np.testing.assert_array_equal(D, D.T)
    assert np.all(np.diag(D) == 0)
    scale = np.abs(D).max()
    assert D.min() >= -1e-6 * scale
    rows = np.random.default_rng(n).choice(n, 6, replace=False)
    ref = _fp64_rows(cfg, df, np.asarray(res['spectrum']), rows)
    err = np.abs(D[rows] - ref).max() / np.abs(ref).max()
    print('N=%d n=%d %s: sample rows vs FP64 contraction %.3g' % (N, n, precision, err))
    assert err < (1e-6 if precision == 'bf16x3' else 2e-6)
    for k in ('img_avg', 'img_avg_flip', 'img_all_intensity'):
        assert np.all(np.isfinite(np.asarray(res[k]))), k
    assert np.asarray(res['img_all_intensity']).min() >= 0
