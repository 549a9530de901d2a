"""Precision gate of the split-BF16 form end to end: D of the whole GPU stage (float32 image
pipeline, 3-term split-BF16 contraction with FP32 accumulation, FP64 epilogue) against the FP64
oracle's D on the same inputs (not against an FP64 contraction of the GPU's own spectra).

Tolerance: max |D - D_oracle| / max |D_oracle| <= 1e-6 (the split-BF16 target of the
distance stage).  The oracle equals the reference's own op() to 1e-12 on the golden cases
(tests/test_oracle.py), so for those the reference's stored D is the comparison.

Cases: the 300-image 70 px golden case (config1), the 48 px golden case with near-duplicate
particles, and a synthetic 300-image PD of 128 px (the box size of the batched workload) with the
oracle run here.  Near-duplicate pairs are also checked elementwise, scaled by the pair's
cross-norm term S_ij (|dD_ij| / S_ij <= 1e-6), which is the error the GEMM form can promise for
a pair whose distance cancels.
"""
import dataclasses

import numpy as np
import pytest

from conftest import golden_micro, load_golden

pytestmark = pytest.mark.gpu

TOL_D = 1e-6


def rel(a, b):
    return float(np.abs(np.asarray(a, dtype=np.float64) - b).max() / np.abs(b).max())


def gpu_D(torch, stack, ind, q, df, nStot, mic, precision='bf16x3', outputs=('D',)):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    stage = DistanceStage(StageParams(precision=precision, **mic))
    st = torch.from_numpy(np.ascontiguousarray(stack, dtype=np.float32)).cuda()
    return stage.run([PdJob(ind=ind, q=q, df=df)], st, int(nStot), outputs=outputs)[0]


def cross_norm(res, mic, df):
    """S_ij = sum_k w (C_j^2 |F_i|^2 + C_i^2 |F_j|^2) over the half plane (FP64, from the GPU's
    spectra and exact CTFs): the scale below which D_ij cancels in the GEMM form."""
    from oracle import distance_oracle as O
    N = mic['N']
    F = res['spectrum'][..., 0].astype(np.float64) + 1j * res['spectrum'][..., 1]
    Q = O.create_grid(N)
    C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * mic['pix_size']), mic['Cs'], d,
                                                    mic['EkV'], mic.get('gaussEnv', np.inf),
                                                    mic['AmpContrast']))[:, :N // 2 + 1]
                  for d in df])
    w = O.half_plane_weights(N)
    a = (w * np.abs(F) ** 2).reshape(len(df), -1)
    c2 = (C ** 2).reshape(len(df), -1)
    A = a @ c2.T                     # A[i, j] = sum_k w |F_i|^2 C_j^2
    return A + A.T


@pytest.mark.parametrize('case', ['config1', 'even48_neardup'])
def test_split_bf16_D_vs_fp64_golden(cuda_ready, case):
    torch = cuda_ready
    g = load_golden(case)
    mic = golden_micro(g)
    res = gpu_D(torch, g['stack16'], g['ind'], g['q'], g['df'], g['nStot'], mic,
                outputs=('D', 'spectrum'))
    D = res['D']
    ref = g['ref_D'].copy()
    np.fill_diagonal(ref, 0)
    err = rel(D, ref)
    print('%s: split-BF16 D vs the reference / FP64 D: %.3g' % (case, err))
    assert err <= TOL_D, (case, err)
    if case == 'even48_neardup':
        S = cross_norm(res, mic, g['df'])
        off = ~np.eye(D.shape[0], dtype=bool)
        scaled = float((np.abs(D - ref)[off] / S[off]).max())
        print('%s: max |dD_ij| / S_ij = %.3g' % (case, scaled))
        assert scaled <= TOL_D, scaled


def test_split_bf16_D_vs_fp64_oracle_128px(cuda_ready):
    """A 300-image PD of 128 px against the FP64 oracle run here (a few seconds on the CPU)."""
    torch = cuda_ready
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    from oracle import distance_oracle as O
    cfg = dataclasses.replace(CONFIGS['config2'], n_fixed=300, seed=21, conj_pd_frac=1.0)
    ds = make_dataset(cfg, device='cpu')
    stack = ds.stack.numpy().astype(np.float32)
    ind = ds.CG[0]
    q, df = ds.q[:, ind], ds.df[ind]
    mic = dict(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    ref = O.pd_op(ind, q, df, stack, ds.nStot, **mic)['D']
    np.fill_diagonal(ref, 0)
    for precision, tol in (('bf16x3', TOL_D), ('fp32', 1e-5)):
        D = gpu_D(torch, stack, ind, q, df, ds.nStot, mic, precision=precision)['D']
        err = rel(D, ref)
        print('128 px, 300 images, %s: D vs FP64 oracle %.3g' % (precision, err))
        assert err <= tol, (precision, err)
