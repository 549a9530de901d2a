"""The GPU CTF (``ctf`` output: the exact 64-bit fixed-point phase and the octant polynomial sine
of csrc/prologue.cu) against the FP64 restatement of ``ctemh_cryoFrank.op``
(modules/ctemh_cryoFrank.py:24-44) in oracle/, element by element, over defoci of 0.3-6 um and
box sizes with the shared-memory FFT (64, 128 px) and without (70, 192 px).

Tolerance: 2e-7 absolute without an envelope (the values lie in [-sqrt(1 + A^2),
sqrt(1 + A^2)]; the sine is within 9.2e-8 of sin(2 pi u / 2^64) over 4 million random phases,
times sqrt(1 + A^2), plus the rounding of the float product and output, half an ulp of 1;
measured 1.3e-7); 4e-7 absolute with a Gaussian envelope (expf; measured 2.0e-7).
The sign of every element with |CTF| > 1e-6 matches the oracle's.
"""
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('N,env', [(128, np.inf), (64, np.inf), (70, np.inf), (192, np.inf),
                                   (128, 0.3)])
def test_ctf_matches_fp64(cuda_ready, N, env):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    from oracle import distance_oracle as O
    n = 48
    cfg = dataclasses.replace(CONFIGS['config1'], name='ctf%d' % N, N=N, n_pd=1, n_fixed=n,
                              seed=700 + N)
    ds = make_dataset(cfg, device='cuda')
    ind = ds.CG[0].astype(np.int64)
    df = np.random.default_rng(N).uniform(3e3, 6e4, size=n)       # 0.3 - 6 um in Angstrom
    params = StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                         gaussEnv=env)
    res = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=df)], ds.stack, ds.nStot,
                                    outputs=('ctf',))[0]
    ctf = np.asarray(res['ctf'], dtype=np.float64).reshape(n, N, N)
    Q = O.create_grid(N)
    ref = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * cfg.pix), cfg.cs, d, cfg.kv, env,
                                                      cfg.ampc)) for d in df])
    err = np.abs(ctf - ref).max()
    print('N=%d env=%s: max |CTF - FP64| %.3g' % (N, env, err))
    assert err < (2e-7 if np.isinf(env) else 4e-7)
    big = np.abs(ref) > 1e-6
    np.testing.assert_array_equal(np.sign(ctf[big]), np.sign(ref[big]))
