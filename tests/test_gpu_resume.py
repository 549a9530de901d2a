"""End-to-end resume of the GetDistancesS2 replacement on the GPU.

A project of 8 PDs (32 px, conjugate views in some PDs) where PDs 1 and 4 finished before (pickle
and marker) and PD 6 crashed in the middle of its pickle write (a corrupt pickle, no marker).
``GetDistancesS2.op`` with a small device budget must admit the six pending PDs in at least
three batches, recompute exactly those (PD 6 included, its pickle replaced), leave the finished
PDs' files untouched, and write pickles equal to what the per-PD drop-in ``op`` writes for each
PD alone.  Reference: GetDistancesS2.py:29-35 and :94 (markers, job list), myio.py:21-30 (a
corrupt pickle reads as None), getDistanceCTF_local_Conj9combinedS2.py:409-419 (pickle, then
marker).
"""
import dataclasses
import os
import pickle
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DONE_BEFORE = (1, 4)
CORRUPT = 6


def _project(tmp, ds):
    from manifoldem_python_gb300 import myio
    from manifoldem_python_gb300 import p as mp
    mp.init()
    mp.user_dir, mp.proj_name = tmp, 'resume'
    mp.create_dir()
    cfg = ds.cfg
    mp.img_stack_file = os.path.join(tmp, 'stack.bin')
    ds.stack.numpy().astype(np.float32).tofile(mp.img_stack_file)
    mp.num_part, mp.numberofJobs, mp.relion_data = ds.num_part, len(ds.CG), False
    mp.nPix, mp.pix_size, mp.Cs, mp.EkV, mp.AmpContrast = cfg.N, cfg.pix, cfg.cs, cfg.kv, cfg.ampc
    myio.fout2(mp.tess_file, dict(CG=ds.CG, q=ds.q, df=ds.df, sh=ds.sh))
    return mp


def _load(path):
    with open(path, 'rb') as f:
        return pickle.load(f)


def test_resume_recomputes_exactly_the_missing_pds(cuda_ready, tmp_path, monkeypatch, capsys):
    from manifoldem_python_gb300 import GetDistancesS2 as G
    from manifoldem_python_gb300.getDistanceCTF_local_Conj9combinedS2 import (OUTPUT_KEYS,
                                                                            op as pd_op,
                                                                            stage_params)
    from manifoldem_python_gb300.pipeline import admit_batches
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config4'], N=32, n_pd=8, n_median=40, n_min=20,
                              n_max=90, conj_pd_frac=0.4, seed=77)
    ds = make_dataset(cfg, device='cpu')
    monkeypatch.chdir(tmp_path)
    mp = _project(str(tmp_path), ds)
    options = dict(verbose=False, avgOnly=False, visual=False, parallel=False,
                   relion_data=False, thres=mp.PDsizeThH)
    # expected: each PD alone through the per-PD drop-in
    exp_dir = tmp_path / 'expected'
    exp_dir.mkdir()
    prog = mp.dist_prog
    for prD, ind in enumerate(ds.CG):
        pd_op([ind, ds.q[:, ind], ds.df[ind], str(exp_dir / ('prD_%d' % prD)), prD],
              G.FILTER_PAR, mp.img_stack_file, ds.sh, ds.nStot, options)
    for f in os.listdir(prog):
        os.remove(os.path.join(prog, f))
    # the state left by an interrupted run
    for prD in DONE_BEFORE:
        shutil.copy(exp_dir / ('prD_%d' % prD), '{}prD_{}'.format(mp.dist_file, prD))
        open(os.path.join(prog, str(prD)), 'a').close()
    corrupt = '{}prD_{}'.format(mp.dist_file, CORRUPT)
    with open(corrupt, 'wb') as f:
        f.write(pickle.dumps({'D': np.zeros(3)})[:20])
    before = {p: open('{}prD_{}'.format(mp.dist_file, p), 'rb').read() for p in DONE_BEFORE}
    # a device budget that splits the pending PDs into at least three batches
    pending = [p for p in range(len(ds.CG)) if p not in DONE_BEFORE]
    counts = [len(ds.CG[p]) for p in pending]
    params = stage_params(mp, G.FILTER_PAR, options)
    budget = None
    for b in np.geomspace(1e5, 1e9, 400):
        if len(admit_batches(counts, params, int(b))) <= 3:
            budget = int(b)
            break
    assert budget is not None and len(admit_batches(counts, params, budget)) >= 3
    mp.gpu_budget_bytes = budget
    ran = []
    real_run_batch = G._run_batch

    def spy(stage, params, jobs, batch, *a, **k):
        ran.append([jobs[i][4] for i in batch])
        return real_run_batch(stage, params, jobs, batch, *a, **k)
    monkeypatch.setattr(G, '_run_batch', spy)
    G.op()
    assert 'Processing %d projection directions.' % len(pending) in capsys.readouterr().out
    assert len(ran) >= 3 and sorted(p for b in ran for p in b) == pending
    assert sorted(int(f) for f in os.listdir(prog)) == list(range(len(ds.CG)))
    for p in DONE_BEFORE:
        assert open('{}prD_{}'.format(mp.dist_file, p), 'rb').read() == before[p]
    for prD in range(len(ds.CG)):
        got = _load('{}prD_{}'.format(mp.dist_file, prD))
        exp = _load(exp_dir / ('prD_%d' % prD))
        assert list(got) == OUTPUT_KEYS
        for k in OUTPUT_KEYS:
            a, b = got[k], exp[k]
            if isinstance(b, np.ndarray) and b.dtype.kind == 'f':
                assert a.dtype == b.dtype and a.shape == b.shape, k
                scale = max(float(np.abs(b).max()), 1e-300)
                assert float(np.abs(a - b).max()) / scale < 1e-6, (prD, k)
            elif isinstance(b, np.ndarray):
                np.testing.assert_array_equal(a, b)
            else:
                assert a == b, (prD, k)
