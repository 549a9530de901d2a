"""The no-allocation entry point, mem_pd_distances_noalloc, through the C ABI.

Callers that cannot allocate device memory (a plugin inside a host application that owns all
device buffers, code called back from another runtime's memory pool, latency-critical paths)
get D for one PD from its spectra with every intermediate in a static device array.  Here it
must reproduce the D of the regular plan path on the same spectra, on two calls in a row (the
static scratch keeps the previous call's contents), and refuse sizes beyond its scratch.
This file is collected last so that a run stopping at the first failure has run the rest.
"""
import ctypes
import dataclasses

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(N, n, seed):
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config1'], N=N, n_fixed=n, conj_pd_frac=0.5, seed=seed)
    return cfg, make_dataset(cfg, device='cpu')


@pytest.mark.parametrize('N,n,precision', [(64, 100, 'fp32'), (128, 120, 'fp32'),
                                           (128, 187, 'bf16x3')])
def test_noalloc_matches_plan_path_twice(cuda_ready, N, n, precision):
    torch = cuda_ready
    from manifoldem_python_gb300 import _lib
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    cfg, ds = _case(N, n, seed=31 + N)
    params = StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                         precision=precision)
    ind = ds.CG[0]
    ref = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                    ds.stack.to('cuda'), ds.nStot, outputs=('D', 'spectrum'),
                                    to_host=False)[0]
    lib = _lib.load()
    cp = params.to_c()
    spectra = ref['spectrum'].contiguous()
    df = torch.from_numpy(np.ascontiguousarray(ds.df[ind], dtype=np.float64)).cuda()
    D_ref = ref['D'].cpu().numpy()
    stream = torch.cuda.current_stream()
    for call in range(2):
        D = torch.full((n * n,), float('nan'), dtype=torch.float64, device='cuda')
        st = lib.mem_pd_distances_noalloc(ctypes.byref(cp), n, spectra.data_ptr(), df.data_ptr(),
                                          D.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert st == 0, _lib.status_string(st)
        torch.cuda.synchronize()
        Dn = D.cpu().numpy().reshape(n, n)
        err = np.abs(Dn - D_ref).max() / np.abs(D_ref).max()
        assert err < 1e-6, (call, err)
        np.testing.assert_array_equal(Dn, Dn.T)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda_ready):
    torch = cuda_ready
    from manifoldem_python_gb300 import _lib
    from manifoldem_python_gb300.pipeline import StageParams
    lib = _lib.load()
    cp = StageParams(N=128, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1).to_c()
    dummy = torch.zeros(16, dtype=torch.float64, device='cuda')
    for n in (188, 2000):       # 187 images of 128 px are the most that fit
        st = lib.mem_pd_distances_noalloc(ctypes.byref(cp), n, dummy.data_ptr(),
                                          dummy.data_ptr(), dummy.data_ptr(), None)
        assert st == _lib.MEM_ERR_TOO_LARGE, n
    assert 'static scratch' in _lib.status_string(st)
