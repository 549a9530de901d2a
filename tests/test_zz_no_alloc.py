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


class _Case:
    """One PD: the plan path's spectra and D (the expected result), and the arguments of a
    no-allocation call on them."""

    def __init__(self, torch, N, n, precision, seed):
        from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
        cfg, ds = _case(N, n, seed=seed)
        params = StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                             AmpContrast=cfg.ampc, precision=precision)
        ind = ds.CG[0]
        ref = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])],
                                        ds.stack.to('cuda'), ds.nStot, outputs=('D', 'spectrum'),
                                        to_host=False)[0]
        self.torch, self.n = torch, n
        self.cp = params.to_c()
        self.spectra = ref['spectrum'].contiguous()
        self.df = torch.from_numpy(np.ascontiguousarray(ds.df[ind], dtype=np.float64)).cuda()
        self.D_ref = ref['D'].cpu().numpy()

    def call(self, lib):
        """One no-allocation call into a NaN-filled D; returns (status, D on the host)."""
        torch, n = self.torch, self.n
        stream = torch.cuda.current_stream()
        D = torch.full((n * n,), float('nan'), dtype=torch.float64, device='cuda')
        st = lib.mem_pd_distances_noalloc(ctypes.byref(self.cp), n, self.spectra.data_ptr(),
                                          self.df.data_ptr(), D.data_ptr(),
                                          ctypes.c_void_p(stream.cuda_stream))
        status = lib.mem_noalloc_status(ctypes.c_void_p(stream.cuda_stream)) if st == 0 else st
        torch.cuda.synchronize()
        return status, D.cpu().numpy().reshape(n, n)

    def check(self, lib, what):
        from manifoldem_python_gb300 import _lib
        st, Dn = self.call(lib)
        assert st == 0, (what, _lib.status_string(st))
        err = np.abs(Dn - self.D_ref).max() / np.abs(self.D_ref).max()
        assert err < 1e-6, (what, err)
        np.testing.assert_array_equal(Dn, Dn.T)


@pytest.mark.parametrize('N,n,precision', [(64, 100, 'fp32'), (128, 120, 'fp32'),
                                           (128, 187, 'bf16x3')])
def test_noalloc_matches_plan_path_twice(cuda_ready, N, n, precision):
    from manifoldem_python_gb300 import _lib
    case = _Case(cuda_ready, N, n, precision, seed=31 + N)
    lib = _lib.load()
    for call in range(2):
        case.check(lib, call)


def test_noalloc_sequence_of_different_calls(cuda_ready):
    """Calls that change the box size, the image count and the contraction form one after the
    other on one device: each must match the plan path, whatever the previous call left in the
    shared array (padding rows, feature-layout tables, sums, status)."""
    from manifoldem_python_gb300 import _lib
    lib = _lib.load()
    cases = [_Case(cuda_ready, 128, 187, 'bf16x3', seed=41),
             _Case(cuda_ready, 64, 100, 'fp32', seed=42),
             _Case(cuda_ready, 128, 120, 'bf16x3', seed=43),
             _Case(cuda_ready, 70, 300, 'bf16x3', seed=44)]
    for i, c in enumerate(cases + cases[:1]):
        c.check(lib, i)


def test_noalloc_reports_an_expired_wait(cuda_ready, monkeypatch):
    """A bounded wait of the split-BF16 contraction that runs out is reported by
    mem_noalloc_status (the producer is told to withhold one chunk, so the wait for it can only
    end by a short limit); the next call with the default settings is correct again."""
    from manifoldem_python_gb300 import _lib
    lib = _lib.load()
    case = _Case(cuda_ready, 128, 150, 'bf16x3', seed=45)
    monkeypatch.setenv('MEM_WAIT_CYCLES', '200000')
    monkeypatch.setenv('MEM_TEST_WITHHOLD_CHUNK', '5')
    st, _ = case.call(lib)
    assert st == _lib.MEM_ERR_DEVICE_TIMEOUT, _lib.status_string(st)
    monkeypatch.delenv('MEM_WAIT_CYCLES')
    monkeypatch.delenv('MEM_TEST_WITHHOLD_CHUNK')
    case.check(lib, 'after the timeout')


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
