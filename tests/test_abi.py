"""The C-ABI library: it builds, loads, exports every function include/*.h declares, plans
without a GPU and rejects bad arguments with the documented status codes (no compute calls)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import REPO
from manifoldem_python_gb300 import _lib
from manifoldem_python_gb300.pipeline import StageParams


@pytest.fixture(scope='module')
def lib():
    _lib.build()
    return _lib.load()


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(REPO, 'include', '*.h')):
        txt = re.sub(r'/\*.*?\*/', '', open(h).read(), flags=re.S)
        names.update(re.findall(r'\b(mem_\w+)\s*\(', txt))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert 'mem_plan_execute' in names and 'mem_pd_batch' in names
    for n in names:
        assert hasattr(lib, n), n
    assert set(names) <= set(_lib.SIGNATURES) | {n for n in names if hasattr(lib, n)}


def test_struct_layouts_match_header():
    assert ctypes.sizeof(_lib.MemParams) == 72
    assert ctypes.sizeof(_lib.MemInputs) == 64
    assert ctypes.sizeof(_lib.MemOutputs) == 72


def _plan(lib, params, counts, psi):
    counts = np.ascontiguousarray(counts, dtype=np.int32)
    psi = np.ascontiguousarray(psi, dtype=np.float64)
    h = ctypes.c_void_p()
    st = lib.mem_plan_create(ctypes.byref(params), len(counts), counts.ctypes.data,
                             psi.ctypes.data, ctypes.byref(h))
    return st, h


def test_plan_tables_without_gpu(lib):
    P = StageParams(N=64, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1).to_c()
    st, h = _plan(lib, P, [300, 129, 1], [10.0, 20.0, 30.0])
    assert st == 0
    try:
        assert lib.mem_plan_num_images(h) == 430
        assert lib.mem_plan_num_pairs(h) == 300 * 299 // 2 + 129 * 128 // 2
        assert lib.mem_plan_d_elements(h) == 300 ** 2 + 129 ** 2 + 1
        sz = ctypes.c_size_t()
        assert lib.mem_plan_workspace_size(h, ctypes.byref(sz)) == 0 and sz.value > 0
        # the workspace holds at least the image, spectrum and feature buffers; a feature row is
        # [U' | V' | r' | s']: one U', V' column per ring of equal |k|^2, one r', s' column per
        # half-plane frequency, each block padded to 64
        pad = lambda x: -(-x // 64) * 64
        ka = np.arange(64)[:, None]
        kb = np.arange(33)[None, :]
        rings = len(np.unique(np.minimum(ka, 64 - ka) ** 2 + kb ** 2))
        Kf = 2 * pad(rings) + 2 * pad(64 * 33)
        assert (rings, Kf) == (457, 5248)
        from manifoldem_python_gb300.pipeline import feature_columns
        assert feature_columns(64) == Kf         # the batch-admission estimate's layout
        assert sz.value >= 430 * 64 * 64 * 4 + 430 * 64 * 33 * 8 + (384 + 256 + 128) * Kf * 4
        small = ctypes.c_size_t(sz.value - 1)
        assert lib.mem_plan_upload(h, ctypes.c_void_p(256), small, None) == _lib.MEM_ERR_WORKSPACE
    finally:
        lib.mem_plan_destroy(h)


def test_invalid_arguments(lib):
    P = StageParams(N=64, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1).to_c()
    assert _plan(lib, P, [0], [1.0])[0] == _lib.MEM_ERR_INVALID
    assert _plan(lib, P, [5], [float('nan')])[0] == _lib.MEM_ERR_INVALID
    big = StageParams(N=520, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1).to_c()
    assert _plan(lib, big, [5], [1.0])[0] == _lib.MEM_ERR_UNSUPPORTED
    bad = StageParams(N=64, pix_size=-1.0, Cs=2.7, EkV=300.0, AmpContrast=0.1).to_c()
    assert _plan(lib, bad, [5], [1.0])[0] == _lib.MEM_ERR_INVALID
    assert lib.mem_plan_execute(None, None, None, None, 0, None) == _lib.MEM_ERR_INVALID
    assert lib.mem_status_string(_lib.MEM_ERR_WORKSPACE) == b'workspace too small'


def test_contraction_schedule_table_is_validated(lib):
    """mem_plan_set_contraction: increasing max_n, persistent 0/1, 2 or 4 accumulators, and
    only before the upload (no GPU needed)."""
    P = StageParams(N=64, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1,
                    precision='bf16x3').to_c()
    st, h = _plan(lib, P, [300, 129, 1, 900], [10.0, 20.0, 30.0, 40.0])
    assert st == 0
    C = _lib.MemContractionConfig
    try:
        good = (C * 3)(C(200, 0, 2, 0, 0, 0), C(640, 1, 4, 128, 256, 0),
                       C(2 ** 31 - 1, 1, 2, 256, 128, 0))
        assert lib.mem_plan_set_contraction(h, 3, good) == _lib.MEM_OK
        for bad in ((C * 2)(C(640, 1, 2, 0), C(200, 1, 2, 0)),      # not increasing
                    (C * 2)(C(200, 2, 2, 0), C(640, 1, 2, 0)),      # persistent not 0/1
                    (C * 2)(C(200, 1, 3, 0), C(640, 1, 2, 0)),      # 3 accumulators
                    (C * 2)(C(200, 1, 2, 64), C(640, 1, 2, 0)),     # 64-wide tiles
                    (C * 2)(C(200, 1, 4, 256), C(640, 1, 2, 0)),    # 4 x 256 TMEM columns
                    (C * 2)(C(200, 1, 2, 128, 192), C(640, 1, 2, 0)),   # 192-row tiles
                    (C * 2)(C(200, 1, 2, 256, 256), C(640, 1, 2, 0))):  # 256 x 256
            assert lib.mem_plan_set_contraction(h, 2, bad) == _lib.MEM_ERR_INVALID
        assert lib.mem_plan_set_contraction(h, 0, good) == _lib.MEM_ERR_INVALID
        assert lib.mem_plan_set_wait_limit(h, 999) == _lib.MEM_ERR_INVALID
        assert lib.mem_plan_set_wait_limit(h, 10 ** 6) == _lib.MEM_OK
    finally:
        lib.mem_plan_destroy(h)
