"""Host-side logic of the GetDistancesS2 replacement: resume markers, job list, pickle format,
HBM admission."""
import os
import pickle
import tempfile

import numpy as np

from manifoldem_python_gb300 import GetDistancesS2 as G
from manifoldem_python_gb300 import myio
from manifoldem_python_gb300 import p as mp
from manifoldem_python_gb300.pipeline import StageParams, admit_batches


def _setup(tmp):
    mp.init()
    mp.user_dir, mp.proj_name = tmp, 'unit'
    mp.create_dir()


def test_divide_skips_finished_pds_and_keeps_reference_job_shape():
    with tempfile.TemporaryDirectory() as tmp:
        _setup(tmp)
        CG = [np.array([0, 5]), np.array([1, 2, 3]), np.array([4])]
        q = np.arange(4 * 6, dtype=float).reshape(4, 6)
        df = np.arange(6, dtype=float) * 100
        open(os.path.join(mp.dist_prog, '1'), 'a').close()        # PD 1 finished
        open(os.path.join(mp.dist_prog, '.hidden'), 'a').close()  # ignored
        jobs = G.divide(CG, q, df, 3)
        assert [j[4] for j in jobs] == [0, 2]
        ind, q1, df1, out, prD = jobs[0]
        np.testing.assert_array_equal(q1, q[:, [0, 5]])
        np.testing.assert_array_equal(df1, df[[0, 5]])
        assert out == '{}prD_{}'.format(mp.dist_file, 0)
        assert G.fileCheck() == [1] and G.count(3) == 2


def test_myio_format_and_corrupt_file():
    with tempfile.TemporaryDirectory() as tmp:
        f = os.path.join(tmp, 'x')
        myio.fout1(f, ['a', 'b'], [1, np.zeros(3)])
        with open(f, 'rb') as fh:
            d = pickle.load(fh)
        assert set(d) == {'a', 'b'}
        with open(f, 'wb') as fh:
            fh.write(b'not a pickle')
        assert myio.fin1(f) is None


def test_admission_splits_by_budget_in_order():
    params = StageParams(N=128, pix_size=2.0, Cs=2.7, EkV=300.0, AmpContrast=0.1)
    counts = [400] * 10 + [3000]
    b = admit_batches(counts, params, budget_bytes=int(1e9))
    assert [i for bb in b for i in bb] == list(range(len(counts)))
    assert len(b) > 1 and b[-1] == [10]
    assert admit_batches(counts, params, budget_bytes=int(1e15)) == [list(range(11))]


def test_params_module_prefers_loaded_reference_p():
    import sys
    import types
    from manifoldem_python_gb300.p import params_module
    fake = types.ModuleType('p')
    fake.nPix = 64
    sys.modules['p'] = fake
    try:
        assert params_module() is fake
    finally:
        del sys.modules['p']
    assert params_module() is mp


def test_balanced_groups_cover_pds_in_order():
    """StreamedStage's PD groups: consecutive, non-empty, covering every PD once, image counts
    close to equal."""
    import numpy as np
    from manifoldem_python_gb300.pipeline import balanced_groups
    rng = np.random.default_rng(3)
    for n_pd, n_groups in ((800, 4), (5, 3), (1, 4), (8, 8), (37, 6)):
        counts = rng.integers(1, 900, n_pd)
        groups = balanced_groups(counts, n_groups)
        assert len(groups) == min(n_groups, n_pd)
        assert [i for g in groups for i in g] == list(range(n_pd))
        assert all(len(g) > 0 for g in groups)
        if n_pd >= 100:
            sizes = [int(counts[list(g)].sum()) for g in groups]
            assert max(sizes) - min(sizes) <= 2 * counts.max()
    # ramped: the first groups grow by the ramp factor, the rest are equal
    counts = rng.integers(100, 900, 800)
    groups = balanced_groups(counts, 8, ramp=1.5, ramp_steps=3)
    assert [i for g in groups for i in g] == list(range(800))
    sizes = np.array([int(counts[list(g)].sum()) for g in groups], dtype=float)
    w = np.array([1, 1.5, 2.25, 3.375, 3.375, 3.375, 3.375, 3.375])
    assert np.abs(sizes / sizes.sum() - w / w.sum()).max() < 2 * counts.max() / sizes.sum()


def test_async_writer_writes_pickles_then_markers(tmp_path):
    """myio.AsyncWriter: every queued pickle is complete and readable with the reference's
    format, each marker exists only with its pickle, and a bound on queued bytes does not
    deadlock a single oversized item."""
    import numpy as np
    from manifoldem_python_gb300 import myio
    keys = ['D', 'imgAll', 'ind']
    with myio.AsyncWriter(workers=3, max_pending_bytes=1 << 20) as w:
        for i in range(12):
            vals = [np.full((50, 50), float(i)), np.zeros((4, 300, 300), np.float32) + i,
                    np.arange(i)]
            w.submit(str(tmp_path / ('pd_%d.pkl' % i)), keys, vals,
                     marker=str(tmp_path / ('%d' % i)))
    for i in range(12):
        d = myio.fin1(str(tmp_path / ('pd_%d.pkl' % i)))
        assert set(d) == set(keys) and float(d['D'][3, 4]) == i
        assert d['imgAll'].dtype == np.float32 and (tmp_path / ('%d' % i)).exists()


def test_async_writer_reraises(tmp_path):
    import numpy as np
    import pytest
    from manifoldem_python_gb300 import myio
    w = myio.AsyncWriter(workers=2)
    w.submit(str(tmp_path / 'missing_dir' / 'x.pkl'), ['a'], [np.zeros(3)])
    with pytest.raises(FileNotFoundError):
        w.close()


def test_mrc_round_trip(tmp_path):
    """The MRC stack reader/writer used for RELION stacks: header fields, orientation (data is
    (nz, ny, nx) as stored), and an extended header skipped by its declared length."""
    import numpy as np
    from manifoldem_python_gb300 import mrc
    data = np.random.default_rng(0).standard_normal((3, 5, 4)).astype(np.float32)
    path = str(tmp_path / 'a.mrcs')
    mrc.write_stack(path, data)
    h = mrc.read_header(path)
    assert (h['nx'], h['ny'], h['nz'], h['mode']) == (4, 5, 3, 2)
    np.testing.assert_array_equal(np.asarray(mrc.read_stack(path)), data)
    raw = bytearray(open(path, 'rb').read())
    ext = 2048
    raw[92:96] = np.int32(ext).tobytes()
    raw = raw[:1024] + bytes(ext) + raw[1024:]
    path2 = str(tmp_path / 'b.mrcs')
    open(path2, 'wb').write(bytes(raw))
    np.testing.assert_array_equal(np.asarray(mrc.read_stack(path2)), data)


def test_stack_runs_split_and_remap():
    """Runs of consecutive stack indices for the copy-engine staging of a streamed group, and
    each entry's position in the staged copy (duplicates, any order)."""
    from manifoldem_python_gb300.pipeline import stack_runs
    si = np.array([5, 6, 7, 7, 20, 21, 9, 6])
    runs, remap = stack_runs(si, 8)
    assert runs == [(5, 3, 0), (9, 1, 3), (20, 2, 4)]
    staged = np.concatenate([np.arange(f, f + c) for f, c, _ in runs])
    np.testing.assert_array_equal(staged[remap], si)
    assert stack_runs(si, 2) is None
    runs, remap = stack_runs(np.arange(100)[::-1], 1)
    assert runs == [(0, 100, 0)]
    np.testing.assert_array_equal(remap, np.arange(100)[::-1])
    runs, remap = stack_runs(np.array([], dtype=np.int64), 1)
    assert runs == [] and remap.size == 0


def test_bench_reads_profile_figures():
    """The figures bench.py takes from the committed ncu summaries: the rotation's DRAM traffic
    per full config4 launch and its shared-memory wavefronts per image (config4 and config5),
    and the contraction's traffic."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location('bench_module', os.path.join(here, 'bench.py'))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.traffic_from_profiles('rotate', 'config4') == 4.82e10
    assert bench.profile_number('rotate', 'config4', 'shared_wavefronts_per_image') == 36790
    assert bench.profile_number('rotate', 'config5', 'shared_wavefronts_per_image') == 149825
    assert bench.traffic_from_profiles('contraction_bf16x3', 'config4') == 3.11e10
    assert bench.profile_number('rotate', 'config3', 'shared_wavefronts_per_image') is None
