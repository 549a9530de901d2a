import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, 'tests', 'golden')
if REPO not in sys.path:
    sys.path.insert(0, REPO)

GOLDEN_CASES = ['even32_conj', 'odd33_env', 'even32_avgonly', 'even48_neardup', 'config1',
                'relion32', 'volmask32']


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (sm_103) and the built library')


def load_golden(case):
    z = np.load(os.path.join(GOLDEN, case + '.npz'))
    return {k: z[k] for k in z.files}


def golden_options(g):
    return dict(verbose=False, avgOnly=bool(g['avgOnly']), visual=False, parallel=False,
                relion_data=golden_relion(g), thres=6000)


def golden_relion(g):
    return bool(g['relion']) if 'relion' in g else False


def golden_mask_volume(g):
    """The mask volume of a case run with p.mask_vol_file, else None."""
    v = g.get('mask_volume')
    return v.astype(np.float32) if v is not None and v.size else None


def golden_shifts(g):
    """(shx, shy) of a RELION case, else None."""
    return (g['shx'], g['shy']) if golden_relion(g) else None


def golden_micro(g):
    return dict(N=int(g['N']), pix_size=float(g['pix_size']), Cs=float(g['Cs']),
                EkV=float(g['EkV']), AmpContrast=float(g['AmpContrast']),
                gaussEnv=float(g['gaussEnv']))


def golden_ref(g, key):
    """Reference output `key`, restricted to the stored image slices when the case keeps only
    slices; returns (array, slice index or None)."""
    if 'ref_' + key in g:
        return g['ref_' + key], None
    return g['ref_%s_slices' % key], g['slice_idx']


@pytest.fixture(scope='session')
def cuda_ready():
    torch = pytest.importorskip('torch')
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from manifoldem_python_gb300 import _lib
    _lib.build()
    _lib.load()
    return torch
