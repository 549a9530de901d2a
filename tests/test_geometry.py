"""Host-side bookkeeping of the product (geometry.py) against the reference's outputs: index and
label bookkeeping bit-exact, angles bit-exact, psi_p equal to the oracle's least-squares fit."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden
from manifoldem_python_gb300.geometry import index_bookkeeping, pd_geometry
from oracle import distance_oracle as O


@pytest.mark.parametrize('case', GOLDEN_CASES)
def test_geometry_bit_exact(case):
    g = load_golden(case)
    geo = pd_geometry(g['ind'], g['q'], int(g['nStot']))
    np.testing.assert_array_equal(geo.imgLabels, g['ref_imgLabels'])
    for k in ('PD', 'PDs', 'Psis', 'Nom', 'Dnom'):
        np.testing.assert_array_equal(getattr(geo, k), g['ref_' + k], err_msg=k)
    assert geo.psi_p == O.psi_ang(g['ref_PD'])


def test_index_bookkeeping_conjugates():
    nStot = 10
    ind = np.array([0, 4, 5, 9, 7], dtype=np.int64)
    sidx, flip, lab = index_bookkeeping(ind, nStot)
    np.testing.assert_array_equal(sidx, [0, 4, 0, 4, 2])
    np.testing.assert_array_equal(flip, [0, 0, 1, 1, 1])
    np.testing.assert_array_equal(lab, [1, 1, -1, -1, -1])
    # odd nStot: the comparison is in floating point (ind < nStot/2)
    sidx, flip, lab = index_bookkeeping(np.array([2, 3]), 5)
    np.testing.assert_array_equal(flip, [0, 1])


def test_empty_pd_raises_like_the_reference():
    """An empty PD: the reference's op() fails in psi_ang (q2Spider's least-squares fit of a NaN
    direction, getDistanceCTF_local_Conj9combinedS2.py:297-313) with scipy's ValueError; the
    host geometry of the GPU stage fails the same way, before anything reaches the GPU."""
    import warnings
    import numpy as np
    import pytest
    from manifoldem_python_gb300.geometry import pd_geometry
    with warnings.catch_warnings():
        warnings.simplefilter('ignore', RuntimeWarning)
        with pytest.raises(ValueError, match='not finite'):
            pd_geometry(np.zeros(0, dtype=np.int64), np.zeros((4, 0)), 20)
