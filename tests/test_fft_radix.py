"""The shared-memory FFT's in-register butterflies (csrc/fft_radix.cuh), built for the host with
g++ and compared with numpy's FFT.  CPU only."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, '..', 'manifoldem_python_gb300', 'csrc')


def _cuda_include():
    for root in (os.environ.get('CUDA_HOME'), '/usr/local/cuda'):
        if root and os.path.exists(os.path.join(root, 'include', 'vector_types.h')):
            return os.path.join(root, 'include')
    return None


def test_dft_butterflies_match_numpy(tmp_path):
    inc = _cuda_include()
    if shutil.which('g++') is None or inc is None:
        pytest.skip('g++ or the CUDA headers are missing')
    exe = str(tmp_path / 'fft_radix_host')
    subprocess.run(['g++', '-std=c++17', '-O1', '-I', CSRC, '-I', inc,
                    os.path.join(HERE, 'native', 'fft_radix_host.cpp'), '-o', exe], check=True)
    lines = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines()
    assert len(lines) == 36
    for a, b in zip(lines[0::2], lines[1::2]):
        ta, tb = a.split(), b.split()
        R, d = int(ta[1]), int(ta[2])
        x = np.array(ta[3:], float).view(complex)
        y = np.array(tb[3:], float).view(complex)
        ref = np.fft.fft(x) if d > 0 else np.fft.ifft(x) * R
        err = np.abs(y - ref).max() / np.abs(ref).max()
        assert err < 4e-7, (R, d, err)
