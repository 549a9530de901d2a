"""Minimal MRC / MRCS stack reader and writer (MRC2014 layout), for RELION particle stacks.

The reference reads RELION stacks with the third-party ``mrcfile`` package
(``getDistanceCTF_local_Conj9combinedS2.py:259-262``: ``mrcfile.mmap(name, 'r').data[i]``),
which is not a dependency here.  This module reads the same images: a 1024-byte main header
(nx, ny, nz, mode in the first four 32-bit words, the extended-header length ``nsymbt`` at byte
92, the machine stamp at byte 212), an optional extended header, then nz images of ny rows of
nx values, returned as a read-only memmap of shape (nz, ny, nx) -- the ``.data`` array of
mrcfile.  Modes 2 (float32), 1 (int16), 6 (uint16) and 12 (float16) are read.
"""
from __future__ import annotations

import os

import numpy as np

_MODES = {0: np.int8, 1: np.int16, 2: np.float32, 6: np.uint16, 12: np.float16}


def _byteorder(stamp: bytes) -> str:
    # 0x44 0x44 / 0x44 0x41: little endian; 0x11 0x11: big endian
    return '>' if stamp[0] == 0x11 else '<'


def read_header(path: str):
    with open(path, 'rb') as f:
        head = f.read(1024)
    if len(head) < 1024:
        raise ValueError('%s: shorter than an MRC header' % path)
    bo = _byteorder(head[212:216])
    nx, ny, nz, mode = np.frombuffer(head[:16], dtype=bo + 'i4')
    nsymbt = int(np.frombuffer(head[92:96], dtype=bo + 'i4')[0])
    if int(mode) not in _MODES:
        raise ValueError('%s: unsupported MRC mode %d' % (path, int(mode)))
    return dict(nx=int(nx), ny=int(ny), nz=int(nz), mode=int(mode), nsymbt=nsymbt, byteorder=bo)


def read_stack(path: str) -> np.ndarray:
    """Memory-mapped image stack, shape (nz, ny, nx), as stored."""
    h = read_header(path)
    dt = np.dtype(_MODES[h['mode']]).newbyteorder(h['byteorder'])
    return np.memmap(path, dtype=dt, mode='r', offset=1024 + h['nsymbt'],
                     shape=(h['nz'], h['ny'], h['nx']))


def write_stack(path: str, data: np.ndarray) -> None:
    """Write a float32 (nz, ny, nx) stack with a little-endian MRC2014 header."""
    data = np.ascontiguousarray(data, dtype='<f4')
    if data.ndim == 2:
        data = data[None]
    nz, ny, nx = data.shape
    head = np.zeros(256, dtype='<i4')
    head[0:4] = (nx, ny, nz, 2)
    head[7:10] = (nx, ny, nz)                       # mx, my, mz
    cell = np.array([nx, ny, nz], dtype='<f4')
    head[10:13] = cell.view('<i4')                  # cell dimensions (pixel units)
    head[13:16] = np.array([90, 90, 90], dtype='<f4').view('<i4')
    head[16:19] = (1, 2, 3)                         # mapc, mapr, maps
    raw = bytearray(head.tobytes())
    raw[208:212] = b'MAP '
    raw[212:216] = bytes([0x44, 0x44, 0, 0])
    with open(path, 'wb') as f:
        f.write(bytes(raw))
        f.write(data.tobytes())
    assert os.path.getsize(path) == 1024 + data.nbytes
