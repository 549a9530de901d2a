"""Build and load the C-ABI library ``libmanifoldem_gb300.so`` (CUDA, sm_103a).

The library is compiled in-tree from ``csrc/*.cu`` with nvcc (one translation unit per process,
compiled in parallel) and loaded with ctypes.  There is no fallback: importing the product path
without the library raises ``LibraryNotBuilt``.
"""
from __future__ import annotations

import ctypes
import glob
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor
from typing import Optional

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, 'csrc')
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, 'include')
BUILD_DIR = os.path.join(REPO, '_build')
LIB_PATH = os.path.join(HERE, 'libmanifoldem_gb300.so')
SOURCES = ['abi.cu', 'prologue.cu', 'gemm_fp32.cu', 'gemm_tc.cu', 'noalloc.cu', 'image_fft.cu',
           'dmap.cu', 'relion.cu', 'mask.cu', 'nlsa.cu', 'rotate_band.cu']
ARCH_FLAGS = ['-gencode', 'arch=compute_103a,code=sm_103a']

# status codes (include/manifoldem_gb300.h)
MEM_OK = 0
MEM_ERR_INVALID = -1
MEM_ERR_UNSUPPORTED = -2
MEM_ERR_WORKSPACE = -3
MEM_ERR_CUDA = -4
MEM_ERR_CUFFT = -5
MEM_ERR_DEVICE_TIMEOUT = -6
MEM_ERR_NO_DEVICE = -7
MEM_ERR_TOO_LARGE = -8
MEM_PREC_FP32 = 0
MEM_PREC_SPLIT_BF16 = 1
MEM_FILTER_BUTTER = 0
MEM_FILTER_GAUSS = 1


class LibraryNotBuilt(RuntimeError):
    pass


class MemError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__('%s failed: %s (status %d)' % (what, status_string(status), status))
        self.status = status


def _nvcc() -> str:
    for c in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if c and os.path.exists(c):
            return c
    raise LibraryNotBuilt('nvcc not found')


def _cuda_lib_dir(nvcc: str) -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc))), 'lib64')


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile csrc/*.cu for sm_103a and link the shared library; returns its path."""
    nvcc = _nvcc()
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in SOURCES]
    deps = srcs + sorted(glob.glob(os.path.join(CSRC, '*.cuh'))) + [
        os.path.join(INCLUDE, 'manifoldem_gb300.h')]
    if not force and os.path.exists(LIB_PATH):
        lib_m = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= lib_m for d in deps):
            return LIB_PATH
    common = ARCH_FLAGS + ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC',
                           '-I', INCLUDE]

    def compile_one(src):
        obj = os.path.join(BUILD_DIR, os.path.basename(src).replace('.cu', '.o'))
        cmd = [nvcc] + common + ['-c', src, '-o', obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise LibraryNotBuilt('nvcc failed on %s:\n%s' % (src, r.stderr))
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(compile_one, srcs))
    libdir = _cuda_lib_dir(nvcc)
    tmp = LIB_PATH + '.tmp'
    cmd = [nvcc, '-shared', '-cudart', 'shared'] + ARCH_FLAGS + objs + [
        '-o', tmp, '-L', libdir, '-lcufft', '-Xlinker', '-rpath', '-Xlinker', libdir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise LibraryNotBuilt('link failed:\n%s' % r.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


# ---------------------------------------------------------------------------- ctypes structs
c_int32, c_int64, c_double, c_void_p, c_size_t = (ctypes.c_int32, ctypes.c_int64,
                                                  ctypes.c_double, ctypes.c_void_p,
                                                  ctypes.c_size_t)


class MemParams(ctypes.Structure):
    _fields_ = [('N', c_int32), ('filter_type', c_int32), ('filter_Qc', c_double),
                ('filter_order', c_double), ('pix_size', c_double), ('Cs', c_double),
                ('EkV', c_double), ('gaussEnv', c_double), ('AmpContrast', c_double),
                ('avg_only', c_int32), ('precision', c_int32)]


ABI_VERSION = 5            # MEM_ABI_VERSION of include/manifoldem_gb300.h these structs follow


class MemInputs(ctypes.Structure):
    _fields_ = [('stack', c_void_p), ('num_stack', c_int64), ('stack_index', c_void_p),
                ('flip', c_void_p), ('psi_rad', c_void_p), ('df', c_void_p),
                ('shift_yx', c_void_p), ('pd_mask', c_void_p)]


class MemContractionConfig(ctypes.Structure):
    _fields_ = [('max_n', c_int32), ('persistent', c_int32), ('accumulators', c_int32),
                ('tile_n', c_int32), ('tile_m', c_int32), ('reserved', c_int32)]


class MemOutputs(ctypes.Structure):
    _fields_ = [('D', c_void_p), ('img_avg', c_void_p), ('img_avg_flip', c_void_p),
                ('img_all_intensity', c_void_p), ('img_all', c_void_p),
                ('img_all_flip', c_void_p), ('ctf', c_void_p), ('spectrum', c_void_p),
                ('pair_norm', c_void_p)]


# exported symbols and their signatures (restype, argtypes)
SIGNATURES = {
    'mem_abi_version': (c_int32, []),
    'mem_status_string': (ctypes.c_char_p, [c_int32]),
    'mem_plan_create': (c_int32, [ctypes.POINTER(MemParams), c_int32, c_void_p, c_void_p,
                                  ctypes.POINTER(c_void_p)]),
    'mem_plan_destroy': (c_int32, [c_void_p]),
    'mem_plan_workspace_size': (c_int32, [c_void_p, ctypes.POINTER(c_size_t)]),
    'mem_plan_num_images': (c_int64, [c_void_p]),
    'mem_plan_d_elements': (c_int64, [c_void_p]),
    'mem_plan_num_pairs': (c_int64, [c_void_p]),
    'mem_plan_upload': (c_int32, [c_void_p, c_void_p, c_size_t, c_void_p]),
    'mem_plan_execute': (c_int32, [c_void_p, ctypes.POINTER(MemInputs),
                                   ctypes.POINTER(MemOutputs), c_void_p, c_size_t, c_void_p]),
    'mem_plan_execute_split': (c_int32, [c_void_p, ctypes.POINTER(MemInputs),
                                         ctypes.POINTER(MemOutputs), c_void_p, c_size_t, c_void_p,
                                         c_void_p]),
    'mem_workspace_status': (c_int32, [c_void_p, c_void_p]),
    'mem_plan_set_wait_limit': (c_int32, [c_void_p, c_int64]),
    'mem_plan_set_contraction': (c_int32, [c_void_p, c_int32,
                                           ctypes.POINTER(MemContractionConfig)]),
    'mem_noalloc_status': (c_int32, [c_void_p]),
    'mem_dm_symmetrise': (c_int32, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    'mem_dm_sweep': (c_int32, [c_void_p, c_int64, c_void_p, c_int32, c_double, c_void_p,
                               c_void_p]),
    'mem_dm_laplacian': (c_int32, [c_void_p, c_int64, c_double, c_void_p, c_void_p]),
    'mem_mask_coefficients_size': (c_int32, [c_int32, ctypes.POINTER(c_size_t)]),
    'mem_mask_prepare': (c_int32, [c_void_p, c_int32, c_void_p, c_void_p]),
    'mem_mask_project': (c_int32, [c_void_p, c_int32, c_int32, c_void_p, c_void_p, c_void_p]),
    'mem_nlsa_con_distances': (c_int32, [c_void_p, c_int32, c_int32, c_void_p, c_void_p]),
    'mem_nlsa_workspace_size': (c_int32, [c_int32, c_int32, c_int32, c_int32, c_int32,
                                          ctypes.POINTER(c_size_t)]),
    'mem_nlsa_snapshots': (c_int32, [c_int32, c_int32, c_int32, c_int32, c_void_p, c_void_p,
                                     c_void_p, c_void_p, c_void_p, c_size_t, c_void_p,
                                     c_void_p]),
    'mem_plan_set_timing': (c_int32, [c_void_p, c_int32]),
    'mem_plan_phase_times': (c_int32, [c_void_p, ctypes.POINTER(ctypes.c_float), c_int32]),
    'mem_phase_name': (ctypes.c_char_p, [c_int32]),
    'mem_pd_distances_noalloc': (c_int32, [ctypes.POINTER(MemParams), c_int32, c_void_p,
                                            c_void_p, c_void_p, c_void_p]),
    'mem_pd_batch': (c_int32, [ctypes.POINTER(MemParams), c_int32, c_void_p, c_void_p,
                               ctypes.POINTER(MemInputs), ctypes.POINTER(MemOutputs), c_void_p,
                               c_size_t, c_void_p]),
}

_lib: Optional[ctypes.CDLL] = None
_lock = threading.Lock()


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Load the library (it must have been built); raises LibraryNotBuilt otherwise."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or LIB_PATH
        if not os.path.exists(path):
            raise LibraryNotBuilt('%s is missing: run manifoldem_python_gb300._lib.build() '
                                  '(or __graft_entry__.build())' % path)
        lib = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.mem_abi_version() != ABI_VERSION:
            raise LibraryNotBuilt('%s has ABI version %d, expected %d: rebuild it'
                                  % (path, lib.mem_abi_version(), ABI_VERSION))
        _lib = lib
        return lib


def status_string(status: int) -> str:
    try:
        return load().mem_status_string(status).decode()
    except LibraryNotBuilt:
        return 'status %d' % status


def check(status: int, what: str) -> None:
    if status != MEM_OK:
        raise MemError(status, what)
