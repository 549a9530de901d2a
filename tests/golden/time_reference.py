"""Time the reference's own distance stage against the FP64 CPU port in ``oracle/`` on the same
machine and the same PD (the 300-image 70 px config1 case of the golden fixtures).

The CPU baseline of ``bench.py`` times the port (the reference itself is not on the GPU host);
this script measures how the two compare where both can run.  Like ``make_golden.py`` it needs a
checkout of the reference (``--ref-modules DIR`` or MANIFOLDEM_REF_MODULES) and runs the
reference through its own module globals with the same stand-ins for its absent imports.

Usage:  python tests/golden/time_reference.py --ref-modules <reference>/modules [--repeat 3]
"""
from __future__ import annotations

import argparse
import dataclasses
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, REPO)

import make_golden  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref-modules', default=make_golden.REF_MODULES)
    ap.add_argument('--repeat', type=int, default=3)
    args = ap.parse_args()
    if not args.ref_modules:
        raise SystemExit('give --ref-modules or MANIFOLDEM_REF_MODULES')
    make_golden.REF_MODULES = args.ref_modules
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    from oracle import distance_oracle as O
    ref_p, ref_op = make_golden.load_reference()
    cfg = dataclasses.replace(CONFIGS['config1'], name='config1')
    ds = make_dataset(cfg, device='cpu')
    stack = ds.stack.numpy().astype(np.float16).astype(np.float32)
    ind = ds.CG[0].astype(np.int64)
    q, df = ds.q[:, ind], ds.df[ind]
    mic = dict(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    options = dict(verbose=False, avgOnly=False, visual=False, parallel=False,
                   relion_data=False, thres=6000)
    filterPar = dict(type='Butter', Qc=0.5, N=8)
    t_ref, t_port = [], []
    with tempfile.TemporaryDirectory() as tmp:
        stack_file = os.path.join(tmp, 'stack.bin')
        stack.tofile(stack_file)
        ref_p.init()
        ref_p.nPix = cfg.N
        ref_p.pix_size, ref_p.Cs, ref_p.EkV = cfg.pix, cfg.cs, cfg.kv
        ref_p.AmpContrast, ref_p.gaussEnv, ref_p.mask_vol_file = cfg.ampc, np.inf, ''
        ref_p.dist_prog = os.path.join(tmp, 'progress')
        os.makedirs(ref_p.dist_prog)
        for r in range(args.repeat):
            out_file = os.path.join(tmp, 'IMGs_prD_%d' % r)
            t0 = time.perf_counter()
            ref_op.op([ind, q, df, out_file, r], filterPar, stack_file, ds.sh, ds.nStot, options)
            t_ref.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            O.pd_op(ind, q, df, stack, ds.nStot, **mic)
            t_port.append(time.perf_counter() - t0)
    print('config1 PD (%d images of %d px), one core each, best of %d:' % (len(ind), cfg.N,
                                                                         args.repeat))
    print('  reference getDistanceCTF_local_Conj9combinedS2.op: %.3f s (includes its pickle write)'
          % min(t_ref))
    print('  FP64 port oracle/distance_oracle.pd_op:          %.3f s' % min(t_port))
    print('  ratio: %.2fx' % (min(t_ref) / min(t_port)))


if __name__ == '__main__':
    main()
