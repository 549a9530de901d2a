"""Generate the golden fixtures of the distance stage by running the reference itself.

Run in a container that has a checkout of the reference (read-only); its ``modules`` directory
is given by ``--ref-modules DIR`` or the environment variable MANIFOLDEM_REF_MODULES.  The GPU
host never runs this.  For each case it writes a seeded synthetic SPIDER stack (values rounded to
float16 so the fixture can store them exactly at half size), runs the reference's
``getDistanceCTF_local_Conj9combinedS2.op`` on it through the reference's own module globals,
reads back the pickle it writes, and stores inputs and outputs in ``tests/golden/<case>.npz``.

The reference imports matplotlib and mrcfile (absent here) and uses ``np.complex`` and ``np.Inf``
(removed from numpy 2); the loader installs empty stand-ins for the two modules and restores the
two aliases before importing.  Nothing else of the reference is changed.

Usage:  python tests/golden/make_golden.py --ref-modules <reference>/modules [case ...]
"""
from __future__ import annotations

import dataclasses
import os
import pickle
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF_MODULES = os.environ.get('MANIFOLDEM_REF_MODULES', '')


def load_reference():
    np.complex = complex
    np.Inf = np.inf
    mpl = types.ModuleType('matplotlib')
    mpl.pyplot = types.ModuleType('matplotlib.pyplot')
    sys.modules.setdefault('matplotlib', mpl)
    sys.modules.setdefault('matplotlib.pyplot', mpl.pyplot)
    # mrcfile stand-in: mmap(name).data is the stack as stored (the only use, :259-262)
    sys.path.insert(0, REPO)
    from manifoldem_python_gb300 import mrc
    mrcfile = types.ModuleType('mrcfile')

    class _Mmap:
        def __init__(self, name, mode='r'):
            self.data = mrc.read_stack(name)

        def is_image_stack(self):
            return True

    class _Open(_Mmap):
        def __enter__(self):
            return self

        def __exit__(self, *exc):
            return False

    mrcfile.mmap = _Mmap
    mrcfile.open = _Open
    sys.modules.setdefault('mrcfile', mrcfile)
    # projectMask imports these names from the third-party `transformations` module but its
    # op() path (getEuler_from_PD, rotateVolumeEuler) does not call them
    tr = types.ModuleType('transformations')
    for name in ('euler_from_quaternion', 'quaternion_from_euler', 'quaternion_conjugate',
                 'quaternion_matrix'):
        setattr(tr, name, None)
    sys.modules.setdefault('transformations', tr)
    for d in (REF_MODULES, os.path.join(REF_MODULES, 'CC')):
        if d not in sys.path:
            sys.path.insert(0, d)
    import p as ref_p                                   # noqa: E402
    import getDistanceCTF_local_Conj9combinedS2 as ref_op  # noqa: E402
    return ref_p, ref_op


def reference_dm(D, seed=0):
    """The reference's diffusion-map embedding of D (k = nS, tune 3, as the manifold stage calls
    it, manifoldTrimmingAuto.py:51-54), with np.random seeded first."""
    import DMembeddingII                                # noqa: E402
    np.random.seed(seed)
    lamb, psi, sigma = DMembeddingII.op(np.array(D, copy=True), D.shape[0], 3, 60000)[:3]
    return lamb, psi, sigma


# name -> (synthetic config overrides, microscope overrides, options overrides,
#          image indices kept of the (nS, N, N) outputs; None keeps them whole)
CASES = {
    # even box, half of the PD are conjugate views (flipped, label -1)
    'even32_conj': (dict(N=32, n_pd=1, n_fixed=16, conj_pd_frac=1.0, seed=101), {}, {}, None),
    # odd box, finite Gaussian envelope in the CTF
    'odd33_env': (dict(N=33, n_pd=1, n_fixed=12, seed=102), dict(gaussEnv=0.15), {}, None),
    # averages only: D stays zero and CTF keeps its (nS, N, N) shape
    'even32_avgonly': (dict(N=32, n_pd=1, n_fixed=10, seed=103), {}, dict(avgOnly=True), None),
    # near-duplicate images (cancellation in the GEMM form)
    'even48_neardup': (dict(N=48, n_pd=1, n_fixed=40, near_dup_frac=0.1, seed=104), {}, {},
                       [0, 7, 39]),
    # the CPU-runnable workload: one PD, 300 images of 70x70 px
    'config1': (dict(N=70, n_pd=1, n_fixed=300, seed=11), {}, {}, [0, 1, 150, 299]),
    # RELION branch: MRC stack read as stored, per-particle shifts (order-3 'wrap' shift),
    # half of the PD conjugate views
    'relion32': (dict(N=32, n_pd=1, n_fixed=14, conj_pd_frac=1.0, seed=105), {},
                 dict(relion_data=True), None),
    # volume mask (p.mask_vol_file): projectMask's 2D mask multiplies the spectra and averages
    'volmask32': (dict(N=32, n_pd=1, n_fixed=14, conj_pd_frac=1.0, seed=106),
                  dict(volmask=True), {}, None),
}


def mask_volume(N):
    """A binary mask volume: an off-centre ellipsoid (float32, (N, N, N))."""
    z, y, x = np.meshgrid(*(np.arange(N, dtype=np.float64),) * 3, indexing='ij')
    c = 0.5 * N
    r = ((x - c - 2.) / (0.36 * N)) ** 2 + ((y - c + 1.) / (0.30 * N)) ** 2 + \
        ((z - c) / (0.26 * N)) ** 2
    return (r < 1).astype(np.float32)

FULL_KEEP = ['D', 'ind', 'q', 'df', 'CTF', 'imgAll', 'PD', 'PDs', 'Psis', 'imgAvg',
             'imgAvgFlip', 'imgAllFlip', 'imgLabels', 'Dnom', 'Nom', 'imgAllIntensity']
SLICE_KEYS = ['CTF', 'imgAll', 'imgAllFlip']


def run_reference_distance(name, synth_over, mic_over, opt_over):
    """The reference's distance stage on a seeded synthetic PD: (pickle dict, fixture inputs)."""
    sys.path.insert(0, REPO)
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    ref_p, ref_op = load_reference()
    mic_over = dict(mic_over)
    cfg = dataclasses.replace(CONFIGS['config1'], name=name, **synth_over)
    ds = make_dataset(cfg, device='cpu')
    stack16 = ds.stack.numpy().astype(np.float16)
    stack = stack16.astype(np.float32)
    ind = ds.CG[0].astype(np.int64)
    q = ds.q[:, ind]
    df = ds.df[ind]
    mic = dict(pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc, gaussEnv=np.inf)
    volmask = bool(mic_over.pop('volmask', False)) if mic_over else False
    mic.update(mic_over)
    options = dict(verbose=False, avgOnly=False, visual=False, parallel=False,
                   relion_data=False, thres=6000)
    options.update(opt_over)
    filterPar = dict(type='Butter', Qc=0.5, N=8)
    sh = ds.sh
    if options['relion_data']:
        rng = np.random.default_rng(cfg.seed + 7)
        sh = (rng.uniform(-2.5, 2.5, stack.shape[0]), rng.uniform(-2.5, 2.5, stack.shape[0]))
    with tempfile.TemporaryDirectory() as tmp:
        stack_file = os.path.join(tmp, 'stack.bin')
        if options['relion_data']:
            from manifoldem_python_gb300 import mrc
            stack_file = os.path.join(tmp, 'stack.mrcs')
            mrc.write_stack(stack_file, stack)
        else:
            stack.tofile(stack_file)
        ref_p.init()
        ref_p.nPix = cfg.N
        ref_p.pix_size = mic['pix_size']
        ref_p.Cs = mic['Cs']
        ref_p.EkV = mic['EkV']
        ref_p.AmpContrast = mic['AmpContrast']
        ref_p.gaussEnv = mic['gaussEnv']
        ref_p.mask_vol_file = ''
        mvol = None
        if volmask:
            from manifoldem_python_gb300 import mrc
            mvol = mask_volume(cfg.N)
            ref_p.mask_vol_file = os.path.join(tmp, 'mask.mrc')
            mrc.write_stack(ref_p.mask_vol_file, mvol)
        ref_p.dist_prog = os.path.join(tmp, 'progress')
        os.makedirs(ref_p.dist_prog)
        out_file = os.path.join(tmp, 'IMGs_prD_0')
        ref_op.op([ind, q, df, out_file, 0], filterPar, stack_file, sh, ds.nStot, options)
        with open(out_file, 'rb') as f:
            res = pickle.load(f)
        assert os.path.exists(os.path.join(ref_p.dist_prog, '0'))
    rec = dict(stack16=stack16, ind=ind, q=q, df=df, nStot=np.int64(ds.nStot), N=np.int64(cfg.N),
               pix_size=mic['pix_size'], Cs=mic['Cs'], EkV=mic['EkV'],
               AmpContrast=mic['AmpContrast'], gaussEnv=mic['gaussEnv'],
               avgOnly=np.bool_(options['avgOnly']), relion=np.bool_(options['relion_data']),
               shx=np.asarray(sh[0], dtype=np.float64), shy=np.asarray(sh[1], dtype=np.float64),
               ref_version=np.array(res['version']), ref_msk2=np.array(res['msk2']),
               mask_volume=(mvol.astype(np.uint8) if mvol is not None else np.zeros(0, np.uint8)),
               ref_CTF_shape=np.array(np.shape(res['CTF'])))
    return res, rec


def make_case(name):
    synth_over, mic_over, opt_over, slice_idx = CASES[name]
    res, rec = run_reference_distance(name, synth_over, mic_over, opt_over)
    for k in FULL_KEEP:
        if slice_idx is not None and k in SLICE_KEYS:
            rec['ref_%s_slices' % k] = np.asarray(res[k])[slice_idx]
        elif k not in ('q', 'df', 'ind'):
            rec['ref_' + k] = np.asarray(res[k])
    if slice_idx is not None:
        rec['slice_idx'] = np.array(slice_idx)
    if not rec['avgOnly'] and rec['ind'].shape[0] >= 40:
        lamb, psi, sigma = reference_dm(res['D'])
        rec.update(ref_dm_lambda=lamb, ref_dm_psi8=psi[:, :8], ref_dm_sigma=sigma)
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **rec)
    print('wrote', path, os.path.getsize(path) // 1024, 'KiB')


# NLSA cases: the reference's NLSA.op (modules/NLSA.py:23-158) on the outputs of its own
# distance stage, driven as psiAnalysisParS2.op drives it (:57-96): posPath = all images, the
# images ordered along diffusion coordinate 0 of D, ConOrder = floor(nS / conOrderRange) with
# conOrderRange 50, psiTrunc 8, tune 3.  Three runs on the same PD: the Wiener branch ('prD')
# with msk2 = 1, the Wiener branch with a 2D mask, and the unfiltered 'cuti' branch.  imgAll and
# CTF are rounded to float32 first so that the fixture stores the exact inputs at half size.
NLSA_CASES = {
    'nlsa32': dict(N=32, n_pd=1, n_fixed=160, seed=107),
}
NLSA_OUT = ['IMGT', 'Topo_mean', 'psirec', 'psiC1', 'sdiag', 'VX', 'mu', 'tau']


def nlsa_disc_mask(N):
    y, x = np.mgrid[0:N, 0:N]
    return ((x - 0.5 * N + 1.5) ** 2 + (y - 0.5 * N) ** 2) < (0.38 * N) ** 2


def make_nlsa_case(name, seed=5):
    res, _ = run_reference_distance(name, NLSA_CASES[name], {}, {})
    import NLSA                                         # noqa: E402
    D = np.asarray(res['D'], dtype=np.float64)
    imgAll = np.asarray(res['imgAll'], dtype=np.float32)
    nS = D.shape[0]
    N = imgAll.shape[1]
    # the pickle holds CTF as (nS, N^2); psiAnalysisParS2.py:73-74 reshapes it
    CTF = np.asarray(res['CTF'], dtype=np.float32).reshape(nS, N, N)
    _, psi, _ = reference_dm(D, seed=0)
    posPath = np.arange(nS)
    PosPsi1 = np.argsort(psi[:, 0])
    DD = D[posPath][:, posPath][PosPsi1][:, PosPsi1]
    ConOrder = int(np.floor(float(nS) / 50))
    par = dict(num=nS, ConOrder=ConOrder, k=nS - ConOrder, tune=3, nS=nS, save=False,
               psiTrunc=8)
    disc = nlsa_disc_mask(N)
    rec = dict(D=D, imgAll=imgAll, CTF=CTF, PosPsi1=PosPsi1, ConOrder=np.int64(ConOrder),
               msk_disc=disc, seed=np.int64(seed))
    runs = {'a': (np.array(res['msk2']), dict(outDir='', prD=0)),
            'b': (disc, dict(outDir='', prD=0)),
            'c': (np.array(1), dict(cuti=0))}
    for tag, (msk2, ext) in runs.items():
        np.random.seed(seed)
        out = NLSA.op(dict(par), DD.copy(), posPath, PosPsi1, imgAll.astype(np.float64), msk2,
                      CTF.astype(np.float64), ext)
        for key, val in zip(NLSA_OUT, out):
            val = np.asarray(val, dtype=np.float64)
            rec['%s_%s' % (tag, key)] = val.astype(np.float32) if key == 'IMGT' else val
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **rec)
    print('wrote', path, os.path.getsize(path) // 1024, 'KiB')


# Manifold trimming cases: the reference's manifoldTrimmingAuto.op (modules/
# manifoldTrimmingAuto.py:38-95) as manifoldAnalysis.op calls it (:81-99: posPath 0, tune 3,
# visual False, doSave Is True) on the reference's D of an earlier fixture, written to a distance
# pickle first.  rad 5 is the default (p.py:77); rad 3 makes the trimming loop run.  np.random
# is seeded before each run.  Stored: the psi pickle's arrays and the eigenvalue file's text.
TRIM_CASES = {
    'trim_config1': dict(source='config1', rads=(5.0, 3.0), seed=0),
    'trim_nlsa32': dict(source='nlsa32', rads=(3.0,), seed=0),
}
TRIM_KEYS = ['lamb', 'psi', 'sigma', 'mu', 'posPath', 'ind', 'logEps', 'logSumWij', 'popt',
             'R_squared']


def make_trim_case(name):
    spec = TRIM_CASES[name]
    ref_p, _ = load_reference()
    ref_p.init()
    sys.modules.setdefault('h5py', types.ModuleType('h5py'))
    import manifoldTrimmingAuto                         # noqa: E402
    import myio                                         # noqa: E402
    src = np.load(os.path.join(HERE, spec['source'] + '.npz'))
    D = np.asarray(src['ref_D'] if 'ref_D' in src.files else src['D'], dtype=np.float64)
    ind = np.asarray(src['ind']) if 'ind' in src.files else np.arange(D.shape[0])
    # D itself stays in the source fixture
    rec = dict(source=np.array(spec['source']), ind=ind, rads=np.array(spec['rads']),
               seed=np.int64(spec['seed']))
    with tempfile.TemporaryDirectory() as tmp:
        ref_p.psi_prog = os.path.join(tmp, 'progress')
        os.makedirs(ref_p.psi_prog)
        dist_file = os.path.join(tmp, 'IMGs_prD_0')
        myio.fout1(dist_file, ['D', 'ind'], [D, ind])
        for r, rad in enumerate(spec['rads']):
            psi_file = os.path.join(tmp, 'psi_%d' % r)
            eig_file = os.path.join(tmp, 'eig_%d.txt' % r)
            np.random.seed(spec['seed'])
            manifoldTrimmingAuto.op([dist_file, psi_file, eig_file, 0], 0, 3, rad, False,
                                    dict(outputFile='', Is=True))
            with open(psi_file, 'rb') as fh:
                out = pickle.load(fh)
            for key in TRIM_KEYS:
                if key != 'ind':
                    rec['r%d_%s' % (r, key)] = np.asarray(out[key])
            with open(eig_file) as fh:
                rec['r%d_eig_txt' % r] = np.array(fh.read())
            print(name, 'rad', rad, 'kept', len(out['posPath']), 'of', D.shape[0])
    path = os.path.join(HERE, name + '.npz')
    np.savez_compressed(path, **rec)
    print('wrote', path, os.path.getsize(path) // 1024, 'KiB')


if __name__ == '__main__':
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument('--ref-modules', default=REF_MODULES,
                    help="the reference's modules directory (or MANIFOLDEM_REF_MODULES)")
    ap.add_argument('cases', nargs='*')
    a = ap.parse_args()
    if not a.ref_modules or not os.path.isdir(a.ref_modules):
        sys.exit('give the reference modules directory: --ref-modules DIR')
    REF_MODULES = a.ref_modules
    names = a.cases or list(CASES) + list(NLSA_CASES) + list(TRIM_CASES)
    for n in names:
        if n in NLSA_CASES:
            make_nlsa_case(n)
        elif n in TRIM_CASES:
            make_trim_case(n)
        else:
            make_case(n)
