"""Drop-in replacement of ManifoldEM's per-PD distance worker, running on the GPU.

``op(input_data, filterPar, imgFileName, sh, nStot, options)`` has the signature, inputs, side
effects and outputs of ``getDistanceCTF_local_Conj9combinedS2.op``
(reference ``modules/getDistanceCTF_local_Conj9combinedS2.py:216-420``):

* ``input_data = [ind, q, df, outFile, prD]`` (as built by ``GetDistancesS2.divide``);
* the module-level configuration ``p`` (nPix, pix_size, Cs, EkV, gaussEnv, AmpContrast,
  mask_vol_file, dist_prog) is read from the reference's ``p`` module when it is loaded, else
  from this package's mirror;
* it writes the 19-key pickle to ``outFile`` (``myio.fout1``) with the reference's keys, dtypes
  and shapes, then creates the empty resume marker ``<p.dist_prog>/<prD>``;
* it returns None.

The image work (normalisation, filtering, masking, the two spline rotations, CTF, FFTs,
averages and D) runs in the CUDA library; host-side geometry stays in numpy/scipy as in the
reference.  There is no CPU fallback.
"""
from __future__ import annotations

import os
from typing import Dict

import numpy as np

from . import myio
from .p import params_module
from .pipeline import DEFAULT_OUTPUTS, DistanceStage, PdJob, StageParams

version = 'getDistanceCTF_local9, V 1.0'
PRECISION = os.environ.get('MANIFOLDEM_GB300_PRECISION', 'fp32')

OUTPUT_KEYS = ['D', 'ind', 'q', 'df', 'CTF', 'imgAll', 'msk2', 'PD', 'PDs', 'Psis', 'imgAvg',
               'imgAvgFlip', 'imgAllFlip', 'imgLabels', 'Dnom', 'Nom', 'imgAllIntensity',
               'version', 'options']


def stage_params(p, filterPar, options, precision=None) -> StageParams:
    return StageParams(N=int(p.nPix), pix_size=float(p.pix_size), Cs=float(p.Cs),
                       EkV=float(p.EkV), AmpContrast=float(p.AmpContrast),
                       gaussEnv=float(getattr(p, 'gaussEnv', np.inf)),
                       filter_type=filterPar['type'], filter_Qc=float(filterPar['Qc']),
                       filter_order=float(filterPar['N']),
                       avg_only=bool(options.get('avgOnly', False)),
                       precision=precision or PRECISION)


def read_spider_images(imgFileName: str, stack_index: np.ndarray, N: int):
    """Images ``stack_index`` of a SPIDER raw float32 stack, in storage order (the stage
    transposes them itself), plus the compact index of every entry."""
    mm = np.memmap(imgFileName, dtype='float32', mode='r')
    uniq, inv = np.unique(stack_index, return_inverse=True)
    imgs = np.empty((uniq.size, N, N), dtype=np.float32)
    for k, s in enumerate(uniq):
        imgs[k] = mm[s * N * N:(s + 1) * N * N].reshape(N, N)
    return imgs, inv.astype(np.int64)


def read_relion_images(imgFileName: str, stack_index: np.ndarray, sh):
    """Images ``stack_index`` of a RELION MRC stack as stored (``:259-262``), the compact index
    of every entry, and the particles' shifts (shx, shy) in compact order."""
    from . import mrc
    data = mrc.read_stack(imgFileName)
    uniq, inv = np.unique(stack_index, return_inverse=True)
    imgs = np.ascontiguousarray(data[uniq], dtype=np.float32)
    sh_c = (np.asarray(sh[0], dtype=np.float64)[uniq], np.asarray(sh[1], dtype=np.float64)[uniq])
    return imgs, inv.astype(np.int64), sh_c


def volume_mask(p, device):
    """The GPU projector of p.mask_vol_file's volume (:303-308), or None without a mask file."""
    path = getattr(p, 'mask_vol_file', '')
    if not path:
        return None
    from . import mrc
    from .pipeline import VolumeMask
    return VolumeMask(np.asarray(mrc.read_stack(path)), device)


def load_images(imgFileName: str, stack_index: np.ndarray, N: int, options: dict, sh):
    """The stage's image input for either branch: (images, compact index, shifts or None)."""
    if options.get('relion_data'):
        return read_relion_images(imgFileName, stack_index, sh)
    imgs, compact = read_spider_images(imgFileName, stack_index, N)
    return imgs, compact, None


def assemble(job: PdJob, geom, res: Dict[str, np.ndarray], N: int, options: dict, msk2=1,
             image_dtype=np.float64):
    """The reference's output dict (keys, dtypes and shapes as written at :409-412).
    ``image_dtype=np.float32`` (opt-in) keeps the per-image arrays CTF, imgAll and imgAllFlip
    in the float32 the GPU computes them in, halving the pickle; keys and shapes are unchanged."""
    nS = job.ind.shape[0]
    avg_only = bool(options.get('avgOnly', False))
    D = res['D'] if not avg_only else np.zeros((nS, nS))
    CTF = res['ctf'].astype(image_dtype)
    if not avg_only:
        CTF = CTF.reshape(nS, N * N)
    vals = [D, job.ind, job.q, job.df, CTF, res['img_all'].astype(image_dtype), msk2, geom.PD,
            geom.PDs, geom.Psis, res['img_avg'], res['img_avg_flip'],
            res['img_all_flip'].astype(image_dtype), geom.imgLabels, geom.Dnom, geom.Nom,
            res['img_all_intensity'], version, options]
    return dict(zip(OUTPUT_KEYS, vals))


def op(input_data, filterPar, imgFileName, sh, nStot, options):
    import torch

    p = params_module()
    ind, q, df, outFile, prD = input_data[:5]
    ind = np.asarray(ind)
    q = np.asarray(q, dtype=np.float64)
    df = np.asarray(df, dtype=np.float64)
    N = int(p.nPix)
    stage = DistanceStage(stage_params(p, filterPar, options))
    mask = volume_mask(p, stage.device)
    job = PdJob(ind=ind, q=q, df=df, outFile=outFile, prD=prD)
    geom = stage.geometry([job], nStot)[0]
    imgs, compact, sh_c = load_images(imgFileName, geom.stack_index, N, options, sh)
    geom.stack_index = compact
    stack = torch.from_numpy(imgs).to(stage.device)
    res = stage.run([job], stack, nStot, outputs=DEFAULT_OUTPUTS, geoms=[geom], sh=sh_c,
                    mask=mask)[0]
    out = assemble(job, geom, res, N, options, msk2=res.get('msk2', 1))
    myio.fout1(outFile, OUTPUT_KEYS, [out[k] for k in OUTPUT_KEYS])
    progress_fname = os.path.join(p.dist_prog, '%s' % prD)
    open(progress_fname, 'a').close()
