"""Module-level configuration the distance stage reads, mirroring the reference's ``p`` module
(``modules/p.py:13-114`` globals, ``:116-225`` directories).  Only the names the distance stage
and its driver use are defined here.  When the reference's own ``p`` module is loaded (imported
as ``p``), the drop-in modules read that one instead (see ``params_module``)."""
import os
import sys

import numpy as np


def init():
    g = globals()
    g.update(proj_name='', user_dir='', resProj=0, relion_data=False, ncpu=1, machinefile=False,
             eps=1e-10, img_stack_file='', align_param_file='', mask_vol_file='', num_part=0,
             Cs=2.7, EkV=300.0, AmpContrast=0.1, gaussEnv=np.inf, nPix=0, pix_size=1.0,
             PDsizeThL=100, PDsizeThH=2000, numberofJobs=0, tess_file='', dist_dir='',
             dist_prog='', dist_file='', num_eigs=15, tune=3, rad=5, out_dir='', psi_dir='',
             psi_prog='', psi_file='')


def create_dir():
    """Distance-stage and diffusion-map directories under ``user_dir`` (reference
    p.py:116-132, :179, :209)."""
    g = globals()
    g['dist_dir'] = os.path.join(user_dir, 'outputs_{}/distances/'.format(proj_name))
    os.makedirs(dist_dir, exist_ok=True)
    g['dist_prog'] = os.path.join(dist_dir, 'progress/')
    os.makedirs(dist_prog, exist_ok=True)
    g['dist_file'] = '{}/IMGs_'.format(dist_dir)
    g['tess_file'] = os.path.join(user_dir, 'outputs_{}/selecGCs'.format(proj_name))
    g['psi_dir'] = os.path.join(user_dir, 'outputs_{}/diff_maps/'.format(proj_name))
    os.makedirs(psi_dir, exist_ok=True)
    g['psi_prog'] = os.path.join(psi_dir, 'progress/')
    os.makedirs(psi_prog, exist_ok=True)
    g['psi_file'] = '{}/gC_trimmed_psi_'.format(psi_dir)


def params_module():
    """The configuration module in effect: the reference's ``p`` if it has been imported under
    that name and populated, else this mirror."""
    ref = sys.modules.get('p')
    if ref is not None and ref is not sys.modules[__name__] and hasattr(ref, 'nPix'):
        return ref
    return sys.modules[__name__]


init()
