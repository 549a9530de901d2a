"""Parameter-file persistence of the distance stage's globals (reference ``modules/set_params.py``):
``op(1)`` loads ``params_<proj_name>.pkl`` into the configuration module, ``op(0)`` writes it
back.  The file holds ``{'params': {name: value}}``."""
import os

from . import myio
from .p import params_module

KEYS = ('proj_name', 'user_dir', 'resProj', 'relion_data', 'ncpu', 'machinefile',
        'avg_vol_file', 'img_stack_file', 'align_param_file', 'mask_vol_file', 'num_part', 'Cs',
        'EkV', 'AmpContrast', 'nPix', 'pix_size', 'obj_diam', 'resol_est', 'ap_index',
        'ang_width', 'sh', 'PDsizeThL', 'PDsizeThH', 'S2rescale', 'S2iso', 'numberofJobs',
        'num_psis', 'dim', 'temperature')


def _file(p):
    return 'params_{}.pkl'.format(p.proj_name)


def op(do):
    p = params_module()
    if do == 1:
        if not os.path.exists(_file(p)):
            return
        data = myio.fin1(_file(p))
        params = (data or {}).get('params', {})
        for k in KEYS:
            if k in params:
                setattr(p, k, params[k])
    elif do == 0:
        params = {k: getattr(p, k) for k in KEYS if hasattr(p, k)}
        myio.fout1(_file(p), ['params'], [params])
    elif do == -1:
        data = myio.fin1(_file(p))
        for k, v in (data or {}).get('params', {}).items():
            print(k, v)
