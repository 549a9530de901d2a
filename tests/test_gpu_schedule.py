"""Contraction schedules of the split-BF16 form (mem_plan_set_contraction): one CTA per tile or
persistent CTAs walking several tiles, two or four TMEM accumulators, one or several size
classes, 128- or 256-wide tiles on one SM, 256 x 128 tiles on a pair of SMs
(tcgen05.mma.cta_group::2).  Every schedule issues the same MMAs in the same order for
every output element, so D must be bit-identical across schedules (and within 1e-6 of an FP64
contraction, tested elsewhere)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(torch, ds, counts, contraction):
    from manifoldem_python_gb300.geometry import pd_geometry
    from manifoldem_python_gb300.pipeline import Plan, StageParams
    cfg = ds.cfg
    params = StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc,
                         precision='bf16x3')
    geoms = [pd_geometry(np.asarray(ind), ds.q[:, ind], ds.nStot) for ind in ds.CG]
    plan = Plan(params, counts, [g.psi_p for g in geoms], contraction=contraction)
    dev = torch.device('cuda')
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    outs = plan.allocate_outputs(('D',))
    plan.execute(ds.stack.to(dev), t(np.concatenate([g.stack_index for g in geoms])),
                 t(np.concatenate([g.flip for g in geoms])),
                 t(np.concatenate([g.psi_rad for g in geoms])),
                 t(np.concatenate([ds.df[ind] for ind in ds.CG]).astype(np.float64)), outs)
    torch.cuda.synchronize()
    plan.device_status()
    return outs['D'].cpu().numpy()


def test_every_schedule_gives_the_same_D(cuda_ready):
    torch = cuda_ready
    import dataclasses
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    cfg = dataclasses.replace(CONFIGS['config4'], N=64, n_pd=5, seed=9, conj_pd_frac=0.4)
    ds = make_dataset(cfg, device='cpu')
    sizes = [100, 2200, 300, 129, 700]          # 2200 images: 171 tiles, more than the SMs
    ds.CG = [ind[:0] for ind in ds.CG]          # rebuilt below with the chosen sizes
    rng = np.random.default_rng(3)
    pool = np.arange(ds.nStot)
    ds.CG = [np.sort(rng.choice(pool, n, replace=False)) for n in sizes]
    big = 2 ** 31 - 1
    schedules = [
        [dict(max_n=big, persistent=0, accumulators=2)],
        [dict(max_n=big, persistent=1, accumulators=2)],
        [dict(max_n=big, persistent=1, accumulators=4)],
        [dict(max_n=150, persistent=0, accumulators=2), dict(max_n=800, persistent=1,
                                                             accumulators=4),
         dict(max_n=big, persistent=1, accumulators=2)],
        [dict(max_n=big, persistent=1, accumulators=2, tile_n=256)],
        [dict(max_n=big, persistent=0, accumulators=2, tile_n=256)],
        [dict(max_n=200, persistent=1, accumulators=4, tile_n=128),
         dict(max_n=big, persistent=1, accumulators=2, tile_n=256)],
        [dict(max_n=big, persistent=0, accumulators=2, tile_m=256)],
        [dict(max_n=big, persistent=1, accumulators=4, tile_m=256)],
        [dict(max_n=150, persistent=0, accumulators=2, tile_n=256),
         dict(max_n=800, persistent=1, accumulators=2, tile_m=256),
         dict(max_n=big, persistent=0, accumulators=4, tile_m=256)],
    ]
    ref = _run(torch, ds, sizes, schedules[0])
    assert np.isfinite(ref).all()
    for sch in schedules[1:]:
        D = _run(torch, ds, sizes, sch)
        np.testing.assert_array_equal(D, ref)
