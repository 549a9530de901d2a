"""Failure paths of the GPU stage, made without faulting the GPU.

* A bounded wait of the tensor-core contraction that runs out: the plan's wait limit is set low
  (mem_plan_set_wait_limit) and the contraction's producer is told to withhold one K chunk
  (MEM_TEST_WITHHOLD_CHUNK, read when the plan is created), so the MMA issuer's wait for that
  chunk can only end by its limit.  The kernel must return, the workspace status must read
  MEM_ERR_DEVICE_TIMEOUT, and the next plan on the same device must run correctly (the kernel
  freed its tensor memory and the context is usable).
* An entry whose stack index lies outside the stack: it is never read (checked before any
  access), the status reads MEM_ERR_INVALID, and the next execute with valid indices clears it.
"""
import ctypes

import numpy as np
import pytest

from conftest import golden_micro, load_golden

pytestmark = pytest.mark.gpu


def _inputs(torch, g):
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    stage = DistanceStage(StageParams(precision='bf16x3', **golden_micro(g)))
    job = PdJob(ind=g['ind'], q=g['q'], df=g['df'])
    geom = stage.geometry([job], int(g['nStot']))[0]
    dev = torch.device('cuda')
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    return dict(stack=t(g['stack16'].astype(np.float32)), sidx=t(geom.stack_index),
                flip=t(geom.flip), psi=t(geom.psi_rad), df=t(g['df'].astype(np.float64)),
                psi_p=geom.psi_p)


def _plan(torch, g, inp):
    from manifoldem_python_gb300.pipeline import Plan, StageParams
    params = StageParams(precision='bf16x3', **golden_micro(g))
    return Plan(params, [g['ind'].shape[0]], [inp['psi_p']])


def _run(torch, plan, inp, sidx=None):
    outs = plan.allocate_outputs(('D',))
    plan.execute(inp['stack'], inp['sidx'] if sidx is None else sidx, inp['flip'], inp['psi'],
                 inp['df'], outs)
    torch.cuda.synchronize()
    n = int(plan.counts[0])
    return outs['D'].cpu().numpy().reshape(n, n)


def _status(plan):
    return plan.lib.mem_workspace_status(plan.handle, plan.workspace.data_ptr())


@pytest.mark.parametrize('tile_m', ['128', '256'])
def test_contraction_wait_runs_out_and_returns(cuda_ready, monkeypatch, tile_m):
    """tile_m 256: the CTA-pair kernel (both CTAs' copies count on the even CTA's barriers)."""
    torch = cuda_ready
    from manifoldem_python_gb300 import _lib
    g = load_golden('config1')               # 300 images: three 128-row blocks, six tiles
    inp = _inputs(torch, g)
    good = _run(torch, _plan(torch, g, inp), inp)
    monkeypatch.setenv('MEM_TEST_WITHHOLD_CHUNK', '7')
    monkeypatch.setenv('MEM_TC_TILE_M', tile_m)
    monkeypatch.setenv('MEM_AUTOTUNE_CACHE', '/nonexistent/autotune.json')
    bad_plan = _plan(torch, g, inp)
    monkeypatch.delenv('MEM_TEST_WITHHOLD_CHUNK')
    monkeypatch.delenv('MEM_TC_TILE_M')
    assert bad_plan.lib.mem_plan_set_wait_limit(bad_plan.handle, 200000) == _lib.MEM_OK
    assert bad_plan.lib.mem_plan_set_wait_limit(bad_plan.handle, 10) == _lib.MEM_ERR_INVALID
    _run(torch, bad_plan, inp)               # returns: every wait is bounded
    assert _status(bad_plan) == _lib.MEM_ERR_DEVICE_TIMEOUT
    with pytest.raises(_lib.MemError) as ei:
        bad_plan.device_status()
    assert ei.value.status == _lib.MEM_ERR_DEVICE_TIMEOUT
    # the device is usable and tensor memory was released: a fresh plan gives the same D
    again = _run(torch, _plan(torch, g, inp), inp)
    np.testing.assert_array_equal(again, good)


def test_out_of_range_stack_index_is_flagged_not_read(cuda_ready):
    torch = cuda_ready
    from manifoldem_python_gb300 import _lib
    g = load_golden('even32_conj')
    inp = _inputs(torch, g)
    plan = _plan(torch, g, inp)
    good = _run(torch, plan, inp)
    assert _status(plan) == _lib.MEM_OK
    bad = inp['sidx'].clone()
    bad[3] = int(inp['stack'].shape[0]) + 7
    bad[5] = -2
    D = _run(torch, plan, inp, sidx=bad)
    assert _status(plan) == _lib.MEM_ERR_INVALID
    assert np.isnan(D[3, 4]) and np.isnan(D[5, 6])
    D = _run(torch, plan, inp)                # the status is cleared by the next execute
    assert _status(plan) == _lib.MEM_OK
    np.testing.assert_array_equal(D, good)
