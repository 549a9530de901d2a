"""Driver of the distance stage over all projection directions, on one GPU.

Mirrors ``GetDistancesS2.op`` (reference ``modules/GetDistancesS2.py:53-124``): it loads the
tessellation file (``CG``, ``q``, ``df``, ``sh``), builds the job list of the PDs that have no
resume marker (``fileCheck``/``divide``, ``:29-47``), runs them, writes one pickle per PD plus its
marker and reports progress through an optional Qt-style signal (``argv[0].emit(percent)``).

Instead of a process pool it submits the pending PDs to the GPU in HBM-admitted batches; each
batch is one plan/execute of the C ABI.  The resume semantics are the reference's: a PD counts
as done when ``<dist_prog>/<prD>`` exists, and markers are written after the pickle.
"""
from __future__ import annotations

import os
import time
from typing import List, Optional

import numpy as np

from . import myio, set_params
from .getDistanceCTF_local_Conj9combinedS2 import (OUTPUT_KEYS, assemble, load_images,
                                                    stage_params, volume_mask)
from .p import params_module
from .pipeline import DEFAULT_OUTPUTS, DistanceStage, PdJob, admit_batches
from .sharding import shard

FILTER_PAR = dict(type='Butter', Qc=0.5, N=8)


def fileCheck() -> List[int]:
    p = params_module()
    fin = []
    for root, dirs, files in os.walk(p.dist_prog):
        for f in sorted(files):
            if not f.startswith('.'):
                fin.append(int(f))
    return fin


def divide(CG, q, df, N) -> list:
    p = params_module()
    ll = []
    fin = fileCheck()
    for prD in range(N):
        ind = CG[prD]
        dist_file = '{}prD_{}'.format(p.dist_file, prD)
        if prD not in fin:
            ll.append([ind, q[:, ind], df[ind], dist_file, prD])
    return ll


def count(N) -> int:
    return N - len(fileCheck())


def rank_jobs(input_data: list, N: int, rank: int, world: int) -> list:
    """This rank's share of the pending jobs (one process per GPU): the longest-processing-
    time-first partition of the jobs by estimated cost, no data exchange between ranks (the
    reference scatters its job list over MPI ranks the same way, GetDistancesS2_mpi.py:58-65).
    Every rank computes the same partition from the same job list, so the shares are disjoint
    and cover every pending PD."""
    if world <= 1:
        return list(input_data)
    mine = shard([len(j[0]) for j in input_data], int(N), rank, world)
    return [input_data[i] for i in mine]


def world_from_env():
    """(rank, world size) of a torchrun / MPI-style launch, (0, 1) otherwise."""
    return int(os.environ.get('RANK', '0')), int(os.environ.get('WORLD_SIZE', '1'))


def run_jobs(jobs: list, stack_file: str, nStot: int, options: dict, progress=None,
             budget_bytes: Optional[int] = None, precision: Optional[str] = None,
             done_offset: int = 0, total: Optional[int] = None, writers: int = 4,
             image_dtype=np.float64, sh=None) -> None:
    """Run ``jobs`` ([ind, q, df, outFile, prD] each) in HBM-admitted GPU batches; the pickles
    and markers of a batch are written by ``writers`` threads while the next batch computes
    (``writers=0``: written in line, as the reference does).  Progress is reported per PD when
    its marker is queued."""
    import torch

    p = params_module()
    N = int(p.nPix)
    params = stage_params(p, FILTER_PAR, options, precision)
    stage = DistanceStage(params)
    if budget_bytes is None:
        free, _ = torch.cuda.mem_get_info(stage.device)
        budget_bytes = int(free * 0.6)
    counts = [int(np.asarray(j[0]).shape[0]) for j in jobs]
    done = done_offset
    total = total or len(jobs)
    writer = myio.AsyncWriter(writers) if writers > 0 else None
    mask = volume_mask(p, stage.device)
    try:
        for batch in admit_batches(counts, params, budget_bytes):
            done = _run_batch(stage, params, jobs, batch, stack_file, nStot, options, N, p,
                              writer, image_dtype, progress, done, total, sh, mask)
    finally:
        if writer is not None:
            writer.close()


def _run_batch(stage, params, jobs, batch, stack_file, nStot, options, N, p, writer,
               image_dtype, progress, done, total, sh=None, mask=None):
    """One HBM-admitted batch: read its images, run the stage, queue its pickles."""
    import torch
    pj = [PdJob(ind=np.asarray(jobs[i][0]), q=np.asarray(jobs[i][1], dtype=np.float64),
                df=np.asarray(jobs[i][2], dtype=np.float64), outFile=jobs[i][3],
                prD=jobs[i][4]) for i in batch]
    geoms = stage.geometry(pj, nStot)
    all_idx = np.concatenate([g.stack_index for g in geoms])
    imgs, compact, sh_c = load_images(stack_file, all_idx, N, options, sh)
    off = 0
    for g in geoms:
        g.stack_index = compact[off:off + g.stack_index.size]
        off += g.stack_index.size
    stack = torch.from_numpy(imgs).to(stage.device)
    results = stage.run(pj, stack, nStot, outputs=DEFAULT_OUTPUTS, geoms=geoms, sh=sh_c,
                        mask=mask)
    for job, geom, res in zip(pj, geoms, results):
        out = assemble(job, geom, res, N, options, msk2=res.get('msk2', 1),
                       image_dtype=image_dtype)
        marker = os.path.join(p.dist_prog, '%s' % job.prD)
        vals = [out[k] for k in OUTPUT_KEYS]
        if writer is not None:
            writer.submit(job.outFile, OUTPUT_KEYS, vals, marker)
        else:
            myio.fout1(job.outFile, OUTPUT_KEYS, vals)
            open(marker, 'a').close()
        done += 1
        if progress is not None:
            progress.emit(int((done / float(total)) * 100))
    del stack, results
    return done


def op(*argv):
    p = params_module()
    set_params.op(1)
    data = myio.fin1(p.tess_file)
    CG = data['CG']
    df = data['df']
    q = data['q']
    sh = data.get('sh')
    size = len(df)
    options = dict(verbose=False, avgOnly=False, visual=False, parallel=False,
                   relion_data=p.relion_data, thres=p.PDsizeThH)
    if p.relion_data is False:
        p.nPix = int(np.sqrt(os.path.getsize(p.img_stack_file) / (4 * p.num_part)))
        set_params.op(0)
    input_data = divide(CG, q, df, p.numberofJobs)
    rank, world = world_from_env()
    # one process per GPU: this rank's share of the pending PDs
    input_data = rank_jobs(input_data, int(p.nPix), rank, world)
    progress = argv[0] if argv else None
    offset = p.numberofJobs - len(input_data)
    if progress is not None:
        progress.emit(int((offset / float(max(p.numberofJobs, 1))) * 100))
    print("Processing {} projection directions.".format(len(input_data)))
    if input_data:
        # device bytes per admitted batch: p.gpu_budget_bytes when the configuration sets it,
        # else 60% of the free device memory
        run_jobs(input_data, p.img_stack_file, size, options, progress=progress,
                 budget_bytes=getattr(p, 'gpu_budget_bytes', None), done_offset=offset,
                 total=p.numberofJobs, sh=sh)
    set_params.op(0)
    return
