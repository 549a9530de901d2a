"""The multi-GPU rank path of the GetDistancesS2 replacement on CPU: two gloo ranks run
``GetDistancesS2.op`` (WORLD_SIZE / RANK from the environment, as torchrun sets them) on one
project after a partial resume.  Each rank must take a disjoint share of exactly the PDs without
a resume marker, and write only its own markers; the PDs finished before stay untouched.
The GPU work is replaced by a stub that writes each job's marker (the rank logic is the subject
here; the GPU stage has its own tests).  Reference: GetDistancesS2_mpi.py:58-65 (scatter of the
job list), GetDistancesS2.py:29-35 (resume markers)."""
import os
import socket

import numpy as np

N_PD = 9
DONE_BEFORE = (0, 3, 7)


def _free_port():
    s = socket.socket()
    s.bind(('127.0.0.1', 0))
    p = s.getsockname()[1]
    s.close()
    return p


def make_project(tmp):
    """A project with a tessellation file, a raw stack (16 px) and markers for DONE_BEFORE."""
    from manifoldem_python_gb300 import myio
    rng = np.random.default_rng(5)
    counts = rng.integers(5, 40, N_PD)
    num_part = int(counts.sum())
    CG, start = [], 0
    for n in counts:
        CG.append(np.arange(start, start + n, dtype=np.int64))
        start += n
    out = os.path.join(tmp, 'outputs_rk')
    os.makedirs(os.path.join(out, 'distances', 'progress'), exist_ok=True)
    q = rng.standard_normal((4, 2 * num_part))
    myio.fout2(os.path.join(out, 'selecGCs'), dict(CG=CG, q=q, df=np.full(2 * num_part, 1e4),
                                                   sh=(np.zeros(num_part), np.zeros(num_part))))
    np.zeros((num_part, 16, 16), np.float32).tofile(os.path.join(tmp, 'stack.bin'))
    for prD in DONE_BEFORE:
        open(os.path.join(out, 'distances', 'progress', str(prD)), 'a').close()
    return num_part


def _rank(rank, world, port, tmp, num_part, q):
    import torch.distributed as dist
    from manifoldem_python_gb300 import GetDistancesS2 as G
    from manifoldem_python_gb300 import p as mp
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    # each rank's own working directory: the parameter file set_params writes there is
    # per process, as on separate hosts
    cwd = os.path.join(tmp, 'rank%d' % rank)
    os.makedirs(cwd, exist_ok=True)
    os.chdir(cwd)
    mp.init()
    mp.user_dir, mp.proj_name = tmp, 'rk'
    mp.create_dir()
    mp.img_stack_file = os.path.join(tmp, 'stack.bin')
    mp.num_part, mp.numberofJobs, mp.relion_data = num_part, N_PD, False
    mine = []

    def stub_run_jobs(jobs, stack_file, nStot, options, **kw):
        for ind, qq, df, out_file, prD in jobs:
            assert int(mp.nPix) == 16 and len(ind) == qq.shape[1] == df.shape[0]
            mine.append(int(prD))
            open(os.path.join(mp.dist_prog, str(prD)), 'a').close()
    G.run_jobs = stub_run_jobs
    dist.barrier()                      # both ranks see the same resume state
    G.op()
    dist.barrier()
    q.put((rank, sorted(mine)))
    dist.destroy_process_group()


def test_two_ranks_share_exactly_the_pending_pds(tmp_path):
    import multiprocessing as mp
    tmp = str(tmp_path)
    num_part = make_project(tmp)
    prog = os.path.join(tmp, 'outputs_rk', 'distances', 'progress')
    before = {p: os.stat(os.path.join(prog, str(p))).st_mtime_ns for p in DONE_BEFORE}
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, tmp, num_part, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    shares = [r[1] for r in res]
    pending = sorted(set(range(N_PD)) - set(DONE_BEFORE))
    assert not set(shares[0]) & set(shares[1]), shares
    assert sorted(shares[0] + shares[1]) == pending, (shares, pending)
    assert all(shares)                                  # both ranks got work
    assert sorted(int(f) for f in os.listdir(prog)) == list(range(N_PD))
    for p, t in before.items():                         # finished PDs were not redone
        assert os.stat(os.path.join(prog, str(p))).st_mtime_ns == t


def test_rank_jobs_partition_is_the_lpt_shard():
    from manifoldem_python_gb300.GetDistancesS2 import rank_jobs
    from manifoldem_python_gb300.sharding import shard
    jobs = [[np.arange(n), None, None, 'f%d' % i, i] for i, n in
            enumerate([300, 20, 1200, 75, 640, 90, 2000])]
    assert rank_jobs(jobs, 128, 0, 1) == jobs
    parts = [rank_jobs(jobs, 128, r, 3) for r in range(3)]
    for r, part in enumerate(parts):
        assert [j[4] for j in part] == shard([len(j[0]) for j in jobs], 128, r, 3)
    assert sorted(j[4] for part in parts for j in part) == list(range(len(jobs)))
