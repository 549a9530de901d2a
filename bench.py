"""Benchmark of the GPU distance stage: all-PD CTF-distance pairs/s on one GB300.

Workload (default, --config config4): 800 projection directions (PDs) of 128x128 px images,
particles per PD log-normal (median 400, sigma 0.6, clipped to 100-3000), 10% of PDs made of
conjugate views, seeded synthetic data (no public dataset is named; the reference's demo stack is
absent).  One step = the whole distance stage for every PD (gather, normalisation, low-pass,
mask, two spline rotations, CTF, spectra, Wiener / phase-flip averages, imgAllIntensity, D),
i.e. ``mem_plan_execute`` over all 800 PDs.  Pickle writing is not part of a step.

Printed JSON line (rank 0):
  value     pairs/s with inputs resident in HBM (timed on the stream with CUDA events)
  e2e       the same through the C-ABI call with host buffers: pinned-host stack and per-image
            metadata copied in, D and the averages copied out, inside the timed region
  roofline  the dominant phase of a step, timed live with CUDA events
  cpu_baseline  the FP64 CPU port of the reference (oracle/) on a bounded sample of PDs,
            extrapolated to the whole workload by a fitted t(n) = a n + b n^2
``--impl reference`` times that CPU port alone (the reference itself is Python and cannot run on
the GPU host) on the same workload and prints the same line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

L2_BYTES = 129 * 1024 * 1024


def load_peaks():
    path = os.path.join(HERE, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return dict(hbm=d['hbm_gbs'], bf16=d['bf16_tflops'],
                    bf16_sust=d['bf16_tflops_sustained'], src='measured')
    return dict(hbm=6800.0, bf16=1900.0, bf16_sust=1700.0, src='fallback')


class ClockSampler:
    """nvidia-smi SM clock / throttle sampling while the timed region runs."""
    Q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,'
         'clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,'
         'clocks_event_reasons.sw_power_cap')

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ['nvidia-smi', '-i', str(self.gpu), '--query-gpu=' + self.Q,
                 '--format=csv,noheader,nounits', '-lms', '100'],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for ln in self.lines:
            f = [x.strip() for x in ln.split(',')]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower() == 'active':
                    reasons.add(nm)
        return {'sm_mhz': statistics.median(sm) if sm else None, 'sm_max_mhz': mx,
                'reasons': sorted(reasons), 'samples': len(sm)}


# ------------------------------------------------------------------------------- CPU side
def _oracle_pd(args):
    """One PD through the FP64 CPU port; returns (n, seconds)."""
    import numpy as _np
    from oracle import distance_oracle as O
    stack, ind, q, df, nStot, mic = args
    t0 = time.perf_counter()
    O.pd_op(ind, q, df, stack, nStot, **mic)
    return int(ind.shape[0]), time.perf_counter() - t0


def cpu_sample_tasks(ds, pds, mic, sizes=None):
    """Compact per-PD inputs (stack of the PD's images, indices remapped) for the CPU port;
    with `sizes`, sub-PDs made of the first sizes[i] images of PD pds[i]."""
    tasks = []
    stack_all = ds.stack
    for t, p in enumerate(pds):
        ind = np.asarray(ds.CG[p])
        if sizes is not None:
            ind = ind[:sizes[t]]
        conj = ind >= ds.num_part
        sidx = np.where(conj, ind - ds.num_part, ind)
        n = ind.size
        imgs = stack_all[sidx].cpu().numpy() if hasattr(stack_all, 'cpu') else stack_all[sidx]
        new_ind = np.arange(n) + np.where(conj, n, 0)
        tasks.append((imgs, new_ind, ds.q[:, ind], ds.df[ind], 2 * n, mic))
    return tasks


def _oracle_dm(task):
    """Worker: the FP64 restatement of DMembeddingII.op on one PD's D; (n, seconds, psi[:, :8])."""
    D, seed = task
    from oracle.dm_embedding import dm_embedding
    t0 = time.perf_counter()
    _, psi, _ = dm_embedding(D, seed=seed)
    return D.shape[0], time.perf_counter() - t0, psi[:, :8]


def dm_report(outs, counts, n_sample, cores):
    """Diffusion-map embedding (the stage's consumer, DMembeddingII.op) of a sample of the
    benchmark's own PDs: GPU op (manifoldem_python_gb300.DMembeddingII) wall time per PD
    against the FP64 CPU port on the host cores, and the largest top-8 subspace angle."""
    import multiprocessing as mp
    import torch
    from scipy.linalg import subspace_angles
    from manifoldem_python_gb300 import DMembeddingII
    cnt = np.asarray(counts)
    order = np.argsort(cnt, kind='stable')
    pick = sorted({int(order[int((q + 0.5) / n_sample * len(order))]) for q in range(n_sample)})
    d_off = np.concatenate([[0], np.cumsum(cnt.astype(np.int64) ** 2)])
    Ds = [outs['D'][d_off[p]:d_off[p + 1]].view(int(cnt[p]), int(cnt[p])) for p in pick]
    import scipy.optimize
    # warm-up on the smallest and the largest PD of the sample: the first eigen-decomposition
    # of the process, and the first of a larger size, load the solver's kernels (seconds)
    for D in (min(Ds, key=len), max(Ds, key=len)):
        np.random.seed(0)
        DMembeddingII.op(D, D.shape[0], 3, 60000)
    torch.cuda.synchronize()
    # count the tanh fits of each embedding (fergusonE.py:46-56 refits from random starts until
    # the parameters' standard errors sum to <= 100)
    fits = [0]
    curve_fit = scipy.optimize.curve_fit

    def counted(*a, **k):
        fits[0] += 1
        return curve_fit(*a, **k)
    gpu_psi, t_gpu, t_each, n_fits = [], 0.0, [], []
    scipy.optimize.curve_fit = counted
    try:
        for D in Ds:
            np.random.seed(0)
            fits[0] = 0
            t0 = time.perf_counter()
            psi = DMembeddingII.op(D, D.shape[0], 3, 60000)[1]
            dt = time.perf_counter() - t0
            t_gpu += dt
            t_each.append(round(1e3 * dt, 1))
            n_fits.append(fits[0])
            gpu_psi.append(psi[:, :8])
    finally:
        scipy.optimize.curve_fit = curve_fit
    host = [(D.cpu().numpy(), 0) for D in Ds]
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    os.environ.setdefault('OPENBLAS_NUM_THREADS', '1')
    t0 = time.perf_counter()
    with mp.get_context('spawn').Pool(processes=min(cores, len(host))) as pool:
        res = pool.map(_oracle_dm, host, chunksize=1)
    cpu_wall = time.perf_counter() - t0
    ang = max(float(np.max(subspace_angles(a, r[2]))) for a, r in zip(gpu_psi, res))
    return dict(pds=len(Ds), n=[int(cnt[p]) for p in pick],
                gpu_ms_per_pd=1e3 * t_gpu / len(Ds), gpu_ms_each=t_each, tanh_fits_each=n_fits,
                cpu_ms_per_pd_one_core=1e3 * float(np.mean([r[1] for r in res])),
                cpu_cores=min(cores, len(host)), cpu_wall_s=cpu_wall,
                max_top8_subspace_angle_rad=ang,
                method='GPU: csrc/dmap.cu sweep + kernel, torch.linalg.eigh, host tanh fit; '
                       'CPU: FP64 port of DMembeddingII/fergusonE/slaplacianonFly (oracle/)')


def _oracle_nlsa(task):
    """Worker: the FP64 restatement of NLSA.op (the reference's per-image Wiener loop) on one
    PD; (seconds, result)."""
    args, seed = task
    from oracle.nlsa_oracle import nlsa
    np.random.seed(seed)
    t0 = time.perf_counter()
    out = nlsa(*args)
    return time.perf_counter() - t0, out


def nlsa_report(ds, params, dev, cores, n_cpu_max=800):
    """NLSA stage (NLSA.op, the consumer of imgAll / CTF / D, reference modules/NLSA.py:23-158)
    on three of the benchmark's own PDs (smallest, median and largest image count): their
    imgAll, CTF and D from the distance stage, the images ordered along diffusion coordinate 0
    and ConOrder = floor(n / 50), as psiAnalysisParS2.op drives it.  GPU NLSA.op wall time per
    PD; the snapshot matrix (mem_nlsa_snapshots: spectra, Wiener denominators, banded
    correlation, inverse transforms) timed alone with CUDA events on the largest PD; the FP64
    CPU port timed on the host cores for the PDs with n <= n_cpu_max (one process per PD), and
    its largest differences from the GPU results."""
    import multiprocessing as mp
    import torch
    from manifoldem_python_gb300 import DMembeddingII, NLSA
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob
    counts = np.array([len(ind) for ind in ds.CG])
    order = np.argsort(counts, kind='stable')
    pick = list(dict.fromkeys([int(order[0]), int(order[len(order) // 2]), int(order[-1])]))
    stage = DistanceStage(params)
    jobs = [PdJob(ind=ds.CG[p].astype(np.int64), q=ds.q[:, ds.CG[p]], df=ds.df[ds.CG[p]])
            for p in pick]
    res = stage.run(jobs, ds.stack, ds.nStot, outputs=('D', 'img_all', 'ctf'))
    runs = []
    for r in res:
        D = np.asarray(r['D'], dtype=np.float64)
        n = D.shape[0]
        N = params.N
        np.random.seed(0)
        psi = DMembeddingII.op(D, n, 3, 60000)[1]
        P = np.argsort(psi[:, 0])
        c = n // 50
        par = dict(num=n, ConOrder=c, k=n - c, tune=3, nS=n, save=False, psiTrunc=8)
        runs.append((par, D[P][:, P], np.arange(n), P,
                     np.asarray(r['img_all'], dtype=np.float64),
                     np.array(1), np.asarray(r['ctf'], dtype=np.float64).reshape(n, N, N),
                     dict(outDir='', prD=0)))
    del res
    np.random.seed(1)
    NLSA.op(*runs[0])                                     # warm-up
    gpu_ms, outs = [], []
    for a in runs:
        np.random.seed(1)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        outs.append(NLSA.op(*a))
        torch.cuda.synchronize(dev)
        gpu_ms.append(1e3 * (time.perf_counter() - t0))
    # the snapshot matrix alone on the largest PD, device time
    big = runs[-1]
    n, c = big[0]['num'], big[0]['ConOrder']
    g = NLSA._Gpu(dev)
    images = g.tensor(big[4], torch.float32, big[3])
    ctf = g.tensor(big[6], torch.float32, big[3])
    snap_ms, snap_tflops = nlsa_snapshot_timing(images, ctf, n, c, dev, 5)
    del images, ctf
    # CPU port on the smaller PDs
    cpu = [i for i, a in enumerate(runs) if a[0]['num'] <= n_cpu_max]
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    os.environ.setdefault('OPENBLAS_NUM_THREADS', '1')
    cpu_s, err = [], {}
    if cpu:
        with mp.get_context('spawn').Pool(processes=min(cores, len(cpu))) as pool:
            got = pool.map(_oracle_nlsa, [(runs[i], 1) for i in cpu], chunksize=1)
        for i, (sec, ref) in zip(cpu, got):
            cpu_s.append(sec)
            o = outs[i]
            flip = np.sum(o[2][:, 2] * ref[2][:, 2]) < 0
            tau_ref = (1 - ref[7]) if flip else ref[7]
            for key, v in (('IMGT_max_abs', np.abs(o[0] - ref[0]).max()),
                           ('sdiag_max_rel', (np.abs(o[4] - ref[4]) / ref[4]).max()),
                           ('tau_max_abs', np.abs(o[7] - tau_ref).max())):
                err[key] = max(err.get(key, 0.0), float(v))
    return dict(pds=len(runs), n=[int(a[0]['num']) for a in runs],
                con_order=[int(a[0]['ConOrder']) for a in runs],
                gpu_ms_per_pd=gpu_ms,
                snapshots_ms_largest=snap_ms,
                snapshots_correlation_tflops=snap_tflops,
                cpu_n=[int(runs[i][0]['num']) for i in cpu],
                cpu_ms_per_pd_one_core=[1e3 * t for t in cpu_s],
                gpu_vs_cpu_port=err,
                method='GPU: csrc/nlsa.cu (ConD, Wiener snapshot correlation), GPU diffusion '
                       'maps, torch GEMMs, host fit; CPU: FP64 port of NLSA.op with the '
                       "reference's per-image FFT loop (oracle/nlsa_oracle.py)")


def nlsa_snapshot_timing(images, ctf, n, c, dev, reps):
    """Device time (CUDA events on the launching stream) of mem_nlsa_snapshots for one PD:
    ms per call and the correlation's algorithmic TFLOP/s (4 c (n - c) K 8 flops, K half-plane
    frequencies, 8 modes)."""
    import torch
    from manifoldem_python_gb300 import NLSA
    g = NLSA._Gpu(dev)
    N = int(images.shape[-1])
    mu_psi = np.random.default_rng(0).standard_normal((n - c, 8)) / n
    NLSA.snapshots(g, images, ctf, mu_psi, np.array(1), c)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(g.stream)
    for _ in range(reps):
        NLSA.snapshots(g, images, ctf, mu_psi, np.array(1), c)
    e1.record(g.stream)
    torch.cuda.synchronize(dev)
    ms = e0.elapsed_time(e1) / reps
    flop = 4.0 * c * (n - c) * N * (N // 2 + 1) * 8
    return ms, flop / (ms * 1e-3) / 1e12


def nlsa_snapshot_case(ds, params, dev, reps):
    """The snapshot matrix alone for the PD of ds (its distance-stage images and CTFs)."""
    import torch
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob
    ind = ds.CG[0].astype(np.int64)
    r = DistanceStage(params).run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack,
                                  ds.nStot, outputs=('img_all', 'ctf'))[0]
    n, N = len(ind), params.N
    images = torch.as_tensor(np.asarray(r['img_all'], dtype=np.float32)).to(dev)
    ctf = torch.as_tensor(np.asarray(r['ctf'], dtype=np.float32).reshape(n, N, N)).to(dev)
    c = n // 50
    ms, tflops = nlsa_snapshot_timing(images, ctf, n, c, dev, reps)
    return dict(n=n, con_order=c, snapshots_ms=ms, snapshots_correlation_tflops=tflops)


def run_cpu_tasks(tasks, cores):
    import multiprocessing as mp
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    os.environ.setdefault('OPENBLAS_NUM_THREADS', '1')
    os.environ.setdefault('MKL_NUM_THREADS', '1')
    ctx = mp.get_context('spawn')
    t0 = time.perf_counter()
    with ctx.Pool(processes=cores) as pool:
        res = pool.map(_oracle_pd, tasks, chunksize=1)
    return res, time.perf_counter() - t0


def extrapolate_pairs_per_s(res, wall, counts, cores):
    """Fit per-PD CPU time t(n) = a n + b n^2 on the sample and predict the wall time of the
    whole workload on `cores` workers (perfect packing, but never below the largest PD's own
    time); returns pairs/s."""
    n = np.array([r[0] for r in res], dtype=np.float64)
    t = np.array([r[1] for r in res], dtype=np.float64)
    A = np.vstack([n, n * n]).T
    coef, *_ = np.linalg.lstsq(A, t, rcond=None)
    a, b = max(coef[0], 0.0), max(coef[1], 0.0)
    if a == 0 and b == 0:
        a = float(np.sum(t) / np.sum(n))
    counts = np.asarray(counts, dtype=np.float64)
    t_pd = a * counts + b * counts * counts
    # one worker per PD, as the reference's pool runs it: no PD finishes faster than alone
    total_t = max(float(np.sum(t_pd)) / cores, float(np.max(t_pd)))
    pairs = float(np.sum(counts * (counts - 1) / 2))
    return pairs / total_t, dict(a=a, b=b, sample_pairs_per_s=float(
        np.sum(n * (n - 1) / 2) / wall))


def choose_sample(counts, cores, max_n):
    """PDs at evenly spaced quantiles of the size distribution, capped at max_n particles."""
    order = np.argsort(counts, kind='stable')
    k = cores
    qs = (np.arange(k) + 0.5) / k
    pick = []
    for qv in qs:
        p = int(order[min(len(order) - 1, int(qv * len(order)))])
        if counts[p] <= max_n and p not in pick:
            pick.append(p)
    return pick


# ------------------------------------------------------------------------------- GPU side
def workload_string(config_name, cfg, counts):
    """The workload named in `config` (the same for the GPU arm and the reference arm)."""
    counts = np.asarray(counts, dtype=np.int64)
    return '%s: %d PDs, %dx%d px, n~lognormal(median %d), %d images, %d pairs per GPU' % (
        config_name, len(counts), cfg.N, cfg.N, cfg.n_median, int(counts.sum()),
        int((counts * (counts - 1) // 2).sum()))


def kernels_per_execute(outputs, avg_only, N, counts=None, classes=None):
    """Kernels of this library one mem_plan_execute launches (cuFFT kernels excluded).
    N = 32, 64, 128 (shared-memory FFTs): lowpass_table, lowpass_fft, rot_const, rotate,
    spectrum_fft, qfix, pd_sums, pd_finalize, features, [inverse_fft + avg_store],
    [inverse_fft + intensity], [contraction: one launch per size class that has PDs].  Other N
    (cuFFT transforms): lowpass_table, gather_normalize, lowpass_apply, rot_const, rotate,
    qfix, pd_sums, pd_finalize, features, [avg_store], [intensity], [contraction]."""
    smem = N in (32, 64, 128) and os.environ.get('MEM_SMEM_FFT', '1') != '0'
    # N = 64, 128: lowpass_fft, rotate and spectrum_fft are one image_stage kernel
    fused = smem and N in (64, 128) and os.environ.get('MEM_FUSED_IMAGE', '0') == '1'
    k = 7 if fused else 9
    if 'img_avg' in outputs or 'img_avg_flip' in outputs:
        k += 2 if smem else 1
    if smem and ('img_all_intensity' in outputs or 'img_all_flip' in outputs):
        k += 1
    if 'img_all_intensity' in outputs:
        k += 1
    if 'D' in outputs and not avg_only:
        if counts is not None and classes:
            used = set()
            for n in counts:
                for i, c in enumerate(classes):
                    if n <= c['max_n'] or i == len(classes) - 1:
                        used.add(i)
                        break
            k += len(used)
        else:
            k += 1
    return k


def traffic_from_profiles(kernel_tag, workload):
    """Per-launch DRAM bytes of the dominant kernel from the committed ncu summary, if any."""
    return profile_number(kernel_tag, workload, 'traffic_bytes_per_full_launch')


def profile_number(kernel_tag, workload, key):
    """A `key: value` figure from the committed ncu summary of the kernel, if any (the last
    one: summaries append the capture of each newer build at the end)."""
    path = os.path.join(HERE, 'profiles', '%s_%s.md' % (kernel_tag, workload))
    if not os.path.exists(path):
        return None
    found = re.findall(key + r':\s*([0-9.eE+]+)', open(path).read())
    return float(found[-1]) if found else None


def shared_memory_roofline(r, args, phase):
    """The shared-memory bound of a phase whose kernel is limited by shared-memory wavefronts
    (the rotation): wavefronts per image from the committed ncu summary of the kernel x the
    images / the phase's live time, against one wavefront per SM per clock at the SM clock
    sampled during the timed region."""
    per_img = profile_number(phase, args.config, 'shared_wavefronts_per_image')
    mhz = (r.get('clocks') or {}).get('sm_mhz')
    if not per_img or not mhz:
        return None
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ach = per_img * r['n_images'] / (r['phases'][phase] * 1e-3)
    peak = sms * mhz * 1e6
    return dict(achieved=ach, peak=peak, unit='wavefronts/s', frac=ach / peak,
                wavefronts_per_image=per_img,
                source='profiles/%s_%s.md (ncu l1tex__data_pipe_lsu_wavefronts_mem_shared.sum '
                       'per image); peak = %d SMs x 1 wavefront per clock x %.0f MHz'
                       % (phase, args.config, sms, mhz))


def time_form(plan, stack, sidx, flip, psi, dfd, outs, args, world, dev, flush):
    """Device time of one step of ``plan`` (CUDA graph replay unless --no-graph): W untimed
    warm-up steps, then exactly K steps timed with CUDA events on the launching stream between
    a barrier and a synchronize; when the stack is smaller than twice L2 every step is timed
    alone after a write of a buffer larger than L2.  Returns (ms per step, max over ranks;
    per-phase ms of one extra step timed by the library's phase events; the graph)."""
    import ctypes
    import torch
    stream = torch.cuda.current_stream(dev)
    graph = None
    if args.graph:
        try:
            graph = plan.capture(stack, sidx, flip, psi, dfd, outs)
        except Exception as exc:           # report, and time direct launches instead
            print('graph capture failed: %s' % exc, file=sys.stderr)
            graph = None

    def step():
        if graph is not None:
            graph.replay()
        else:
            plan.execute(stack, sidx, flip, psi, dfd, outs, stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    plan.device_status()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    scrub = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=dev) if flush else None
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps if flush else 1)]
    if flush:
        for e0, e1 in ev:
            scrub.fill_(1.0)
            e0.record(stream)
            step()
            e1.record(stream)
    else:
        ev[0][0].record(stream)
        for _ in range(args.steps):
            step()
        ev[0][1].record(stream)
    torch.cuda.synchronize(dev)
    ms = sum(e0.elapsed_time(e1) for e0, e1 in ev) / args.steps
    del scrub
    if world > 1:
        t = torch.tensor([ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    plan.device_status()
    # live phase timing of one more step (CUDA events between the phases)
    lib = plan.lib
    lib.mem_plan_set_timing(plan.handle, 1)
    plan.execute(stack, sidx, flip, psi, dfd, outs, stream)
    phase_ms = (ctypes.c_float * 9)()
    lib.mem_plan_phase_times(plan.handle, phase_ms, 9)
    lib.mem_plan_set_timing(plan.handle, 0)
    phases = {lib.mem_phase_name(i).decode(): float(phase_ms[i]) for i in range(9)}
    return ms, phases, graph


def run_gpu(args, rank, world):
    import torch
    from manifoldem_python_gb300.pipeline import Plan, StageParams
    from manifoldem_python_gb300.geometry import pd_geometry
    from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
    import dataclasses

    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    if args.n_pd:
        cfg = dataclasses.replace(cfg, n_pd=args.n_pd)
    cfg = dataclasses.replace(cfg, seed=cfg.seed + 1000 * rank)
    t0 = time.time()
    ds = make_dataset(cfg, device=dev)
    torch.cuda.synchronize(dev)
    t_gen = time.time() - t0
    geoms = [pd_geometry(np.asarray(ind), ds.q[:, ind], ds.nStot) for ind in ds.CG]
    counts = [int(len(ind)) for ind in ds.CG]
    params = StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                         AmpContrast=cfg.ampc, precision=args.precision)
    # the contraction schedule per PD size class: measured by the autotuner (cached per GPU and
    # box size), outside the timed region
    tuned, t_tune = None, 0.0
    if args.autotune and params.precision == 'bf16x3':
        from manifoldem_python_gb300 import autotune
        t0 = time.time()
        tuned = autotune.tune(params, dev, force=args.autotune == 'force')
        t_tune = time.time() - t0
    plan = Plan(params, counts, [g.psi_p for g in geoms], dev)
    plan_classes = plan.contraction
    outputs = tuple(args.outputs.split(','))
    outs = plan.allocate_outputs(outputs)
    sidx_h = np.concatenate([g.stack_index for g in geoms])
    flip_h = np.concatenate([g.flip for g in geoms])
    psi_h = np.concatenate([g.psi_rad for g in geoms])
    df_h = np.concatenate([ds.df[ind] for ind in ds.CG]).astype(np.float64)
    sidx = torch.from_numpy(sidx_h).to(dev)
    flip = torch.from_numpy(flip_h).to(dev)
    psi = torch.from_numpy(psi_h).to(dev)
    dfd = torch.from_numpy(df_h).to(dev)
    stack = ds.stack
    stream = torch.cuda.current_stream(dev)
    flush = stack.numel() * stack.element_size() < 2 * L2_BYTES
    with ClockSampler(dev.index) as clk:
        ms, phases, graph = time_form(plan, stack, sidx, flip, psi, dfd, outs, args, world, dev,
                                      flush)
        graph_used = graph is not None
        # the other contraction form(s) on the same PDs, images and outputs (the metric compares
        # split-BF16 with the plain FP32 form): a plan of its own, timed the same way
        forms = {args.precision: dict(ms_per_step=ms, contraction_ms=phases['contraction'],
                                      pairs_per_s=plan.n_pairs / (ms * 1e-3), phases_ms=phases)}
        for other in [f for f in args.forms.split(',') if f and f != args.precision]:
            oparams = dataclasses.replace(params, precision=other)
            oplan = Plan(oparams, counts, [g.psi_p for g in geoms], dev)
            oms, ophases, ograph = time_form(oplan, stack, sidx, flip, psi, dfd, outs, args,
                                             world, dev, flush)
            forms[other] = dict(ms_per_step=oms, contraction_ms=ophases['contraction'],
                                pairs_per_s=oplan.n_pairs / (oms * 1e-3), phases_ms=ophases)
            del ograph, oplan
            torch.cuda.synchronize(dev)
            torch.cuda.empty_cache()
    del graph
    if len(forms) > 1:      # the outputs hold the benchmarked form's results again
        plan.execute(stack, sidx, flip, psi, dfd, outs, stream)
        torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()

    dm = None
    if not args.no_dm and 'D' in outs and rank == 0:
        dm = dm_report(outs, counts, args.dm_pds, os.cpu_count() or 1)
    nlsa = None
    if not args.no_nlsa and rank == 0:
        nlsa = nlsa_report(ds, params, dev, os.cpu_count() or 1)

    # end to end through the public API with host buffers
    e2e = None
    n_pairs, n_images = plan.n_pairs, plan.n_images
    if not args.no_e2e:
        pin = True
        try:
            stack_h = torch.empty(stack.shape, dtype=stack.dtype, pin_memory=True)
        except RuntimeError:
            stack_h, pin = torch.empty(stack.shape, dtype=stack.dtype), False
        stack_h.copy_(stack)
        res_names = tuple(k for k in ('D', 'img_avg', 'img_avg_flip', 'img_all_intensity')
                          if k in outs)
        if args.e2e_mode == 'streamed' and pin:
            # the stack stays in pinned host memory; per group of PDs the load kernel reads its
            # images over the host link while the previous group computes (StreamedStage)
            from manifoldem_python_gb300.pipeline import StreamedStage
            del outs, plan
            ds.stack = stack_h          # later host-side uses read the pinned copy
            del stack
            torch.cuda.empty_cache()
            st = StreamedStage(params, counts, [g.psi_p for g in geoms], n_groups=args.e2e_groups,
                               outputs=res_names, device=dev, ramp=args.e2e_ramp,
                               ramp_steps=args.e2e_ramp_steps, dma=args.e2e_dma)
            st.set_metadata(sidx_h, flip_h, psi_h, df_h)
            h2d = st.image_bytes(stack_h.shape[0]) + st.metadata_bytes()
            d2h = st.result_bytes()

            def e2e_step():
                st.run(stack_h)
            staged = st.staged_groups()
            how = ('%d of them staged by the copy engines (contiguous stack ranges), the rest '
                   'read by the load kernel over the host link' % staged) if staged else \
                'read by the load kernel over the host link'
            mode = 'streamed: stack in pinned host memory, %d PD groups (image counts %s), %s, ' \
                   'on load / compute / copy streams' % (
                       len(st.groups), [int(sum(counts[i] for i in g)) for g in st.groups], how)
        else:
            meta_h = [torch.from_numpy(x).pin_memory() if pin else torch.from_numpy(x)
                      for x in (sidx_h, flip_h, psi_h, df_h)]
            res_h = {k: torch.empty(outs[k].shape, dtype=outs[k].dtype, pin_memory=pin)
                     for k in res_names}
            h2d = stack_h.numel() * 4 + sum(m.numel() * m.element_size() for m in meta_h)
            d2h = sum(v.numel() * v.element_size() for v in res_h.values())

            def e2e_step():
                stack.copy_(stack_h, non_blocking=True)
                for dst, src in zip((sidx, flip, psi, dfd), meta_h):
                    dst.copy_(src, non_blocking=True)
                plan.execute(stack, sidx, flip, psi, dfd, outs, stream)
                for k in res_names:
                    res_h[k].copy_(outs[k], non_blocking=True)
            mode = 'copy: stack copied host to device, then one execute'

        e2e_step()
        torch.cuda.synchronize(dev)
        k_e2e = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(k_e2e):
            e2e_step()
        torch.cuda.synchronize(dev)
        e2e_ms = (time.perf_counter() - t0) * 1000 / k_e2e
        if world > 1:
            t = torch.tensor([e2e_ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            e2e_ms = float(t.item())
        e2e = dict(ms=e2e_ms, h2d=int(h2d), d2h=int(d2h), pinned=pin, mode=mode)
        del stack_h
    return dict(ms=ms, pairs=n_pairs, n_images=n_images, counts=counts,
                graph=graph_used, l2_flush=flush, forms=forms, tuned=tuned, t_tune=t_tune,
                phases=phases, clocks=clk.summary(), t_gen=t_gen, e2e=e2e, ds=ds, cfg=cfg, dm=dm,
                nlsa=nlsa,
                kernels=kernels_per_execute(outputs, False, cfg.N, counts, plan_classes),
                outputs=outputs)


def run_gpu_batched(args, rank, world, budget_frac=0.8):
    """A workload larger than one device (config5: 1500 PDs of 250 px, about 2.2 million
    images): the PDs are admitted into batches by the device-memory budget
    (pipeline.admit_batches, as GetDistancesS2.run_jobs does), each batch's images are rendered
    on the device outside the timed region, and each batch is timed like a single-plan
    workload (graph replay, W warm-up and K timed steps); a step of the workload is the sum of
    its batches' steps."""
    import dataclasses
    import torch
    from manifoldem_python_gb300.geometry import pd_geometry
    from manifoldem_python_gb300.pipeline import Plan, StageParams, admit_batches
    from manifoldem_python_gb300.synthetic import CONFIGS, make_geometry, render_pds
    dev = torch.device('cuda', int(os.environ.get('LOCAL_RANK', 0)))
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    if args.n_pd:
        cfg = dataclasses.replace(cfg, n_pd=args.n_pd)
    cfg = dataclasses.replace(cfg, seed=cfg.seed + 1000 * rank)
    t0 = time.time()
    geo = make_geometry(cfg)
    counts = [int(len(ind)) for ind in geo['CG']]
    params = StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                         AmpContrast=cfg.ampc, precision=args.precision)
    tuned, t_tune = None, 0.0
    if args.autotune and params.precision == 'bf16x3':
        from manifoldem_python_gb300 import autotune
        t1 = time.time()
        tuned = autotune.tune(params, dev, force=args.autotune == 'force')
        t_tune = time.time() - t1
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info(dev)
    batches = admit_batches(counts, params, int(free * budget_frac))
    outputs = tuple(args.outputs.split(','))
    total_ms, pairs, n_images, n_kern, t_render = 0.0, 0, 0, 0, 0.0
    phases, per_batch = {}, []
    with ClockSampler(dev.index) as clk:
        for b in batches:
            t1 = time.time()
            ds = render_pds(cfg, geo, b, device=dev)
            torch.cuda.synchronize(dev)
            t_render += time.time() - t1
            geoms = [pd_geometry(np.asarray(ind), ds.q[:, ind], ds.nStot) for ind in ds.CG]
            bc = [int(len(ind)) for ind in ds.CG]
            plan = Plan(params, bc, [g.psi_p for g in geoms], dev)
            outs = plan.allocate_outputs(outputs)
            t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
            sidx = t(np.concatenate([g.stack_index for g in geoms]))
            flip = t(np.concatenate([g.flip for g in geoms]))
            psi = t(np.concatenate([g.psi_rad for g in geoms]))
            dfd = t(np.concatenate([ds.df[ind] for ind in ds.CG]).astype(np.float64))
            ms, ph, graph = time_form(plan, ds.stack, sidx, flip, psi, dfd, outs, args, world,
                                      dev, False)
            total_ms += ms
            pairs += plan.n_pairs
            n_images += plan.n_images
            n_kern += kernels_per_execute(outputs, False, cfg.N, bc, plan.contraction)
            for k, v in ph.items():
                phases[k] = phases.get(k, 0.0) + v
            per_batch.append(dict(pds=len(b), images=plan.n_images, pairs=plan.n_pairs,
                                  ms=ms, contraction_ms=ph['contraction']))
            del graph, plan, outs, ds, sidx, flip, psi, dfd
            torch.cuda.synchronize(dev)
            torch.cuda.empty_cache()
    forms = {args.precision: dict(ms_per_step=total_ms, contraction_ms=phases['contraction'],
                                  pairs_per_s=pairs / (total_ms * 1e-3), phases_ms=phases)}
    # one PD of the workload, rendered alone, for the precision report
    small = int(np.argmin(counts))
    ds = render_pds(cfg, geo, [small], device=dev)
    return dict(ms=total_ms, pairs=pairs, n_images=n_images, counts=counts, graph=args.graph,
                l2_flush=False, forms=forms, tuned=tuned, t_tune=t_tune, phases=phases,
                clocks=clk.summary(), t_gen=time.time() - t0, e2e=None, ds=ds, cfg=cfg,
                dm=None, nlsa=None, kernels=n_kern, outputs=outputs,
                precision_counts=[counts[small]],
                batches=dict(count=len(batches), budget_bytes=int(free * budget_frac),
                             render_s=t_render, per_batch=per_batch),
                stack_gb=sum(counts) * cfg.N * cfg.N * 4 / 1e9)


def roofline(r, args):
    peaks = load_peaks()
    ph = r['phases']
    dom = max(ph, key=ph.get)
    cfg = r['cfg']
    N = cfg.N
    K = 4 * N * (N // 2 + 1)
    if dom == 'contraction':
        flops = 2.0 * K * r['pairs']
        ach = flops / (ph[dom] * 1e-3) / 1e12
        peak = peaks['bf16_sust']
        return dict(phase=dom, bound='tensor', achieved=ach, peak=peak, unit='TFLOP/s',
                    frac=ach / peak, traffic=traffic_from_profiles('contraction_' + args.precision,
                                                                   args.config),
                    peak_source=peaks['src'] + ' bf16 sustained', algorithmic_flops=flops)
    # image-side phases: algorithmic bytes per image of the phase
    NN, Kc = N * N, N * (N // 2 + 1)
    per_img = {'gather': 2 * 4 * NN, 'lowpass': 2 * (4 * NN + 8 * Kc), 'rotate': 2 * 4 * NN,
               'spectrum': 4 * NN + 8 * Kc, 'sums': 8 * Kc, 'features': 8 * Kc + 16 * Kc + 8 * Kc,
               'averages': 0, 'flip': 8 * Kc + 4 * NN, }.get(dom, 4 * NN)
    kernel = dom
    if dom == 'lowpass' and ph.get('rotate', 0.0) < 1e-3 * ph['lowpass']:
        # the fused image kernel (lowpass, rotate and spectrum phases in one launch): reads the
        # raw image once and writes its half-plane spectrum once
        per_img = 4 * NN + 8 * Kc
        kernel = 'image_stage'
    b = per_img * r['n_images']
    ach = b / (ph[dom] * 1e-3) / 1e9
    return dict(phase=kernel, bound='hbm', achieved=ach, peak=peaks['hbm'], unit='GB/s',
                frac=ach / peaks['hbm'], traffic=traffic_from_profiles(kernel, args.config),
                peak_source=peaks['src'] + ' hbm', algorithmic_bytes=b)


def precision_report(args, ds, counts, cfg, precision):
    """D of one sample PD (about 150 images) in the benchmarked form against (a) an FP64
    contraction of the GPU's own spectra and exact CTFs, (b) the full FP64 CPU oracle on the
    same images, and the largest principal angle between the top-8 diffusion-map coordinates
    of the GPU D and of the oracle D (DMembeddingII restatement, k = n, tune 3)."""
    import torch
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    from oracle import distance_oracle as O
    from oracle.dm_embedding import top8_subspace_angle
    cnt = np.asarray(counts)
    p = int(np.argmin(np.abs(cnt - 150)))
    ind = np.asarray(ds.CG[p])[:150]          # a sub-PD when every PD is large
    stage = DistanceStage(StageParams(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                      AmpContrast=cfg.ampc, precision=precision))
    res = stage.run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack, ds.nStot,
                    outputs=('D', 'spectrum'))[0]
    N = cfg.N
    F = res['spectrum'][..., 0].astype(np.float64) + 1j * res['spectrum'][..., 1]
    Q = O.create_grid(N)
    C = np.stack([np.fft.ifftshift(O.ctf_cryo_frank(Q / (2 * cfg.pix), cfg.cs, d, cfg.kv,
                                                    np.inf, cfg.ampc))[:, :N // 2 + 1]
                  for d in ds.df[ind]])
    D64 = O.distances_from_half_plane(C, F, N)
    np.fill_diagonal(D64, 0)
    D = res['D']
    task = cpu_sample_tasks(ds, [p], dict(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                          AmpContrast=cfg.ampc), sizes=[ind.size])[0]
    ref = O.pd_op(task[1], task[2], task[3], task[0], task[4], N=N, pix_size=cfg.pix, Cs=cfg.cs,
                  EkV=cfg.kv, AmpContrast=cfg.ampc)['D']
    np.fill_diagonal(ref, 0)
    rel = lambda a, b: float(np.abs(a - b).max() / np.abs(b).max())
    return dict(pd=p, n=int(ind.size), form=precision,
                max_rel_err_vs_fp64_contraction=rel(D, D64),
                max_rel_err_vs_fp64_oracle=rel(D, ref),
                dm_top8_subspace_angle_rad=top8_subspace_angle(D, ref))


def fullsize_precision(ds, cfg, dev, pd=0):
    """D of one whole PD of the workload (config3: 4000 images of 192 px, 5% near-duplicates) in
    the split-BF16 form against an FP64 contraction of the GPU's own spectra with exact FP64
    CTFs, computed on the device in float64: normwise error, the error scaled by each pair's
    cross-norm term S_ij (the scale below which the GEMM form cancels), the elementwise relative
    error on the near-duplicate pairs, and the largest principal angle between the top-8
    diffusion-map coordinates (DMembeddingII.op, k = n, tune 3) of the two matrices."""
    import torch
    from scipy.linalg import subspace_angles
    from manifoldem_python_gb300 import DMembeddingII
    from manifoldem_python_gb300.pipeline import DistanceStage, PdJob, StageParams
    ind = np.asarray(ds.CG[pd])
    n, N = int(ind.size), cfg.N
    stage = DistanceStage(StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv,
                                      AmpContrast=cfg.ampc, precision='bf16x3'), device=dev)
    res = stage.run([PdJob(ind=ind, q=ds.q[:, ind], df=ds.df[ind])], ds.stack, ds.nStot,
                    outputs=('D', 'spectrum'), to_host=False)[0]
    f64 = torch.float64
    F = torch.view_as_complex(res['spectrum'].contiguous()).to(torch.complex128).reshape(n, -1)
    Nh = N // 2 + 1
    ka = torch.arange(N, device=dev)
    fa = torch.minimum(ka, N - ka).to(f64)
    kb = torch.arange(Nh, device=dev, dtype=f64)
    k2 = ((fa[:, None] ** 2 + kb[None, :] ** 2) / (N * cfg.pix) ** 2).reshape(-1)
    lam = 12.3986 / math.sqrt((2 * 511.0 + cfg.kv) * cfg.kv)
    dfd = torch.as_tensor(np.asarray(ds.df[ind], dtype=np.float64), device=dev)
    wr = (0.5 * math.pi * cfg.cs * 1e7 * lam ** 3 * k2[None, :] - math.pi * lam * dfd[:, None]) \
        * k2[None, :]
    C = torch.sin(wr) - cfg.ampc * torch.cos(wr)                  # ctemh_cryoFrank, no envelope
    w = torch.full((N, Nh), 2.0, device=dev, dtype=f64)
    w[:, 0] = 1.0
    if N % 2 == 0:
        w[:, -1] = 1.0
    w = w.reshape(-1)
    a = (w[None, :] * F.abs() ** 2)                                 # n x Kc
    A = a @ (C ** 2).T                                              # A[i, j] = sum w |F_i|^2 C_j^2
    H = torch.sqrt(w)[None, :] * C * F
    G = (H @ H.conj().T).real
    S = A + A.T
    D64 = S - 2 * G
    D64.fill_diagonal_(0.0)
    D = res['D']
    off = ~torch.eye(n, dtype=torch.bool, device=dev)
    dd = (D - D64).abs()
    rep = dict(pd=pd, n=n, form='bf16x3',
               max_rel_err_vs_fp64_contraction=float(dd.max() / D64.abs().max()),
               max_err_scaled_by_S=float((dd[off] / S[off]).max()))
    dup = np.asarray(ds.near_dup_of)
    pos = {int(g): i for i, g in enumerate(np.where(ind >= ds.num_part, ind - ds.num_part, ind))}
    pairs = [(pos[int(d)], pos[int(s_)]) for d, s_ in enumerate(dup)
             if s_ >= 0 and int(d) in pos and int(s_) in pos]
    if pairs:
        ii = torch.as_tensor([p[0] for p in pairs], device=dev)
        jj = torch.as_tensor([p[1] for p in pairs], device=dev)
        rel_el = (D[ii, jj] - D64[ii, jj]).abs() / D64[ii, jj].abs()
        rep.update(near_duplicate_pairs=len(pairs),
                   near_duplicate_max_elementwise_rel_err=float(rel_el.max()),
                   near_duplicate_median_elementwise_rel_err=float(rel_el.median()),
                   near_duplicate_D_over_S=float((D64[ii, jj] / S[ii, jj]).median()))
    del A, G, H, S, F, a, C
    Dh, D64h = D.cpu().numpy(), D64.cpu().numpy()
    t0 = time.time()
    np.random.seed(0)
    pa = DMembeddingII.op(Dh, n, 3, 60000)[1]
    np.random.seed(0)
    pb = DMembeddingII.op(D64h, n, 3, 60000)[1]
    rep['dm_top8_subspace_angle_rad'] = float(np.max(subspace_angles(pa[:, :8], pb[:, :8])))
    rep['dm_seconds'] = time.time() - t0
    rep['method'] = ('FP64 D of the GPU spectra and exact CTFs by float64 GEMMs on the device '
                     '(A + A^T - 2 Re(H H^H)); diffusion maps by the GPU DMembeddingII.op')
    return rep


def dropin_io_report(ds, cfg, n_pd=20, workdir=None):
    """The drop-in driver's real end-to-end cost (GetDistancesS2.run_jobs, reference
    GetDistancesS2.py:94-120 with myio.fout1, myio.py:38-51): the first n_pd PDs of the
    workload from a SPIDER stack file on disk to one 19-key pickle and resume marker per PD, in
    three modes -- float64 per-image arrays written in line (the reference's format and order),
    float64 with four writer threads overlapping the GPU batches, and the float32 opt-in with
    four writers.  Reports seconds, bytes written and GB/s to disk beside the GPU stage time."""
    import shutil
    import tempfile
    from manifoldem_python_gb300 import GetDistancesS2 as G
    from manifoldem_python_gb300 import p as mp
    base = tempfile.mkdtemp(prefix='dropin_io_', dir=workdir)
    try:
        pds = list(range(min(n_pd, len(ds.CG))))
        # a stack file holding only these PDs' particles, job indices remapped to it (conjugate
        # views stay above the new particle count)
        npart = ds.num_part
        phys = [np.where(ds.CG[i] >= npart, ds.CG[i] - npart, ds.CG[i]) for i in pds]
        keep = np.unique(np.concatenate(phys))
        remap = np.full(npart, -1, dtype=np.int64)
        remap[keep] = np.arange(keep.size)
        inds = [remap[ph] + np.where(ds.CG[i] >= npart, keep.size, 0)
                for i, ph in zip(pds, phys)]
        stack_file = os.path.join(base, 'stack.bin')
        sel = ds.stack[keep] if hasattr(ds.stack, 'cpu') else np.asarray(ds.stack)[keep]
        host = sel.cpu().numpy() if hasattr(sel, 'cpu') else np.asarray(sel)
        host.astype(np.float32).tofile(stack_file)
        nStot = 2 * int(keep.size)
        mp.init()
        mp.nPix, mp.pix_size, mp.Cs, mp.EkV, mp.AmpContrast = cfg.N, cfg.pix, cfg.cs, cfg.kv, \
            cfg.ampc
        options = dict(verbose=False, avgOnly=False, visual=False, parallel=False,
                       relion_data=False, thres=6000)
        jobs_of = lambda d: [[ind, ds.q[:, ds.CG[i]], ds.df[ds.CG[i]],
                              os.path.join(d, 'IMGs_prD_%d' % i), i] for i, ind in zip(pds, inds)]
        n_img = int(sum(len(ds.CG[i]) for i in pds))
        out = dict(pds=len(pds), images=n_img, N=cfg.N)
        for name, dtype, writers in (('f64_inline', np.float64, 0), ('f64_4writers', np.float64, 4),
                                     ('f32_4writers', np.float32, 4)):
            d = os.path.join(base, name)
            mp.dist_prog = os.path.join(d, 'progress')
            os.makedirs(mp.dist_prog)
            t0 = time.perf_counter()
            G.run_jobs(jobs_of(d), stack_file, nStot, options, writers=writers,
                       image_dtype=dtype, precision='bf16x3')
            sec = time.perf_counter() - t0
            nbytes = sum(os.path.getsize(os.path.join(d, f)) for f in os.listdir(d)
                         if f.startswith('IMGs_prD_'))
            out[name] = dict(seconds=sec, bytes=nbytes, gb_per_s=nbytes / sec / 1e9)
            shutil.rmtree(d)
        out['method'] = ('GetDistancesS2.run_jobs on the PDs, stack read from a raw file, '
                         'pickles to local disk; f32 = the image_dtype opt-in (CTF, imgAll, '
                         'imgAllFlip kept in the float32 the GPU computes them in)')
        return out
    finally:
        shutil.rmtree(base, ignore_errors=True)


def cpu_baseline(args, ds, counts, cfg, steps=1, budget_s=20.0):
    cores = os.cpu_count() or 1
    mic = dict(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    pick = choose_sample(np.asarray(counts), cores, max_n=args.cpu_max_n)
    sizes = None
    if len(pick) < 4:
        # few (large) PDs: time sub-PDs of the largest PD at several sizes
        big = int(np.argmax(counts))
        top = min(int(counts[big]), args.cpu_max_n)
        sizes = sorted(set(int(x) for x in np.linspace(max(20, top // 6), top, min(cores, 6))))
        pick = [big] * len(sizes)
    tasks = cpu_sample_tasks(ds, pick, mic, sizes)
    vals, walls = [], []
    for _ in range(steps):
        res, wall = run_cpu_tasks(tasks, cores)
        v, fit = extrapolate_pairs_per_s(res, wall, counts, cores)
        vals.append(v)
        walls.append(wall)
    ns = sizes if sizes is not None else sorted(int(counts[p]) for p in pick)
    what = 'sub-PDs of the largest PD' if sizes is not None else 'PDs at size quantiles'
    sample = ('%d %s (n=%s) of the %s workload, one per core, FP64 CPU port '
              '(oracle/distance_oracle.pd_op); pairs/s extrapolated to all %d PDs with '
              't(n)=a n + b n^2 fitted on the sample (a=%.3g s, b=%.3g s); sample wall %.1f s'
              % (len(pick), what, ns, args.config, len(counts), fit['a'], fit['b'], walls[-1]))
    return dict(value=float(np.median(vals)), unit='pairs/s', cores=cores, kind='port',
                sample=sample), walls


def cpu_port_rate(args, cfg, counts, steps, warmup=0):
    """The FP64 CPU port of the reference (oracle/) on the host cores: PDs at evenly spaced
    size quantiles (at most --cpu-max-n images; sub-PDs of the largest PD when fewer than four
    qualify), rendered on the CPU, one process per core; pairs/s extrapolated to the whole
    workload by t(n) = a n + b n^2.  Returns (median pairs/s, wall seconds per step, cores,
    description of the sample)."""
    from manifoldem_python_gb300.synthetic import make_dataset
    cores = os.cpu_count() or 1
    pick = choose_sample(np.asarray(counts), cores, max_n=args.cpu_max_n)
    sizes = None
    if len(pick) < 4:
        big = int(np.argmax(counts))
        top = min(int(counts[big]), args.cpu_max_n)
        sizes = sorted(set(int(x) for x in np.linspace(max(20, top // 6), top, min(cores, 6))))
        pick = [big] * len(sizes)
    uniq = sorted(set(pick))
    ds = make_dataset(cfg, device='cpu', pd_select=uniq)
    mic = dict(N=cfg.N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
    tasks = cpu_sample_tasks(ds, [uniq.index(p) for p in pick], mic, sizes)
    for _ in range(warmup):
        run_cpu_tasks(tasks[:1], 1)
    vals, walls = [], []
    for _ in range(steps):
        res, wall = run_cpu_tasks(tasks, cores)
        v, fit = extrapolate_pairs_per_s(res, wall, counts, cores)
        vals.append(v)
        walls.append(wall)
    ns = sizes if sizes is not None else sorted(int(counts[p]) for p in pick)
    sample = ('%d %s (n=%s) of the %s workload per step, one per core, FP64 CPU port of '
              'the reference (oracle/); pairs/s extrapolated to all %d PDs by '
              't(n)=a n + b n^2' % (len(pick), 'sub-PDs' if sizes else 'PDs at size quantiles',
                                    ns, args.config, len(counts)))
    return float(np.median(vals)), walls, cores, sample


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=10)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='ours', choices=['ours', 'reference'])
    ap.add_argument('--config', default='config4')
    ap.add_argument('--n-pd', type=int, default=0, help='override the number of PDs')
    ap.add_argument('--precision', default='bf16x3', choices=['fp32', 'bf16x3'],
                    help='the contraction form of the headline value and e2e')
    ap.add_argument('--forms', default='fp32,bf16x3',
                    help='contraction forms timed on the same plan data in the same run '
                         '(comma list; "" = only --precision)')
    ap.add_argument('--outputs', default='D,img_avg,img_avg_flip,img_all_intensity')
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-e2e', action='store_true')
    ap.add_argument('--e2e-mode', default='streamed', choices=['streamed', 'copy'],
                    help='streamed: stack left in pinned host memory, PD groups pipelined over '
                         'load / compute / copy streams; copy: one host-to-device copy of the '
                         'stack, then one execute')
    ap.add_argument('--e2e-groups', type=int, default=11)
    ap.add_argument('--e2e-ramp', type=float, default=1.35,
                    help='growth factor of the first PD groups of the streamed e2e pass')
    ap.add_argument('--e2e-ramp-steps', type=int, default=5)
    ap.add_argument('--e2e-dma', default='off', choices=['auto', 'off'],
                    help='streamed e2e: off = every group read over the host link by the load '
                         'kernel; auto = groups whose images are a few contiguous stack ranges '
                         'are copied by the copy engines into staging buffers (slower on GB300: '
                         '207 against 170 ms per config4 pass)')
    ap.add_argument('--no-dm', action='store_true',
                    help='skip the diffusion-map embedding of a sample of PDs (GPU vs CPU port)')
    ap.add_argument('--dm-pds', type=int, default=8)
    ap.add_argument('--no-nlsa', action='store_true',
                    help='skip the NLSA-stage report (GPU NLSA.op against the CPU port)')
    ap.add_argument('--nlsa-case', default='',
                    help='"N,n": run only the NLSA report on one synthetic PD of n images of '
                         'N px (its distance-stage outputs as input) and print it as JSON')
    ap.add_argument('--nlsa-snapshots-only', action='store_true',
                    help='with --nlsa-case: time only the snapshot matrix (mem_nlsa_snapshots) '
                         'of the PD, ConOrder = floor(n / 50), 8 modes, --steps launches')
    ap.add_argument('--no-precision', action='store_true',
                    help='skip the FP64 / diffusion-map precision report of one sample PD')
    ap.add_argument('--cpu-max-n', type=int, default=900)
    ap.add_argument('--dropin-io', type=int, default=0,
                    help='time GetDistancesS2.run_jobs with pickle writes on this many PDs')
    ap.add_argument('--batched', action='store_true',
                    help='admit the PDs into device-memory batches rendered one at a time '
                         '(default for config5, whose images do not fit on one device)')
    ap.add_argument('--fullsize-precision', action='store_true',
                    help='D of the whole first PD against a device FP64 contraction, with '
                         'near-duplicate and diffusion-map errors (default for config3)')
    ap.add_argument('--autotune', default='cached', choices=['cached', 'force', ''],
                    help="contraction schedule per PD size class: the autotuner's cached table "
                         "(measured first if absent), 'force' = measure again, '' = the "
                         "library's default schedule")
    ap.add_argument('--no-graph', dest='graph', action='store_false',
                    help='launch the stage directly instead of replaying a captured CUDA graph')
    args = ap.parse_args()

    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    metric = 'all-PD CTF-distance pairs/s'

    if args.nlsa_case:
        import dataclasses
        import torch
        from manifoldem_python_gb300.pipeline import StageParams
        from manifoldem_python_gb300.synthetic import CONFIGS, make_dataset
        N, n = (int(v) for v in args.nlsa_case.split(','))
        cfg = dataclasses.replace(CONFIGS['config1'], name='nlsa', N=N, n_pd=1, n_fixed=n,
                                  seed=5)
        dev = torch.device('cuda')
        ds = make_dataset(cfg, device=dev)
        params = StageParams(N=N, pix_size=cfg.pix, Cs=cfg.cs, EkV=cfg.kv, AmpContrast=cfg.ampc)
        if args.nlsa_snapshots_only:
            rep = nlsa_snapshot_case(ds, params, dev, args.steps)
        else:
            rep = nlsa_report(ds, params, dev, os.cpu_count() or 1,
                              n_cpu_max=0 if args.no_cpu_baseline else 800)
        print(json.dumps(dict(nlsa_case=dict(N=N, n=n), nlsa=rep)))
        return

    if args.impl == 'reference':
        if rank != 0:
            return
        from manifoldem_python_gb300.synthetic import CONFIGS, particle_counts
        import dataclasses
        cfg = CONFIGS[args.config]
        if args.n_pd:
            cfg = dataclasses.replace(cfg, n_pd=args.n_pd)
        counts = particle_counts(cfg)[:cfg.n_pd]
        v, walls, cores, sample = cpu_port_rate(args, cfg, counts, args.steps, args.warmup)
        line = dict(metric=metric, value=v, unit='pairs/s', n_gpus=args.gpus, steps=args.steps,
                    warmup=args.warmup, ms_per_step=float(np.median(walls)) * 1000,
                    higher_is_better=True, scaling='weak', vs_baseline=None, dtype='f64',
                    data='synthetic', impl='reference',
                    config=dict(workload=workload_string(args.config, cfg, counts)),
                    cpu_baseline=dict(value=v, unit='pairs/s', cores=cores, kind='port',
                                      sample=sample),
                    e2e=dict(value=v, unit='pairs/s', h2d_bytes_per_step=0,
                             d2h_bytes_per_step=0))
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        torch.distributed.init_process_group('nccl')
    batched = args.batched or args.config == 'config5'
    r = run_gpu_batched(args, rank, world) if batched else run_gpu(args, rank, world)
    pairs_total = r['pairs'] * world
    value = pairs_total / (r['ms'] * 1e-3)
    if rank != 0:
        if world > 1:
            torch.distributed.barrier()
        return
    rl = roofline(r, args)
    cfg = r['cfg']
    line = dict(
        metric=metric, value=value, unit='pairs/s', n_gpus=world, steps=args.steps,
        warmup=args.warmup, ms_per_step=r['ms'], higher_is_better=True, scaling='weak',
        vs_baseline=None, dtype={'fp32': 'f32', 'bf16x3': 'bf16x3+f32acc'}[args.precision],
        data='synthetic (seeded generator, 3-D Gaussian-blob volume, CTF, SNR %.2g)' % cfg.snr,
        config=dict(workload=workload_string(args.config, cfg, r['counts']),
                    precision=args.precision, outputs=list(r['outputs']),
                    l2=('L2 flushed before every timed step (%.2f GB image stack)'
                        if r['l2_flush'] else 'inputs larger than L2 (%.1f GB image stack)') % (
                        r.get('stack_gb', r['ds'].stack.numel() * 4 / 1e9)),
                    parallelism='PD-sharded, one process per GPU' if world > 1 else 'single GPU',
                    cuda_graph=r['graph']),
        roofline=dict(bound=rl['bound'], achieved=rl['achieved'], peak=rl['peak'],
                      unit=rl['unit'], frac=rl['frac'], traffic=rl['traffic'],
                      kernel=rl['phase'], peak_source=rl['peak_source'],
                      traffic_source=(('profiles/%s_%s.md: ncu dram__bytes_read.sum + '
                                       'dram__bytes_write.sum of the same kernel on a smaller '
                                       'case, scaled to this launch by the work it covers')
                                      % ((('contraction_' + args.precision) if
                                          rl['phase'] == 'contraction' else rl['phase']),
                                         args.config)) if rl['traffic'] else None),
        phases_ms=r['phases'],
        clocks=r['clocks'],
        gpu_launches=r['kernels'] * args.steps,
    )
    smem_rl = shared_memory_roofline(r, args, rl['phase']) if rl['bound'] == 'hbm' else None
    if smem_rl:
        line['roofline']['shared_memory'] = smem_rl
    if r['e2e']:
        e = r['e2e']
        line['e2e'] = dict(value=pairs_total / (e['ms'] * 1e-3), unit='pairs/s',
                           h2d_bytes_per_step=e['h2d'], d2h_bytes_per_step=e['d2h'],
                           ms_per_step=e['ms'], pinned=e['pinned'], mode=e['mode'])
    if r['phases'].get('contraction'):
        from manifoldem_python_gb300.pipeline import feature_columns
        peaks = load_peaks()
        Kalg = 4 * cfg.N * (cfg.N // 2 + 1)
        c_ms = r['phases']['contraction']
        alg = 2.0 * Kalg * r['pairs'] / (c_ms * 1e-3) / 1e12
        exe = 2.0 * 3 * feature_columns(cfg.N) * r['pairs'] / (c_ms * 1e-3) / 1e12
        line['contraction'] = dict(
            ms=c_ms, algorithmic_tflops=alg, frac_of_bf16_sustained=alg / peaks['bf16_sust'],
            issued_tflops_needed_pairs=exe,
            issued_frac_of_bf16_sustained=exe / peaks['bf16_sust'],
            note='algorithmic: 2 K flop per unordered pair, K = 4 N (N/2+1) (the reference '
                 'formulation); issued: three BF16 products over the Kf ring-feature columns '
                 'per needed pair (tile padding and diagonal halves not counted)')
    if r.get('batches'):
        line['config']['batches'] = ('%d HBM-admitted PD batches, images rendered on the device '
                                     'outside the timed region; a step is the sum of the '
                                     "batches' steps" % r['batches']['count'])
        line['batches'] = r['batches']
    if r.get('dm'):
        line['dm_embedding'] = r['dm']
    if r.get('nlsa'):
        line['nlsa'] = r['nlsa']
    if r.get('tuned'):
        line['contraction_schedule'] = dict(
            classes=r['tuned'], tuning_s=r['t_tune'],
            method='manifoldem_python_gb300/autotune.py: per size class, every candidate '
                   'schedule timed on a synthetic batch of the class (median of 5 executes)')
    forms = r['forms']
    if not args.no_precision:
        for f in forms:
            pr = precision_report(args, r['ds'], r.get('precision_counts', r['counts']), cfg, f)
            forms[f]['D_err_vs_fp64_oracle'] = pr['max_rel_err_vs_fp64_oracle']
            forms[f]['D_err_vs_fp64_contraction'] = pr['max_rel_err_vs_fp64_contraction']
            forms[f]['dm_top8_subspace_angle_rad'] = pr['dm_top8_subspace_angle_rad']
            if f == args.precision:
                line['precision'] = pr
    line['forms'] = forms
    if 'fp32' in forms and 'bf16x3' in forms:
        a, b = forms['fp32'], forms['bf16x3']
        line['speedup_bf16x3_vs_fp32'] = dict(
            step=a['ms_per_step'] / b['ms_per_step'],
            contraction=a['contraction_ms'] / b['contraction_ms'])
    if args.fullsize_precision or (args.config == 'config3' and not args.no_precision):
        import torch
        line['precision_fullsize'] = fullsize_precision(r['ds'], cfg, torch.device('cuda'))
    if args.dropin_io:
        line['dropin_io'] = dropin_io_report(r['ds'], cfg, n_pd=args.dropin_io)
    if not args.no_cpu_baseline:
        if r.get('batches'):
            v, _, cores, sample = cpu_port_rate(args, cfg, r['counts'], 1)
            line['cpu_baseline'] = dict(value=v, unit='pairs/s', cores=cores, kind='port',
                                        sample=sample)
        else:
            cb, _ = cpu_baseline(args, r['ds'], r['counts'], cfg)
            line['cpu_baseline'] = cb
    print(json.dumps(line))
    if world > 1:
        torch.distributed.barrier()


if __name__ == '__main__':
    main()
