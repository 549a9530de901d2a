"""Batched host API of the GPU distance stage.

``DistanceStage`` runs the distance stage for a batch of projection directions (PDs) on one GPU
through the C ABI (``include/manifoldem_gb300.h``): host-side bookkeeping in numpy
(``geometry.py``), device buffers from torch, one plan / upload / execute per batch.  PDs are
admitted into batches by an HBM budget so that any number of PDs runs on one GPU.

There is no CPU path: without the CUDA library or a GPU every call raises.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Dict, Iterable, List, Optional, Sequence

import numpy as np

from . import _lib
from .geometry import PdGeometry, pd_geometry

OUTPUT_NAMES = ('D', 'img_avg', 'img_avg_flip', 'img_all_intensity', 'img_all', 'img_all_flip',
                'ctf', 'spectrum', 'pair_norm')
DEFAULT_OUTPUTS = ('D', 'img_avg', 'img_avg_flip', 'img_all_intensity', 'img_all',
                   'img_all_flip', 'ctf')


@dataclasses.dataclass
class StageParams:
    """Microscope and stage parameters (the reference's p.* globals, filterPar, options)."""
    N: int
    pix_size: float
    Cs: float
    EkV: float
    AmpContrast: float
    gaussEnv: float = math.inf
    filter_type: str = 'Butter'
    filter_Qc: float = 0.5
    filter_order: float = 8
    avg_only: bool = False
    precision: str = 'fp32'          # 'fp32' or 'bf16x3'

    def to_c(self) -> _lib.MemParams:
        ft = {'Butter': _lib.MEM_FILTER_BUTTER, 'Gauss': _lib.MEM_FILTER_GAUSS}.get(self.filter_type)
        if ft is None:
            raise ValueError('%s filter is unsupported' % self.filter_type)
        prec = {'fp32': _lib.MEM_PREC_FP32, 'bf16x3': _lib.MEM_PREC_SPLIT_BF16}[self.precision]
        return _lib.MemParams(N=int(self.N), filter_type=ft, filter_Qc=float(self.filter_Qc),
                              filter_order=float(self.filter_order),
                              pix_size=float(self.pix_size), Cs=float(self.Cs),
                              EkV=float(self.EkV), gaussEnv=float(self.gaussEnv),
                              AmpContrast=float(self.AmpContrast),
                              avg_only=int(bool(self.avg_only)), precision=prec)


def _ptr(t) -> Optional[int]:
    return None if t is None else int(t.data_ptr())


class Plan:
    """A C-ABI plan plus its torch-allocated workspace, reusable across executions."""

    def __init__(self, params: StageParams, counts: Sequence[int], psi_p: Sequence[float],
                 device=None, contraction=None):
        """``contraction``: the split-BF16 contraction's schedule per size class (a list of
        dicts max_n / persistent / accumulators, see ``autotune``); default: the autotuner's
        cached table for this GPU and box size if there is one, else the library's default."""
        import torch
        self.lib = _lib.load()
        self.params = params
        self.device = torch.device(device or 'cuda')
        self.counts = np.ascontiguousarray(counts, dtype=np.int32)
        self.psi_p = np.ascontiguousarray(psi_p, dtype=np.float64)
        self._cparams = params.to_c()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.mem_plan_create(ctypes.byref(self._cparams),
                                                int(len(self.counts)),
                                                self.counts.ctypes.data, self.psi_p.ctypes.data,
                                                ctypes.byref(h)), 'mem_plan_create')
        self.handle = h
        if contraction is None and params.precision == 'bf16x3':
            from . import autotune
            contraction = autotune.lookup(torch.cuda.get_device_name(self.device), params.N,
                                          params.precision)
        self.contraction = contraction
        if contraction:
            from . import autotune
            arr = autotune.to_c(contraction)
            _lib.check(self.lib.mem_plan_set_contraction(h, len(contraction), arr),
                       'mem_plan_set_contraction')
        sz = ctypes.c_size_t()
        _lib.check(self.lib.mem_plan_workspace_size(h, ctypes.byref(sz)), 'workspace_size')
        self.ws_bytes = int(sz.value)
        self.n_images = int(self.lib.mem_plan_num_images(h))
        self.d_elems = int(self.lib.mem_plan_d_elements(h))
        self.n_pairs = int(self.lib.mem_plan_num_pairs(h))
        self.workspace = torch.empty(self.ws_bytes, dtype=torch.uint8, device=self.device)
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.lib.mem_plan_upload(h, self.workspace.data_ptr(), self.ws_bytes,
                                            ctypes.c_void_p(stream.cuda_stream)),
                   'mem_plan_upload')

    def allocate_outputs(self, names: Iterable[str] = DEFAULT_OUTPUTS) -> Dict[str, object]:
        import torch
        N = self.params.N
        n_pd, n_img = len(self.counts), self.n_images
        shapes = {
            'D': ((self.d_elems,), torch.float64),
            'img_avg': ((n_pd, N, N), torch.float64),
            'img_avg_flip': ((n_pd, N, N), torch.float64),
            'img_all_intensity': ((n_pd, N, N), torch.float64),
            'img_all': ((n_img, N, N), torch.float32),
            'img_all_flip': ((n_img, N, N), torch.float32),
            'ctf': ((n_img, N, N), torch.float32),
            'spectrum': ((n_img, N, N // 2 + 1, 2), torch.float32),
            'pair_norm': ((n_img,), torch.float64),
        }
        out = {}
        for name in names:
            if name == 'D' and self.params.avg_only:
                continue
            shp, dt = shapes[name]
            out[name] = torch.empty(shp, dtype=dt, device=self.device)
        return out

    def execute(self, stack, stack_index, flip, psi_rad, df, outputs: Dict[str, object],
                stream=None, shift_yx=None, pd_mask=None) -> None:
        """Enqueue the stage on ``stream`` (default: torch's current stream).  All tensors
        must be on the plan's device.  ``shift_yx`` ([n_images, 2] float64): a RELION stack,
        see ``relion_shifts``; ``pd_mask`` ([n_pd, N, N] uint8): volume masks, see
        ``VolumeMask``."""
        import torch
        stream = stream or torch.cuda.current_stream(self.device)
        cin = _lib.MemInputs(stack=stack.data_ptr(), num_stack=int(stack.shape[0]),
                             stack_index=stack_index.data_ptr(), flip=flip.data_ptr(),
                             psi_rad=psi_rad.data_ptr(), df=df.data_ptr(),
                             shift_yx=_ptr(shift_yx), pd_mask=_ptr(pd_mask))
        cout = _lib.MemOutputs(**{k: _ptr(outputs.get(k)) for k in OUTPUT_NAMES})
        self._keep = (cin, cout)
        _lib.check(self.lib.mem_plan_execute(self.handle, ctypes.byref(cin), ctypes.byref(cout),
                                             self.workspace.data_ptr(), self.ws_bytes,
                                             ctypes.c_void_p(stream.cuda_stream)),
                   'mem_plan_execute')

    def execute_split(self, stack, stack_index, flip, psi_rad, df, outputs: Dict[str, object],
                      load_stream, stream) -> None:
        """``execute`` with the stack-reading kernel on ``load_stream`` and the rest on
        ``stream`` (mem_plan_execute_split); ``stack`` may be a pinned host tensor."""
        cin = _lib.MemInputs(stack=stack.data_ptr(), num_stack=int(stack.shape[0]),
                             stack_index=stack_index.data_ptr(), flip=flip.data_ptr(),
                             psi_rad=psi_rad.data_ptr(), df=df.data_ptr(), shift_yx=None,
                             pd_mask=None)
        cout = _lib.MemOutputs(**{k: _ptr(outputs.get(k)) for k in OUTPUT_NAMES})
        self._keep = (cin, cout)
        _lib.check(self.lib.mem_plan_execute_split(
            self.handle, ctypes.byref(cin), ctypes.byref(cout), self.workspace.data_ptr(),
            self.ws_bytes, ctypes.c_void_p(load_stream.cuda_stream),
            ctypes.c_void_p(stream.cuda_stream)), 'mem_plan_execute_split')

    def capture(self, stack, stack_index, flip, psi_rad, df, outputs: Dict[str, object]):
        """Capture one execute (every kernel and cuFFT launch of the stage) in a CUDA graph and
        return it; ``graph.replay()`` reruns the stage on the same buffers.  Input and output
        tensors must stay alive and in place while the graph is used."""
        import torch
        side = torch.cuda.Stream(self.device)
        side.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(side):            # one untimed run outside capture
            self.execute(stack, stack_index, flip, psi_rad, df, outputs, side)
        torch.cuda.current_stream(self.device).wait_stream(side)
        torch.cuda.synchronize(self.device)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph):
            self.execute(stack, stack_index, flip, psi_rad, df, outputs)
        return graph

    def device_status(self) -> None:
        """Raise if a bounded device-side wait expired or an input index was out of range."""
        _lib.check(self.lib.mem_workspace_status(self.handle, self.workspace.data_ptr()),
                   'device status')

    def close(self):
        if getattr(self, 'handle', None) is not None and self.handle.value:
            self.lib.mem_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclasses.dataclass
class PdJob:
    """One PD: the reference's input_data = [ind, q, df, outFile, prD] (GetDistancesS2.py:37-47)."""
    ind: np.ndarray
    q: np.ndarray
    df: np.ndarray
    outFile: Optional[str] = None
    prD: int = 0


RING_MAX_KC = 40960      # half planes up to this size use ring features (the library's kRingMaxKc)


def feature_columns(N: int) -> int:
    """Columns of a feature row: [U' | V' | r' | s'] with one U', V' column per ring of equal
    |k|^2 (half planes up to RING_MAX_KC frequencies) or per frequency, each block padded to 64
    (the library's feature_layout)."""
    Nh = N // 2 + 1
    Kc = N * Nh
    pad = lambda x: -(-x // 64) * 64
    if Kc <= RING_MAX_KC:
        ka = np.arange(N)[:, None]
        kb = np.arange(Nh)[None, :]
        rings = int(np.unique(np.minimum(ka, N - ka) ** 2 + kb ** 2).size)
        return 2 * pad(rings) + 2 * pad(Kc)
    return 4 * pad(Kc)


def workspace_bytes_per_image(params: StageParams) -> int:
    """Approximate device bytes one image needs (workspace and full outputs)."""
    N = params.N
    feat = 4 * feature_columns(N)          # FP32 features, or bf16 hi + lo
    # + per-image tables: defocus phase, PD / row indices, pair norm, two rotations (64 B)
    return 4 * N * N * 4 + 8 * N * (N // 2 + 1) + feat + 128


def admit_batches(counts: Sequence[int], params: StageParams, budget_bytes: int) -> List[List[int]]:
    """Split PDs (in order) into consecutive batches whose device footprint fits the budget."""
    per_img = workspace_bytes_per_image(params)
    batches, cur, cur_bytes = [], [], 0
    for i, n in enumerate(counts):
        b = n * per_img + 8 * n * n + 4 * params.N * params.N * 8
        if cur and cur_bytes + b > budget_bytes:
            batches.append(cur)
            cur, cur_bytes = [], 0
        cur.append(i)
        cur_bytes += b
    if cur:
        batches.append(cur)
    return batches


class DistanceStage:
    """The GPU distance stage for a set of PDs sharing one image stack."""

    def __init__(self, params: StageParams, device=None):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError('the GPU distance stage needs a CUDA device (no CPU path)')
        self.params = params
        self.device = torch.device(device or 'cuda')
        _lib.load()

    def geometry(self, jobs: Sequence[PdJob], nStot: int) -> List[PdGeometry]:
        return [pd_geometry(np.asarray(j.ind), np.asarray(j.q, dtype=np.float64), nStot)
                for j in jobs]

    def run(self, jobs: Sequence[PdJob], stack, nStot: int, outputs=DEFAULT_OUTPUTS,
            geoms: Optional[Sequence[PdGeometry]] = None, to_host: bool = True, sh=None,
            mask: Optional['VolumeMask'] = None):
        """Run every job; returns one dict per PD with host numpy (``to_host``) or device
        arrays.  ``stack`` is a device tensor (num_part, N, N) float32 in SPIDER storage order,
        or, with ``sh`` = (shx, shy) per particle, the images of a RELION stack as stored.
        With a volume ``mask`` every PD's projected mask multiplies its spectra and averages
        and is returned as ``msk2`` (N x N bool)."""
        import torch
        geoms = list(geoms) if geoms is not None else self.geometry(jobs, nStot)
        counts = [int(np.asarray(j.ind).shape[0]) for j in jobs]
        plan = Plan(self.params, counts, [g.psi_p for g in geoms], self.device)
        dev = self.device
        sidx = torch.from_numpy(np.concatenate([g.stack_index for g in geoms])).to(dev)
        flip = torch.from_numpy(np.concatenate([g.flip for g in geoms])).to(dev)
        psi = torch.from_numpy(np.concatenate([g.psi_rad for g in geoms])).to(dev)
        df = torch.from_numpy(np.concatenate([np.asarray(j.df, dtype=np.float64).reshape(-1)
                                              for j in jobs])).to(dev)
        outs = plan.allocate_outputs(outputs)
        shifts = None
        if sh is not None:
            shifts = torch.from_numpy(relion_shifts(
                np.concatenate([g.stack_index for g in geoms]), sh)).to(dev)
        masks = mask.project(geoms) if mask is not None else None
        plan.execute(stack, sidx, flip, psi, df, outs, shift_yx=shifts, pd_mask=masks)
        torch.cuda.synchronize(dev)
        plan.device_status()
        res = split_outputs(plan, counts, outs, to_host)
        if masks is not None:
            for r, m in zip(res, masks.bool()):
                r['msk2'] = m.cpu().numpy() if to_host else m
        return res


class VolumeMask:
    """projectMask.op (modules/projectMask.py:118-135) on the GPU for one mask volume: the
    spline coefficients are prepared once (mem_mask_prepare), the mask of each PD is projected
    with the PD's affine map (mem_mask_project, geometry.mask_transform)."""

    def __init__(self, volume, device=None):
        import torch
        self.lib = _lib.load()
        self.device = torch.device(device or 'cuda')
        vol = np.ascontiguousarray(volume, dtype=np.float32)
        if vol.ndim != 3 or not (vol.shape[0] == vol.shape[1] == vol.shape[2]):
            raise ValueError('the mask volume must be an N x N x N cube')
        self.N = int(vol.shape[0])
        size = ctypes.c_size_t()
        _lib.check(self.lib.mem_mask_coefficients_size(self.N, ctypes.byref(size)),
                   'mask size')
        v = torch.from_numpy(vol).to(self.device)
        self.coeffs = torch.empty(size.value // 8, dtype=torch.float64, device=self.device)
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.lib.mem_mask_prepare(v.data_ptr(), self.N, self.coeffs.data_ptr(),
                                             ctypes.c_void_p(stream.cuda_stream)),
                   'mem_mask_prepare')
        torch.cuda.synchronize(self.device)

    def project(self, geoms: Sequence[PdGeometry]):
        """uint8 (n_pd, N, N) device tensor of 0/1 masks, one per PD geometry."""
        import torch
        from .geometry import mask_transform
        xf = np.empty((len(geoms), 12), dtype=np.float64)
        for i, g in enumerate(geoms):
            R, off = mask_transform(np.asarray(g.PD, dtype=np.float64).reshape(-1), self.N)
            xf[i, :9] = R.reshape(-1)
            xf[i, 9:] = off
        xf_d = torch.from_numpy(xf).to(self.device)
        out = torch.empty((len(geoms), self.N, self.N), dtype=torch.uint8, device=self.device)
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.lib.mem_mask_project(self.coeffs.data_ptr(), self.N, len(geoms),
                                             xf_d.data_ptr(), out.data_ptr(),
                                             ctypes.c_void_p(stream.cuda_stream)),
                   'mem_mask_project')
        return out


def relion_shifts(stack_index: np.ndarray, sh) -> np.ndarray:
    """Per-entry shifts (axis 0, axis 1) = (sh_y - 0.5, sh_x - 0.5) of the entry's particle, the
    arguments of the reference's scipy shift (``getDistanceCTF_local_Conj9combinedS2.py:263``);
    ``sh`` = (shx, shy) indexed by particle."""
    idx = np.asarray(stack_index, dtype=np.int64)
    out = np.empty((idx.size, 2), dtype=np.float64)
    out[:, 0] = np.asarray(sh[1], dtype=np.float64)[idx] - 0.5
    out[:, 1] = np.asarray(sh[0], dtype=np.float64)[idx] - 0.5
    return out


def group_weights(n_groups: int, ramp: float = 1.0, ramp_steps: int = 0) -> np.ndarray:
    """Relative image counts of the groups: ramp^min(g, ramp_steps) for group g (all equal for
    ramp 1 or ramp_steps 0)."""
    g = np.arange(max(1, int(n_groups)))
    return float(ramp) ** np.minimum(g, max(0, int(ramp_steps)))


def stack_runs(stack_index, max_runs: int):
    """The distinct stack indices of a group as runs of consecutive indices: (runs, remap) with
    runs = [(first index, count, offset in the staged copy)] and remap = each entry's position
    in the staged copy, or None when there are more than ``max_runs`` runs."""
    si = np.asarray(stack_index, dtype=np.int64)
    if si.size == 0:
        return [], si.copy()
    u = np.unique(si)
    breaks = np.nonzero(np.diff(u) != 1)[0] + 1
    if breaks.size + 1 > max_runs:
        return None
    starts = np.concatenate([[0], breaks])
    ends = np.concatenate([breaks, [u.size]])
    runs = [(int(u[a]), int(b - a), int(a)) for a, b in zip(starts, ends)]
    return runs, np.searchsorted(u, si).astype(np.int64)


def balanced_groups(counts: Sequence[int], n_groups: int, ramp: float = 1.0,
                    ramp_steps: int = 0) -> List[range]:
    """Consecutive PD ranges (at most n_groups, none empty) whose image counts follow
    group_weights: equal by default; with ramp > 1 the first ramp_steps groups grow
    geometrically, so that a pipeline that loads group g + 1 while it computes group g starts
    computing after loading a small first group."""
    counts = np.asarray(counts, dtype=np.int64)
    n_groups = max(1, min(int(n_groups), len(counts)))
    w = np.cumsum(group_weights(n_groups, ramp, ramp_steps))
    cum = np.cumsum(counts)
    cuts = [0]
    for g in range(1, n_groups):
        c = int(np.searchsorted(cum, cum[-1] * w[g - 1] / w[-1], side='left')) + 1
        cuts.append(min(max(c, cuts[-1] + 1), len(counts) - (n_groups - g)))
    cuts.append(len(counts))
    return [range(a, b) for a, b in zip(cuts[:-1], cuts[1:])]


class StreamedStage:
    """The stage for many PDs with the image stack left in pinned host memory.

    The PDs are split into ``n_groups`` consecutive groups, one plan each, of about equal image
    count after a geometric ramp over the first ``ramp_steps`` groups (``balanced_groups``): at
    128 px the host link delivers images about 1.3x faster than the stage computes them (0.31 us
    against 0.41 us per image on a GB300), so each group may be up to about that much larger than
    the one before without the compute stream waiting, and a small first group shortens the wait
    before the first computation.  Every ``run`` issues, per group, the per-image metadata copy and
    the image copy on a high-priority load stream, the rest of the stage on a compute stream, and
    the copy of the results into pinned host buffers on a copy stream.  Group g+1's images arrive
    while group g computes, and group g's results leave while group g+1 computes.

    The image copy: by default every group is read by a small grid of the library's load
    kernel over the host link (``mem_plan_execute_split``), which gathers scattered images
    without staging the stack.  With ``dma='auto'`` a group whose images form at most
    ``max_runs`` runs of consecutive stack indices (a stack stored in PD order) is instead
    copied run by run by the copy engines into a device staging buffer of its own, and its plan
    executes on the staged images.  On a GB300 the load kernel is the faster of the two for
    config4's 11 groups (170 ms against 207 ms per pass), so it stays the default.
    """

    def __init__(self, params: StageParams, counts: Sequence[int], psi_p: Sequence[float],
                 n_groups: int = 11, outputs=('D', 'img_avg', 'img_avg_flip', 'img_all_intensity'),
                 device=None, ramp: float = 1.35, ramp_steps: int = 5, dma: str = 'off',
                 max_runs: int = 64):
        if dma not in ('auto', 'off'):
            raise ValueError("dma must be 'auto' or 'off'")
        self.dma, self.max_runs = dma, int(max_runs)
        import torch
        self.device = torch.device(device or 'cuda')
        self.counts = [int(c) for c in counts]
        self.groups = balanced_groups(self.counts, n_groups, ramp, ramp_steps)
        psi_p = np.asarray(psi_p, dtype=np.float64)
        self.plans = [Plan(params, [self.counts[i] for i in g], psi_p[list(g)], self.device)
                      for g in self.groups]
        self.outputs = outputs
        self.dev_out = [p.allocate_outputs(outputs) for p in self.plans]
        self.host_out = [{k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
                          for k, v in d.items()} for d in self.dev_out]
        lo, hi = torch.cuda.Stream.priority_range() if hasattr(torch.cuda.Stream,
                                                                 'priority_range') else (0, -1)
        self.load_stream = torch.cuda.Stream(self.device, priority=min(lo, hi))
        self.stream = torch.cuda.Stream(self.device)
        self.copy_stream = torch.cuda.Stream(self.device)
        img_off = np.concatenate([[0], np.cumsum(self.counts)])
        self.img_ranges = [(int(img_off[g.start]), int(img_off[g.stop])) for g in self.groups]
        self._meta_h = None

    def set_metadata(self, stack_index, flip, psi_rad, df) -> None:
        """Per-image inputs over all PDs in plan order (host arrays); copied per run."""
        import torch
        arrays = [np.ascontiguousarray(stack_index, dtype=np.int64),
                  np.ascontiguousarray(flip, dtype=np.uint8),
                  np.ascontiguousarray(psi_rad, dtype=np.float64),
                  np.ascontiguousarray(df, dtype=np.float64)]
        self._meta_h, self._meta_d, self._runs, self._staging = [], [], [], []
        self._remap_h, self._remap_d = [], []
        N = self.plans[0].params.N if self.plans else 0
        for a, b in self.img_ranges:
            sel = [x[a:b].copy() for x in arrays]
            found = stack_runs(sel[0], self.max_runs) if self.dma == 'auto' else None
            runs, remap_h, remap_d, staging = None, None, None, None
            if found is not None:
                runs, remap = found
                remap_h = torch.from_numpy(remap).pin_memory()
                remap_d = torch.empty_like(remap_h, device=self.device)
                staging = torch.empty((sum(r[1] for r in runs), N, N), dtype=torch.float32,
                                      device=self.device)
            self._runs.append(runs)
            self._remap_h.append(remap_h)
            self._remap_d.append(remap_d)
            self._staging.append(staging)
            hs = [torch.from_numpy(x).pin_memory() for x in sel]
            self._meta_h.append(hs)
            self._meta_d.append([torch.empty_like(h, device=self.device) for h in hs])

    def metadata_bytes(self) -> int:
        """Per-image metadata bytes one run copies (staged groups: their staging indices in
        place of the stack indices)."""
        total = 0
        for hs, rh in zip(self._meta_h, self._remap_h):
            ts = hs if rh is None else [rh] + list(hs[1:])
            total += sum(t.numel() * t.element_size() for t in ts)
        return total

    def staged_groups(self) -> int:
        """Groups whose images the copy engines stage (the rest use the load kernel)."""
        return sum(r is not None for r in self._runs)

    def image_bytes(self, num_stack: int) -> int:
        """Image bytes one run copies to the device: the staged runs, and for the other groups
        the entries' images (read once each by the load kernel)."""
        N = self.plans[0].params.N if self.plans else 0
        total = 0
        for g, (a, b) in enumerate(self.img_ranges):
            n = sum(r[1] for r in self._runs[g]) if self._runs[g] is not None else b - a
            total += n * N * N * 4
        return total

    def result_bytes(self) -> int:
        return sum(t.numel() * t.element_size() for d in self.host_out for t in d.values())

    def run(self, stack):
        """One pass over all PDs; ``stack`` is a pinned host (or device) tensor.  Returns the
        per-group pinned host outputs (valid until the next run)."""
        import torch
        if self._meta_h is None:
            raise RuntimeError('set_metadata first')
        cur = torch.cuda.current_stream(self.device)
        for s in (self.load_stream, self.stream, self.copy_stream):
            s.wait_stream(cur)
        host_stack = not stack.is_cuda
        for g, plan in enumerate(self.plans):
            staged = host_stack and self._runs[g] is not None
            with torch.cuda.stream(self.load_stream):
                for i, (dst, src) in enumerate(zip(self._meta_d[g], self._meta_h[g])):
                    if not (staged and i == 0):          # staged: the staging indices instead
                        dst.copy_(src, non_blocking=True)
                if staged:
                    self._remap_d[g].copy_(self._remap_h[g], non_blocking=True)
                    buf = self._staging[g]
                    for first, count, off in self._runs[g]:
                        buf[off:off + count].copy_(stack[first:first + count], non_blocking=True)
            sidx, flip, psi, df = self._meta_d[g]
            if staged:
                loaded = torch.cuda.Event()
                loaded.record(self.load_stream)
                self.stream.wait_event(loaded)
                plan.execute(self._staging[g], self._remap_d[g], flip, psi, df, self.dev_out[g],
                             self.stream)
            else:
                plan.execute_split(stack, sidx, flip, psi, df, self.dev_out[g],
                                   self.load_stream, self.stream)
            done = torch.cuda.Event()
            done.record(self.stream)
            self.copy_stream.wait_event(done)
            with torch.cuda.stream(self.copy_stream):
                for k, v in self.dev_out[g].items():
                    self.host_out[g][k].copy_(v, non_blocking=True)
        self.copy_stream.synchronize()
        self.stream.synchronize()
        return self.host_out

    def device_status(self) -> None:
        for p in self.plans:
            p.device_status()


def split_outputs(plan: Plan, counts: Sequence[int], outs: Dict[str, object], to_host: bool):
    """Per-PD views of the batched outputs."""
    N = plan.params.N
    res = []
    img_off = np.concatenate([[0], np.cumsum(counts)])
    d_off = np.concatenate([[0], np.cumsum(np.asarray(counts, dtype=np.int64) ** 2)])
    host = {k: (v.cpu().numpy() if to_host else v) for k, v in outs.items()}
    for p, n in enumerate(counts):
        r = {}
        for k, v in host.items():
            if k == 'D':
                r[k] = v[d_off[p]:d_off[p + 1]].reshape(n, n)
            elif k in ('img_avg', 'img_avg_flip', 'img_all_intensity'):
                r[k] = v[p]
            else:
                r[k] = v[img_off[p]:img_off[p + 1]]
        res.append(r)
    return res
