"""Seeded synthetic cryo-EM inputs for the per-projection-direction distance stage.

The reference ships no image stack (its demo ``.mrcs`` is absent), so every test and benchmark
runs on data made here.  The generator follows the workload descriptions the distance stage is
benchmarked on:

* a volume of isotropic 3-D Gaussian blobs (radii U[3,8] px, centres uniform inside a sphere of
  radius 0.35*N); one blob (two for the 2-D latent) moves linearly with a latent coordinate t;
* each particle is the projection of that volume along its orientation, given as Spider Euler
  angles (phi, theta, psi) and converted to a quaternion with the reference's convention
  (``read_alignfile.py:93-94`` -> ``util.eul_to_quat(flip=True)`` ``util.py:76-92`` and
  ``qMult_bsx.op`` ``qMult_bsx.py:14-34``);
* the projection is multiplied by a CTF (300 kV, Cs 2.7 mm, amplitude contrast 0.1, a per-particle
  defocus and a B-factor envelope exp(-B k^2/4)) and Gaussian noise is added at a given SNR;
* particles are grouped into projection directions (PDs) whose centres lie on a Fibonacci sphere;
  a fraction of PDs is built from conjugate views (indices >= nStot/2, read flipped up-down by the
  distance stage, ``getDistanceCTF_local_Conj9combinedS2.py:247-275``), with quaternions
  augmented as in ``util.augment`` (``util.py:94-106``).

The image stack is returned in the SPIDER raw layout the distance stage reads: image j occupies
float32 elements [j*N*N, (j+1)*N*N) and the stage sees ``stack[j].T``.

Geometry (angles, quaternions, bins) is drawn with numpy ``default_rng(seed)``; images are drawn
with torch on the requested device so that the large configurations generate in seconds on a GPU.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional, Sequence

import numpy as np

__all__ = ["SynthConfig", "Dataset", "CONFIGS", "make_dataset", "particle_counts", "quat_from_euler",
           "augment_quat"]


@dataclasses.dataclass
class SynthConfig:
    name: str
    N: int                     # box size in pixels
    n_pd: int = 1              # number of projection directions
    n_fixed: Optional[int] = None   # particles per PD when not drawn
    n_median: float = 400.0
    n_sigma: float = 0.6       # log-normal sigma of the particle count (not specified by the
                               # workload description; 0.6 is the recorded choice)
    n_min: int = 100
    n_max: int = 3000
    pix: float = 2.0           # Angstrom per pixel
    kv: float = 300.0
    cs: float = 2.7            # mm
    ampc: float = 0.1
    df_range: Sequence[float] = (10000.0, 30000.0)   # Angstrom (1.0-3.0 um)
    bfactor: float = 50.0      # A^2, applied only when images are generated
    snr: float = 0.1
    n_latent: int = 1
    conj_pd_frac: float = 0.0  # fraction of PDs made of conjugate views
    near_dup_frac: float = 0.0  # fraction of images that are near-duplicates of another image
    near_dup_noise: float = 0.01
    jitter_deg: float = 1.0
    seed: int = 0


CONFIGS = {
    "config1": SynthConfig("config1", N=70, n_pd=1, n_fixed=300, seed=11),
    "config2": SynthConfig("config2", N=128, n_pd=1, n_fixed=2000, seed=12),
    "config3": SynthConfig("config3", N=192, n_pd=1, n_fixed=4000, near_dup_frac=0.05, seed=13),
    "config4": SynthConfig("config4", N=128, n_pd=800, n_median=400, n_min=100, n_max=3000,
                           conj_pd_frac=0.10, seed=14),
    "config5": SynthConfig("config5", N=250, n_pd=1500, n_median=1200, n_min=200, n_max=6000,
                           df_range=(5000.0, 40000.0), snr=0.05, n_latent=2,
                           conj_pd_frac=0.10, seed=15),
}


@dataclasses.dataclass
class Dataset:
    cfg: SynthConfig
    stack: object              # torch.Tensor (num_part, N, N) float32, SPIDER storage order
    q: np.ndarray              # (4, 2*num_part) float64, augmented with conjugates
    df: np.ndarray             # (2*num_part,) float64 Angstrom, duplicated for conjugates
    CG: List[np.ndarray]       # per PD int64 indices into the augmented set
    sh: tuple                  # (shx, shy) zeros (SPIDER data carries no shifts)
    latent: np.ndarray         # (num_part, n_latent)
    near_dup_of: np.ndarray    # (num_part,) index of the source image, -1 if none

    @property
    def num_part(self) -> int:
        return int(self.q.shape[1] // 2)

    @property
    def nStot(self) -> int:
        return int(self.q.shape[1])


def _qmul(q: np.ndarray, s: np.ndarray) -> np.ndarray:
    """Hamilton product of 4xM quaternion arrays (scalar first)."""
    q0, qv = q[0], q[1:4]
    s0, sv = s[0], s[1:4]
    vec = q0 * sv + s0 * qv + np.cross(qv, sv, axis=0)
    return np.vstack((q0 * s0 - np.sum(qv * sv, axis=0), vec))


def quat_from_euler(phi, theta, psi, flip=True) -> np.ndarray:
    """Spider Euler angles (radians) -> 4xM quaternions, q = qzs * (qy * qz)."""
    phi, theta, psi = (np.atleast_1d(np.asarray(a, dtype=np.float64)) for a in (phi, theta, psi))
    z = np.zeros_like(phi)
    qz = np.vstack((np.cos(phi / 2), z, z, -np.sin(phi / 2)))
    qy = np.vstack((np.cos(theta / 2), z, -np.sin(theta / 2), z))
    sp = np.sin(psi / 2)
    if flip:
        sp = -sp
    qzs = np.vstack((np.cos(psi / 2), z, z, sp))
    return _qmul(qzs, _qmul(qy, qz))


def augment_quat(q: np.ndarray) -> np.ndarray:
    """Append the conjugate views [-q1, q0, -q3, q2] after the originals."""
    qc = np.vstack((-q[1], q[0], -q[3], q[2]))
    return np.hstack((q, qc))


def _deaugment(qc: np.ndarray) -> np.ndarray:
    """Inverse of the conjugate map: the original whose conjugate is ``qc``."""
    return np.vstack((qc[1], -qc[0], qc[3], -qc[2]))


def _rot_rows(q: np.ndarray):
    """Rows of the rotation matrix of unit quaternions q (4xM): r1, r2, r3 (each 3xM).

    r3 equals the projection direction the distance stage derives from q
    (``getDistanceCTF_local_Conj9combinedS2.py:182-184``)."""
    w, x, y, zq = q
    r1 = np.vstack((1 - 2 * (y * y + zq * zq), 2 * (x * y + w * zq), 2 * (x * zq - w * y)))
    r2 = np.vstack((2 * (x * y - w * zq), 1 - 2 * (x * x + zq * zq), 2 * (y * zq + w * x)))
    r3 = np.vstack((2 * (x * zq - w * y), 2 * (y * zq + w * x), 1 - 2 * (x * x + y * y)))
    return r1, r2, r3


def _fibonacci_sphere(n: int) -> np.ndarray:
    i = np.arange(n) + 0.5
    z = 1 - 2 * i / n
    r = np.sqrt(np.maximum(0.0, 1 - z * z))
    ang = math.pi * (3 - math.sqrt(5)) * i
    return np.vstack((r * np.cos(ang), r * np.sin(ang), z))


def _dir_to_euler(d: np.ndarray):
    """Unit direction -> (phi, theta) such that the q built from (phi, theta, psi) has r3 == d."""
    theta = np.arccos(np.clip(d[2], -1, 1))
    phi = np.arctan2(d[1], d[0])
    return phi, theta


def _particle_counts(cfg: SynthConfig, rng) -> np.ndarray:
    if cfg.n_fixed is not None:
        return np.full(cfg.n_pd, int(cfg.n_fixed), dtype=np.int64)
    n = rng.lognormal(mean=math.log(cfg.n_median), sigma=cfg.n_sigma, size=cfg.n_pd)
    return np.clip(np.round(n), cfg.n_min, cfg.n_max).astype(np.int64)


def _orientations_for(d: np.ndarray, n: int, jitter_deg: float, rng) -> np.ndarray:
    phi0, theta0 = _dir_to_euler(d)
    # Spider convention: pick (phi, theta) whose r3 points along d, then jitter.
    qtest = quat_from_euler(phi0, theta0, 0.0)
    r3 = _rot_rows(qtest)[2][:, 0]
    if np.dot(r3, d) < 0.999:     # fall back to a direct search of the sign convention
        for sp, st in ((-1, 1), (1, -1), (-1, -1)):
            qtest = quat_from_euler(sp * phi0, st * theta0, 0.0)
            if np.dot(_rot_rows(qtest)[2][:, 0], d) > 0.999:
                phi0, theta0 = sp * phi0, st * theta0
                break
    jit = np.deg2rad(jitter_deg)
    phi = phi0 + rng.normal(0, jit, n) / max(math.sin(theta0), 0.05)
    theta = theta0 + rng.normal(0, jit, n)
    psi = rng.uniform(0, 2 * math.pi, n)
    return quat_from_euler(phi, theta, psi)


def particle_counts(cfg: SynthConfig) -> np.ndarray:
    """Particles per PD of ``cfg`` (the first draw of its generator)."""
    return _particle_counts(cfg, np.random.default_rng(cfg.seed))


def make_geometry(cfg: SynthConfig, pd_limit: Optional[int] = None) -> dict:
    """Everything of the dataset of ``cfg`` except the images: particle counts, orientations,
    defoci, latent coordinates, near-duplicates, the blob volume and the noise seed (host
    arrays).  ``make_dataset`` renders from it; a workload too large for one device renders it
    PD batch by PD batch with ``render_pds``.  ``pd_limit`` keeps only the first PDs."""
    rng = np.random.default_rng(cfg.seed)
    counts = _particle_counts(cfg, rng)
    n_pd = cfg.n_pd if pd_limit is None else min(pd_limit, cfg.n_pd)
    counts = counts[:n_pd]
    centres = _fibonacci_sphere(cfg.n_pd)[:, :n_pd]
    conj_pd = np.zeros(n_pd, dtype=bool)
    if cfg.conj_pd_frac > 0:
        k = int(round(cfg.conj_pd_frac * cfg.n_pd))
        sel = rng.permutation(cfg.n_pd)[:k]
        conj_pd[sel[sel < n_pd]] = True

    num_part = int(counts.sum())
    q_orig = np.empty((4, num_part))
    in_conj = np.zeros(num_part, dtype=bool)
    CG = []
    start = 0
    for pd in range(n_pd):
        n = int(counts[pd])
        qv = _orientations_for(centres[:, pd], n, cfg.jitter_deg, rng)
        idx = np.arange(start, start + n, dtype=np.int64)
        if conj_pd[pd]:
            # the conjugate views (index + num_part) lie along this PD; store their originals
            q_orig[:, start:start + n] = _deaugment(qv)
            in_conj[start:start + n] = True
            # mix: half of the PD are conjugate views, half plain views of the same direction
            half = n // 2
            q_orig[:, start + half:start + n] = qv[:, half:]
            in_conj[start + half:start + n] = False
            idx = idx.copy()
            idx[:half] += num_part
        else:
            q_orig[:, start:start + n] = qv
        CG.append(idx)
        start += n

    df_orig = rng.uniform(cfg.df_range[0], cfg.df_range[1], num_part)
    latent = rng.uniform(0, 1, (num_part, cfg.n_latent))
    near_dup_of = np.full(num_part, -1, dtype=np.int64)
    if cfg.near_dup_frac > 0:
        for pd in range(n_pd):
            idx = np.arange(CG[pd].size) + int(np.sum(counts[:pd]))
            k = int(round(cfg.near_dup_frac * idx.size))
            if k == 0:
                continue
            perm = rng.permutation(idx)
            dst, src = perm[:k], perm[k:2 * k]
            near_dup_of[dst] = src
            q_orig[:, dst] = q_orig[:, src]
            df_orig[dst] = df_orig[src]
            latent[dst] = latent[src]

    # volume of Gaussian blobs
    N = cfg.N
    n_blob = 20
    radii = rng.uniform(3, 8, n_blob)
    u = rng.normal(size=(3, n_blob))
    u /= np.linalg.norm(u, axis=0)
    centre = u * (0.35 * N * rng.uniform(0, 1, n_blob) ** (1 / 3))
    amp = rng.uniform(0.5, 1.5, n_blob)
    moves = rng.normal(size=(3, cfg.n_latent))
    moves *= (0.15 * N) / np.linalg.norm(moves, axis=0)
    noise_seed = int(rng.integers(0, 2**62))

    return dict(CG=CG, q_orig=q_orig, df_orig=df_orig, latent=latent, near_dup_of=near_dup_of,
                num_part=num_part, radii=radii, centre=centre, amp=amp, moves=moves,
                noise_seed=noise_seed)


def make_dataset(cfg: SynthConfig, device="cpu", dtype=None, pd_limit: Optional[int] = None,
                 pd_select: Optional[Sequence[int]] = None) -> Dataset:
    """Build the dataset of ``cfg``.  ``pd_limit`` keeps only the first PDs; ``pd_select`` keeps
    the listed PDs of the full workload (same geometry), rendering only their particles."""
    return render_pds(cfg, make_geometry(cfg, pd_limit), pd_select, device, dtype)


def render_pds(cfg: SynthConfig, geom: dict, pd_select: Optional[Sequence[int]] = None,
               device="cpu", dtype=None) -> Dataset:
    """The dataset of the PDs ``pd_select`` (all when None) of a geometry from
    ``make_geometry``: their particles rendered on ``device``, indices remapped to them."""
    CG, q_orig, df_orig = geom['CG'], geom['q_orig'], geom['df_orig']
    latent, near_dup_of, num_part = geom['latent'], geom['near_dup_of'], geom['num_part']
    radii, centre, amp, moves = geom['radii'], geom['centre'], geom['amp'], geom['moves']
    noise_seed = geom['noise_seed']
    if pd_select is not None:
        sel = [int(i) for i in pd_select]
        phys = [np.where(CG[i] >= num_part, CG[i] - num_part, CG[i]) for i in sel]
        keep = np.unique(np.concatenate(phys))
        remap = np.full(num_part, -1, dtype=np.int64)
        remap[keep] = np.arange(keep.size)
        new_cg = []
        for i, ph in zip(sel, phys):
            conj = CG[i] >= num_part
            new_cg.append(remap[ph] + np.where(conj, keep.size, 0))
        CG = new_cg
        q_orig, df_orig, latent = q_orig[:, keep], df_orig[keep], latent[keep]
        nd = near_dup_of[keep]
        near_dup_of = np.where(nd >= 0, remap[np.maximum(nd, 0)], -1)
        near_dup_of[near_dup_of < 0] = -1
        num_part = keep.size

    q_aug = augment_quat(q_orig)
    df_aug = np.concatenate((df_orig, df_orig))

    stack = _render(cfg, q_orig, df_orig, latent, near_dup_of, radii, centre, amp, moves,
                    noise_seed, device, dtype)
    shx = np.zeros(2 * num_part)
    return Dataset(cfg=cfg, stack=stack, q=q_aug, df=df_aug, CG=CG, sh=(shx, shx.copy()),
                   latent=latent, near_dup_of=near_dup_of)


def _render(cfg, q, df, latent, near_dup_of, radii, centre, amp, moves, noise_seed, device,
            dtype, chunk=8192):
    """Projection + CTF + noise, in chunks, on ``device``; returns (num_part, N, N) float32."""
    import torch

    dev = torch.device(device)
    cdt = torch.float64 if (dtype is None and dev.type == "cpu") else (dtype or torch.float32)
    N = cfg.N
    num_part = q.shape[1]
    r1, r2, _ = _rot_rows(q)
    out = torch.empty((num_part, N, N), dtype=torch.float32, device=dev)
    coords = torch.arange(N, dtype=cdt, device=dev) - N / 2
    fr = torch.fft.fftfreq(N, d=cfg.pix, dtype=cdt, device=dev)
    k2 = fr[:, None] ** 2 + fr[None, :] ** 2
    lam = 12.3986 / math.sqrt((2 * 511.0 + cfg.kv) * cfg.kv)
    env = torch.exp(-cfg.bfactor * k2 / 4)
    g = torch.Generator(device=dev)
    g.manual_seed(noise_seed)
    radii_t = torch.as_tensor(radii, dtype=cdt, device=dev)
    amp_t = torch.as_tensor(amp, dtype=cdt, device=dev)
    s1 = s2 = 0.0
    for s in range(0, num_part, chunk):
        e = min(num_part, s + chunk)
        c = np.repeat(centre[:, :, None], e - s, axis=2)          # 3 x B x P
        for li in range(cfg.n_latent):
            c[:, li, :] = c[:, li, :] + moves[:, li:li + 1] * (latent[s:e, li] - 0.5)[None, :]
        pu = np.einsum("dbp,dp->pb", c, r1[:, s:e])                # P x B
        pv = np.einsum("dbp,dp->pb", c, r2[:, s:e])
        pu = torch.as_tensor(pu, dtype=cdt, device=dev)
        pv = torch.as_tensor(pv, dtype=cdt, device=dev)
        gu = torch.exp(-(coords[None, None, :] - pu[:, :, None]) ** 2 / (2 * radii_t[None, :, None] ** 2))
        gv = torch.exp(-(coords[None, None, :] - pv[:, :, None]) ** 2 / (2 * radii_t[None, :, None] ** 2))
        img = torch.einsum("pbx,pby->pxy", gu * amp_t[None, :, None], gv)
        dfb = torch.as_tensor(df[s:e], dtype=cdt, device=dev)
        w = (0.5 * math.pi * cfg.cs * 1e7 * lam ** 3 * k2[None] - math.pi * lam * dfb[:, None, None]) * k2[None]
        ctf = (torch.sin(w) - cfg.ampc * torch.cos(w)) * env[None]
        img = torch.fft.ifft2(torch.fft.fft2(img) * ctf).real
        s1 += float(img.sum(dtype=torch.float64))
        s2 += float((img.to(torch.float64) ** 2).sum())
        out[s:e] = img.to(torch.float32)
    cnt = float(num_part) * N * N
    sig_var = max(s2 / cnt - (s1 / cnt) ** 2, 1e-30)
    sigma = math.sqrt(sig_var / cfg.snr)
    for s in range(0, num_part, chunk):
        e = min(num_part, s + chunk)
        noise = torch.randn((e - s, N, N), generator=g, dtype=cdt, device=dev) * sigma
        out[s:e] += noise.to(torch.float32)
    if np.any(near_dup_of >= 0):
        # near-duplicates: the source image (signal and its noise) plus a small extra noise
        dst = torch.as_tensor(np.nonzero(near_dup_of >= 0)[0], device=dev)
        src = torch.as_tensor(near_dup_of[near_dup_of >= 0], device=dev)
        extra = torch.randn((dst.numel(), N, N), generator=g, dtype=cdt, device=dev)
        out[dst] = out[src] + (extra * sigma * cfg.near_dup_noise).to(torch.float32)
    return out
