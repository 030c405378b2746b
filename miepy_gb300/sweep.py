"""Batched wavelength sweeps of one sphere cluster.

The reference computes a spectrum by building one ``sphere_cluster`` per
wavelength (sphere_cluster.py:27-125), each with its own Mie coefficients
(mie_single/mie_sphere.py:16-76), source decomposition (sources/plane_waves.py:
126-156), aggregate T-matrix (interactions.cpp:370-415) and solve
(interactions.cpp:347-368), one after the other.  Here every wavelength of the
sweep is one cluster of a single ragged ClusterBatch: the per-wavelength lmax may
differ (an adaptive rule), all translation matrices are assembled by one launch,
all solves advance together through the same captured launch sequence (finished
wavelengths drop out of the masked kernels), and one epilogue launch produces the
cross-sections of every wavelength.  Wavelengths are split into consecutive
batches only when a batch would exceed ``max_batch_bytes`` of HBM.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch

from .engine import ClusterBatch, footprint_bytes, require_cuda
from .materials import constant_material, material_struct
from .mie import mie_coefficients
from .modes import lmax_to_rmax
from .sources import plane_wave


def adaptive_lmax(wavelength, lo=400e-9, hi=1000e-9, lmax_lo=3, lmax_hi=7):
    """lmax(lambda) = clip(round(lmax_lo + (lmax_hi - lmax_lo) (hi - lambda) / (hi - lo)), lmax_lo, lmax_hi):
    the largest lmax at the shortest wavelength."""
    f = (hi - np.asarray(wavelength, float)) / (hi - lo)
    return np.clip(np.round(lmax_lo + (lmax_hi - lmax_lo) * f), lmax_lo, lmax_hi).astype(int)


@dataclass
class SweepResult:
    wavelength: np.ndarray                 # [W]
    lmax: np.ndarray                       # [W]
    C_sca: np.ndarray                      # [W, R] summed over particles and multipoles
    C_abs: np.ndarray
    C_ext: np.ndarray
    status: np.ndarray                     # [W, R] solver status per wavelength
    iterations: np.ndarray                 # [W, R]
    per_particle: np.ndarray | None = None  # [W] list of [N, R, 3, 2, lmax] (Csca, Cabs, Cext)
    batches: list = field(default_factory=list)


def sweep_specs(position, radius, material, wavelengths, lmax, medium=None, sources=None):
    """One ClusterBatch spec per wavelength: Mie coefficients, wavenumber and the
    source decomposition p_src [N, 2, rmax, R] (R = number of sources)."""
    position = np.asarray(np.atleast_2d(position), float)
    N = position.shape[0]
    radius = np.broadcast_to(np.asarray(radius, float), (N,))
    mats = material if isinstance(material, (list, tuple, np.ndarray)) else [material] * N
    medium = medium if medium is not None else constant_material(eps=1.0, mu=1.0)
    sources = sources if sources is not None else [plane_wave.from_string("x")]
    wl = np.atleast_1d(np.asarray(wavelengths, float))
    lm = np.asarray(lmax(wl) if callable(lmax) else np.broadcast_to(np.asarray(lmax, int), wl.shape), int)
    specs = []
    for w, L in zip(wl, lm):
        md = material_struct(np.asarray(mats, dtype=object), medium, wavelength=w)
        conducting = np.array([getattr(m, "name", None) == "metal" for m in mats])
        ms, mi = mie_coefficients(radius, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, int(L), conducting)
        k = float(np.real(md.k_b))
        p_src = np.stack([src.structure(position, k, int(L)) for src in sources], axis=-1)   # [N,2,rmax,R]
        specs.append(dict(position=position, mie_scat=ms, mie_int=mi, k=k, p_src=p_src,
                          eps_b=float(np.real(md.eps_b)), wavelength=float(w), lmax=int(L)))
    return specs


def _batches(specs, R, precision, max_batch_bytes):
    """Consecutive groups of specs whose HBM footprint stays within max_batch_bytes."""
    if max_batch_bytes is None:
        return [list(range(len(specs)))]
    groups, cur, used = [], [], 0
    for i, s in enumerate(specs):
        f = footprint_bytes(np.asarray(s["position"]).reshape(-1, 3).shape[0], s["lmax"], R, precision)
        if cur and used + f > max_batch_bytes:
            groups.append(cur)
            cur, used = [], 0
        cur.append(i)
        used += f
    if cur:
        groups.append(cur)
    return groups


def wavelength_sweep(position, radius, material, wavelengths, lmax=adaptive_lmax, medium=None, sources=None,
                     precision="mixed", tol=1e-8, inner_tol=1e-4, max_refine=8, maxiter=1000, device=None,
                     max_batch_bytes=None, per_particle=False, specs=None):
    """Spectra of a sphere cluster over many wavelengths, solved as ragged batches.

    lmax: an int, or a function of the wavelength array (default: ``adaptive_lmax``).
    sources: list of sources solved together as right-hand sides (default: one
    x-polarised plane wave along +z).  Returns a SweepResult with the total cross-
    sections per wavelength and right-hand side.
    """
    dev = require_cuda(device)
    if specs is None:
        specs = sweep_specs(position, radius, material, wavelengths, lmax, medium, sources)
    R = int(np.asarray(specs[0]["p_src"]).shape[-1]) if np.asarray(specs[0]["p_src"]).ndim == 4 else 1
    W = len(specs)
    C = np.zeros((W, R, 3))
    status = np.zeros((W, R), np.int32)
    iters = np.zeros((W, R), np.int32)
    parts = [None] * W if per_particle else None
    batches = []
    for group in _batches(specs, R, precision, max_batch_bytes):
        eps_b = {specs[i]["eps_b"] for i in group}
        if len(eps_b) != 1:
            raise ValueError("a batch needs one medium permittivity (the epilogue takes one eps_b)")
        b = ClusterBatch([specs[i] for i in group], R=R, precision=precision, device=dev)
        b.assemble()
        b.solve(tol=tol, maxiter=maxiter, inner_tol=inner_tol, max_refine=max_refine)
        b.epilogue(eps_b.pop())
        xs = b.xs[: b.totals["obs"] * R * 6 * b.xs_L].view(-1, R, 3, 2 * b.xs_L)
        for s, i in enumerate(group):
            l = b.layout[s]
            blk = xs[l["obs_off"]: l["obs_off"] + l["N"], :, :, : 2 * l["lmax"]]
            C[i] = blk.sum(dim=(0, 3)).cpu().numpy()
            if per_particle:
                parts[i] = blk.reshape(l["N"], R, 3, 2, l["lmax"]).cpu().numpy()
        status[group] = b.status.reshape(len(group), R)
        iters[group] = b.iters.reshape(len(group), R)
        batches.append(b)
    wl = np.array([s["wavelength"] for s in specs])
    lm = np.array([s["lmax"] for s in specs])
    return SweepResult(wavelength=wl, lmax=lm, C_sca=C[:, :, 0], C_abs=C[:, :, 1], C_ext=C[:, :, 2], status=status,
                       iterations=iters, per_particle=parts, batches=batches)


def drude_cluster(N=100, seed=3, rmin=40e-9, rmax=80e-9, box=2e-6, max_tries=1_000_000):
    """Seeded non-overlapping spheres: radii U[rmin, rmax], centres U[0, box]^3,
    accepted when clear of every accepted sphere (config of the sweep benchmark)."""
    rng = np.random.default_rng(seed)
    pos, rad = [], []
    tries = 0
    while len(pos) < N:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("rejection sampling did not place all spheres")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, box, 3)
        if all(np.linalg.norm(c - p) > r + q for p, q in zip(pos, rad)):
            pos.append(c)
            rad.append(r)
    return np.array(pos), np.array(rad)
