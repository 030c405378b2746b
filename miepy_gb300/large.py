"""Large single systems: a jittered hexagonal lattice of spheres, its solve, and
near-field maps on a plane.

The reference would build one ``sphere_cluster`` (sphere_cluster.py:27-125) and
evaluate ``E_field`` point by point in Python (sphere_cluster.py:244-391,
vsh/expansion.py:13-42).  Here the solve is one ClusterBatch and the field map is
one launch of the near-field kernel: FP64 (``gb_near_field``, the parity path) or
FP32 exterior sums (``gb_near_field32``) for maps of ~1e9 point-particle terms.
"""

from __future__ import annotations

import numpy as np
import torch

from . import _native as nat
from .engine import ClusterBatch, current_stream
from .materials import constant_material, material_struct
from .mie import mie_coefficients
from .modes import lmax_to_rmax
from .sources import plane_wave


def hex_lattice(N=2000, pitch=300e-9, jitter=30e-9, seed=5, cells=45):
    """N sites of a cells x cells hexagonal lattice in the z = 0 plane (the N
    closest to its centre), each moved by U[-jitter, jitter] in x and y; centred on
    the origin."""
    rng = np.random.default_rng(seed)
    rows, cols = np.meshgrid(np.arange(cells), np.arange(cells), indexing="ij")
    x = cols * pitch + (rows % 2) * pitch / 2
    y = rows * pitch * np.sqrt(3) / 2
    xy = np.column_stack([x.ravel(), y.ravel()])
    c = xy.mean(axis=0)
    keep = np.sort(np.argsort(np.linalg.norm(xy - c, axis=1), kind="stable")[:N])
    xy = xy[keep] - c + rng.uniform(-jitter, jitter, size=(N, 2))
    return np.column_stack([xy, np.zeros(N)])


def plane_grid(position, n=512, margin=500e-9, z=0.0):
    """n x n points on the plane z spanning the particles' bounding box + margin: [n*n, 3]."""
    lo = position[:, :2].min(axis=0) - margin
    hi = position[:, :2].max(axis=0) + margin
    x = np.linspace(lo[0], hi[0], n)
    y = np.linspace(lo[1], hi[1], n)
    X, Y = np.meshgrid(x, y, indexing="ij")
    return np.column_stack([X.ravel(), Y.ravel(), np.full(X.size, z)])


def lattice_spec(position, radius=80e-9, index=2.0, wavelength=600e-9, lmax=3, medium_index=1.0, source=None):
    N = position.shape[0]
    mat = constant_material(index=index)
    md = material_struct(np.asarray([mat] * N, dtype=object), constant_material(index=medium_index),
                         wavelength=wavelength)
    rad = np.full(N, radius)
    ms, mi = mie_coefficients(rad, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, lmax)
    k = float(np.real(md.k_b))
    src = source if source is not None else plane_wave.from_string("x")
    spec = dict(position=position, mie_scat=ms, mie_int=mi, k=k, p_src=src.structure(position, k, lmax))
    return spec, md, rad


def near_field(batch: ClusterBatch, s, md, radius, points, precision="fp32", interior=True, magnetic=False):
    """Scattered (+ interior) field of cluster s of a solved batch (R = 1, after
    epilogue) at points [P, 3]: device complex128 [P, 3]."""
    if batch.R != 1:
        raise ValueError("near_field expects a batch with one right-hand side")
    l = batch.layout[s]
    N, L = l["N"], l["lmax"]
    dev = batch.device
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a)).to(dev, dtype=dt)
    pos = batch.pos[l["pos_off"]: l["pos_off"] + 3 * N]
    rad = d(radius, torch.float64)
    ps = batch.p_scat[l["vec_off"]: l["vec_off"] + l["D"]]
    pi_ = batch.p_int[l["vec_off"]: l["vec_off"] + l["D"]]
    wl = 2 * np.pi * np.real(md.n_b) / np.real(md.k_b)
    k_int = d(2 * np.pi * np.asarray(md.n, complex) / wl, torch.complex128)
    hfac = -1j * np.sqrt(md.eps_b / md.mu_b) if magnetic else 1.0
    hint = d(-1j * np.sqrt(np.asarray(md.eps, complex) / np.asarray(md.mu, complex)), torch.complex128)
    P = points if isinstance(points, torch.Tensor) else d(points, torch.float64)
    out = torch.empty((P.shape[0], 3), dtype=torch.complex128, device=dev)
    fn = nat.lib().gb_near_field32 if precision == "fp32" else nat.lib().gb_near_field
    nat.check(fn(N, L, nat.ptr(pos), nat.ptr(rad), nat.ptr(ps), nat.ptr(pi_), float(np.real(md.k_b)),
                 nat.ptr(k_int), P.shape[0], nat.ptr(P), int(bool(interior)), int(bool(magnetic)),
                 float(np.real(hfac)), float(np.imag(hfac)), nat.ptr(hint), nat.ptr(out), current_stream(dev)),
              "near field")
    out._inputs = (rad, k_int, hint, P)
    return out
