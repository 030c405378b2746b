"""Drop-in GPU backend for miepy's plugin surface.

The reference dispatches its hot path to the module ``miepy.backends.jax`` when
``miepy.backends.set_backend('gpu')`` is active (backends/__init__.py:16-28) and
imports exactly three names from it:

  interactions.sphere_aggregate_tmatrix_jax(positions, mie, k)   (interactions.py:141-143)
  interactions.solve_linear_system_jax(agg_tmatrix, p_src, method) (interactions.py:81-83)
  flux.particle_cross_sections_jax(p_scat, p_inc, p_src, k)       (flux.py:21-26)

This module provides the three with the same signatures and return shapes,
computed by the CUDA extension.  ``install()`` registers them under
``miepy.backends.jax`` so that an unmodified miepy picks them up.

sphere_aggregate_tmatrix_jax returns a DeviceAggregateTMatrix: the packed matrix
stays on the GPU and solve_linear_system_jax solves it there; converting it with
numpy.asarray materialises the reference's dense [N,2,rmax,N,2,rmax] array.
"""

from __future__ import annotations

import sys
import types

import numpy as np
import torch

from . import _native as nat
from .engine import ClusterBatch, current_stream, require_cuda
from .modes import lmax_to_rmax, rmax_to_lmax

BICGSTAB_TOL = 1e-5       # the reference's BiCGSTAB tolerance
EXACT_TOL = 1e-14         # stands in for the LU branch (no LU on the GPU path)


def _is_exact(method):
    return getattr(method, "name", None) == "exact" or str(method).endswith("exact")


class DeviceAggregateTMatrix:
    """Aggregate T-matrix of a sphere cluster held on the GPU in packed form.

    The reference edits the aggregate in two places: sphere_cluster.py:704-710
    subtracts the interface's reflection matrix (``agg -= R``) and
    interactions.py:172-184 adds lattice sums entry by entry.  Arithmetic returns
    the dense matrix as a host array; item access works on a dense host copy made
    on first use, which solve_linear_system_jax then solves on the device.
    """

    def __init__(self, positions, mie, k):
        self.positions = np.asarray(positions, dtype=float).reshape(-1, 3)
        self.mie = np.asarray(mie, dtype=complex)
        self.N = self.positions.shape[0]
        self.lmax = self.mie.shape[-1]
        self.rmax = lmax_to_rmax(self.lmax)
        self.k = float(np.real(k))
        self.shape = (self.N, 2, self.rmax, self.N, 2, self.rmax)
        self.ndim = 6
        self.dtype = np.dtype(complex)
        zeros = np.zeros((self.N, 2, self.rmax), dtype=complex)
        self._batch = ClusterBatch([dict(position=self.positions, mie_scat=self.mie.reshape(self.N, 2, self.lmax),
                                         k=self.k, p_src=zeros)], R=1, precision="fp64")
        self._batch.assemble()
        self._hold = [None]   # dense host copy (shared with reshaped views), once entries are read or edited

    @property
    def size(self):
        return int(np.prod(self.shape))

    def reshape(self, *shape):
        shape = shape[0] if len(shape) == 1 and isinstance(shape[0], (tuple, list)) else shape
        if int(np.prod([s for s in shape if s != -1])) not in (self.size, 0) and -1 not in shape:
            raise ValueError(f"cannot reshape {self.shape} into {shape}")
        view = object.__new__(DeviceAggregateTMatrix)
        view.__dict__.update(self.__dict__)
        view.shape = tuple(shape)
        view.ndim = len(shape)
        return view

    def dense_device(self):
        """The reference-layout dense matrix [D, D] as a device tensor."""
        D = 2 * self.rmax * self.N
        dev = self._batch.device
        pos = torch.from_numpy(self.positions).to(dev)
        mie = torch.from_numpy(np.ascontiguousarray(self.mie.reshape(self.N, 2, self.lmax))).to(dev)
        out = torch.empty((D, D), dtype=torch.complex128, device=dev)
        nat.check(nat.lib().gb_assemble_sphere_dense(self.N, self.lmax, nat.ptr(pos), nat.ptr(mie), self.k,
                                                     nat.ptr(out), current_stream(dev)), "dense assembly")
        return out

    @property
    def _host(self):
        return self._hold[0]

    def __array__(self, dtype=None, copy=None):
        if self._host is not None:
            a = self._host.reshape(self.shape)
        else:
            a = self.dense_device().cpu().numpy().reshape(self.shape)
        return a.astype(dtype) if dtype is not None else a

    def _entries(self):
        if self._host is None:
            self._hold[0] = self.dense_device().cpu().numpy()
        return self._host.reshape(self.shape)

    def __getitem__(self, key):
        return self._entries()[key]

    def __setitem__(self, key, value):
        self._entries()[key] = value

    def __sub__(self, other):
        return np.asarray(self) - np.asarray(other)

    def __add__(self, other):
        return np.asarray(self) + np.asarray(other)

    def __rsub__(self, other):
        return np.asarray(other) - np.asarray(self)

    __radd__ = __add__
    __isub__ = __sub__
    __iadd__ = __add__


def sphere_aggregate_tmatrix_jax(positions, mie, k):
    """positions [N,3], mie [N,2,lmax], k -> T [N,2,rmax,N,2,rmax] (device-resident)."""
    require_cuda()
    mie = np.asarray(mie)
    N = np.asarray(positions).reshape(-1, 3).shape[0]
    lmax = mie.shape[-1]
    rmax = lmax_to_rmax(lmax)
    if N == 1:
        return np.zeros((1, 2, rmax, 1, 2, rmax), dtype=complex)
    return DeviceAggregateTMatrix(positions, mie, k)


def particle_aggregate_tmatrix(positions, tmatrix, k):
    """positions [N,3], tmatrix [N,2,rmax,2,rmax], k -> T_agg [N,2,rmax,N,2,rmax]
    (interactions.cpp:416-462): the translation blocks A_ij from the GPU assembler
    (unit Mie coefficients), then block (i, j) = A_ij T_j by the library's batched
    complex128 block product (gb_particle_aggregate_dense)."""
    dev = require_cuda()
    pos = np.ascontiguousarray(np.asarray(positions, dtype=float).reshape(-1, 3))
    N = pos.shape[0]
    T = np.asarray(tmatrix, dtype=complex).reshape(N, -1)
    B = int(round(np.sqrt(T.shape[1])))
    rmax = B // 2
    lmax = rmax_to_lmax(rmax)
    if N == 1:
        return np.zeros((1, 2, rmax, 1, 2, rmax), dtype=complex)
    D = B * N
    L = nat.lib()
    d_pos = torch.from_numpy(pos).to(dev)
    Tj = torch.from_numpy(np.ascontiguousarray(T.reshape(N, B, B))).to(dev)
    ws = torch.empty(L.gb_particle_aggregate_workspace_size(N, lmax), dtype=torch.uint8, device=dev)
    out = torch.empty(D * D, dtype=torch.complex128, device=dev)
    nat.check(L.gb_particle_aggregate_dense(N, lmax, nat.ptr(d_pos), nat.ptr(Tj), float(np.real(k)), nat.ptr(ws),
                                            ws.numel(), nat.ptr(out), current_stream(dev)), "particle aggregate")
    return out.view(N, 2, rmax, N, 2, rmax).cpu().numpy()


def lattice_cells(symmetry, count=5000):
    """The cell offsets [ncell, 3] a periodic symmetry sums over (interactions.py:168-169)."""
    x, y, z = symmetry.generate(count)
    return np.ascontiguousarray(np.array([x, y, z], dtype=float).T.reshape(-1, 3))


def sphere_aggregate_tmatrix_periodic(positions, mie, k, symmetry, k_hat):
    """positions [N,3], mie [N,2,lmax], k, a periodic symmetry, the source's unit wave
    vector k_hat -> T_agg [N,2,rmax,N,2,rmax] (interactions.py:153-186): the aggregate
    plus the lattice sums over symmetry.generate(5000), on the GPU
    (gb_aggregate_periodic_dense)."""
    dev = require_cuda()
    pos = np.ascontiguousarray(np.asarray(positions, dtype=float).reshape(-1, 3))
    N = pos.shape[0]
    mie = np.asarray(mie, dtype=complex).reshape(N, 2, -1)
    lmax = mie.shape[-1]
    rmax = lmax_to_rmax(lmax)
    D = 2 * rmax * N
    cells = lattice_cells(symmetry)
    kh = np.asarray(k_hat, dtype=float).reshape(3)
    d_pos = torch.from_numpy(pos).to(dev)
    d_mie = torch.from_numpy(np.ascontiguousarray(mie)).to(dev)
    d_cells = torch.from_numpy(cells).to(dev)
    out = torch.empty(D * D, dtype=torch.complex128, device=dev)
    nat.check(nat.lib().gb_aggregate_periodic_dense(N, lmax, nat.ptr(d_pos), nat.ptr(d_mie), float(np.real(k)),
                                                    nat.ptr(d_cells), cells.shape[0], float(kh[0]), float(kh[1]),
                                                    float(kh[2]), nat.ptr(out), current_stream(dev)),
              "periodic aggregate")
    return out.view(N, 2, rmax, N, 2, rmax).cpu().numpy()


def reflection_matrix_nia(positions, mie, k, reflected, z):
    """positions [N,3], mie [N,2,lmax], k, reflection coefficient, interface height z ->
    R [N,2,rmax,N,2,rmax] c128 (interactions.py:208-225 / interactions.cpp:464-512),
    computed on the GPU by gb_reflection_matrix_dense."""
    dev = require_cuda()
    pos = np.ascontiguousarray(np.asarray(positions, dtype=float).reshape(-1, 3))
    N = pos.shape[0]
    mie = np.ascontiguousarray(np.asarray(mie, dtype=complex).reshape(N, -1))
    lmax = mie.shape[1] // 2
    rmax = lmax_to_rmax(lmax)
    D = 2 * rmax * N
    d_pos = torch.from_numpy(pos).to(dev)
    d_mie = torch.from_numpy(mie).to(dev)
    out = torch.empty(D * D, dtype=torch.complex128, device=dev)
    r = complex(reflected)
    nat.check(nat.lib().gb_reflection_matrix_dense(N, lmax, nat.ptr(d_pos), nat.ptr(d_mie), float(np.real(k)), r.real,
                                                   r.imag, float(z), nat.ptr(out), current_stream(dev)),
              "reflection matrix")
    return out.cpu().numpy().reshape(N, 2, rmax, N, 2, rmax)


def _block_diagonal(M_inv_blocks, block_size, D):
    """The diagonal of M_inv_blocks [D, bs] when every block is diagonal, else None."""
    M = np.asarray(M_inv_blocks, dtype=complex).reshape(D, block_size)
    rows = np.arange(D)
    diag = M[rows, rows % block_size]
    off = M.copy()
    off[rows, rows % block_size] = 0
    return diag if not np.any(off) else None


def solve_linear_system_jax(agg_tmatrix, p_src, method, M_inv_blocks=None, block_size=0):
    """Solve p_inc = (I + T)^-1 p_src; returns numpy [N, 2, rmax].

    M_inv_blocks / block_size (optional; the reference's CPU solve_linear_system
    takes them, src/miepy/interactions.py:71-92, its GPU dispatch does not): a
    block-diagonal right preconditioner [N * bs, bs] as built by
    build_block_preconditioner_sphere / _particle (src/miepy/interactions.py:9-68).
    A diagonal one (the sphere builder's) is folded into the packed solve; any other
    runs the dense solve on (I + T) M."""
    require_cuda()
    p_src = np.asarray(p_src, dtype=complex)
    N, rmax = p_src.shape[0], p_src.shape[-1]
    D = N * 2 * rmax
    tol = EXACT_TOL if _is_exact(method) else BICGSTAB_TOL
    if M_inv_blocks is not None:
        block_size = int(block_size)
        if block_size < 1 or D % block_size or np.asarray(M_inv_blocks).size != D * block_size:
            raise ValueError(f"M_inv_blocks must be [{D}, bs] with bs dividing {D}")
    diag = _block_diagonal(M_inv_blocks, block_size, D) if M_inv_blocks is not None else None
    if isinstance(agg_tmatrix, DeviceAggregateTMatrix) and agg_tmatrix._host is None and \
            (M_inv_blocks is None or diag is not None) and agg_tmatrix.lmax <= 8:   # the packed solvers' orders
        b = agg_tmatrix._batch
        b.b.copy_(torch.from_numpy(p_src.reshape(-1)).to(b.device))
        pre = False
        if diag is not None:   # rows of the packed solve are the reference's (i, a, r) order
            pre = torch.from_numpy(np.ascontiguousarray(diag)).to(b.device)
        b.solve(tol=tol, maxiter=1000, precondition=pre)
        return b.cluster_view(0, b.x)[..., 0].cpu().numpy()
    dev = require_cuda()
    if isinstance(agg_tmatrix, DeviceAggregateTMatrix) and agg_tmatrix._host is None:
        T = agg_tmatrix.dense_device().reshape(D, D)   # assembled dense on the device
    else:   # a dense matrix supplied by the caller
        T = torch.as_tensor(np.ascontiguousarray(np.asarray(agg_tmatrix, dtype=complex).reshape(D, D))).to(dev)
    bb = torch.from_numpy(np.ascontiguousarray(p_src.reshape(-1))).to(dev)
    x = torch.empty_like(bb)
    L = nat.lib()
    st = current_stream(dev)
    Minv = None
    if M_inv_blocks is not None:
        Minv = torch.from_numpy(np.ascontiguousarray(np.asarray(M_inv_blocks, dtype=complex).reshape(-1))).to(dev)
        Tp = torch.empty_like(T)
        nat.check(L.gb_dense_precondition_matrix(D, block_size, nat.ptr(T), nat.ptr(Minv), nat.ptr(Tp), st),
                  "dense preconditioning")
        T = Tp
    need = L.gb_solve_dense_workspace_size(D, 1)
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    status = np.zeros(1, np.int32)
    iters = np.zeros(1, np.int32)
    resid = np.zeros(1)
    u = torch.empty_like(bb) if Minv is not None else x
    rc = L.gb_solve_dense(D, 1, nat.ptr(T), nat.ptr(bb), nat.ptr(u), tol, 1000, nat.ptr(ws), ws.numel(),
                          status.ctypes.data, iters.ctypes.data, resid.ctypes.data, st)
    if rc not in (nat.GB_OK, nat.GB_NOT_CONVERGED):
        nat.check(rc, "dense solve")
    if Minv is not None:
        nat.check(L.gb_block_diag_apply(D, 1, block_size, nat.ptr(Minv), nat.ptr(u), nat.ptr(x), st), "x = M u")
    return x.cpu().numpy().reshape(N, 2, rmax)


def particle_cross_sections_jax(p_scat, p_inc, p_src, k):
    """(p_scat, p_inc, p_src [2, rmax], k) -> (Cscat, Cabs, Cext), each [2, lmax]."""
    dev = require_cuda()
    arrs = [torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=complex))).to(dev) for a in (p_scat, p_inc, p_src)]
    rmax = arrs[0].shape[-1]
    lmax = rmax_to_lmax(rmax)
    out = torch.empty(6 * lmax, dtype=torch.float64, device=dev)
    nat.check(nat.lib().gb_particle_cross_sections(1, lmax, nat.ptr(arrs[0]), nat.ptr(arrs[1]), nat.ptr(arrs[2]),
                                                   float(np.real(k)), nat.ptr(out), current_stream(dev)),
              "cross sections")
    o = out.cpu().numpy().reshape(3, 2, lmax)
    return o[0], o[1], o[2]


def install():
    """Register this backend as ``miepy.backends.jax`` (the module miepy's
    set_backend('gpu') imports).  Returns the registered package module."""
    pkg = types.ModuleType("miepy.backends.jax")
    pkg.__path__ = []
    pkg.HAS_JAX = True
    inter = types.ModuleType("miepy.backends.jax.interactions")
    inter.sphere_aggregate_tmatrix_jax = sphere_aggregate_tmatrix_jax
    inter.solve_linear_system_jax = solve_linear_system_jax
    flux = types.ModuleType("miepy.backends.jax.flux")
    flux.particle_cross_sections_jax = particle_cross_sections_jax
    pkg.interactions = inter
    pkg.flux = flux
    sys.modules["miepy.backends.jax"] = pkg
    sys.modules["miepy.backends.jax.interactions"] = inter
    sys.modules["miepy.backends.jax.flux"] = flux
    backends = sys.modules.get("miepy.backends")
    if backends is not None:
        backends.jax = pkg
    return pkg
