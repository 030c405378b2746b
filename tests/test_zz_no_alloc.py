"""The no-allocation dense solve against the workspace dense solve and the reference.

gb_solve_dense_noalloc runs the same FP64 BiCGSTAB as gb_solve_dense in a fixed
device scratch array instead of a caller workspace.  It is for callers that cannot
allocate device memory (HBM reserved up front, or loops in which cudaMalloc/cudaFree
would synchronise the device).  Two calls in a row (of different sizes, so that the
second meets the first one's leftovers in the shared array) must each agree with
gb_solve_dense on the same input and with the p_inc of the reference's exact solve
in the golden fixture (right-hand side q is p_src (1 + 0.5i q), so its solution is
p_inc (1 + 0.5i q)), within the dense solve's bar: rtol 1e-10, atol 1e-14 of the
largest coefficient.  Repeated calls leave the device's free memory and the torch
allocator's reservation unchanged.
"""

import numpy as np
import pytest
import torch

from miepy_gb300 import _native as nat
from miepy_gb300.engine import current_stream
from tests import _golden as G

pytestmark = pytest.mark.gpu

EXACT_TOL = 1e-14
CASES = (("dimer_lmax6_exact", 2), ("ag5_lmax2_exact", 1))   # a larger system with two right-hand sides, then a smaller


def _dense_inputs(name, R):
    g = G.load(name)
    p_src = np.asarray(g["p_src"], dtype=complex)
    D = p_src.size
    T = np.ascontiguousarray(np.asarray(g["agg_tmatrix"], dtype=complex).reshape(D, D))
    scale = np.array([1.0 + 0.5j * q for q in range(R)])
    b = p_src.reshape(-1, 1) * scale[None, :]                       # [D][R]
    want = np.asarray(g["p_inc"], dtype=complex).reshape(-1, 1) * scale[None, :]
    return D, T, np.ascontiguousarray(b), want


def _solve_workspace(L, dev, D, R, T, b):
    x = torch.empty_like(b)
    ws = torch.empty(L.gb_solve_dense_workspace_size(D, R), dtype=torch.uint8, device=dev)
    status = np.zeros(R, np.int32)
    rc = L.gb_solve_dense(D, R, nat.ptr(T), nat.ptr(b), nat.ptr(x), EXACT_TOL, 1000, nat.ptr(ws), ws.numel(),
                          status.ctypes.data, None, None, current_stream(dev))
    assert rc in (nat.GB_OK, nat.GB_NOT_CONVERGED), nat.last_error()
    torch.cuda.synchronize(dev)
    return x.cpu().numpy()


def _noalloc_call(L, dev, D, R, T, b, x):
    status = np.zeros(R, np.int32)
    iters = np.zeros(R, np.int32)
    resid = np.zeros(R)
    rc = L.gb_solve_dense_noalloc(D, R, nat.ptr(T), nat.ptr(b), nat.ptr(x), EXACT_TOL, 1000, status.ctypes.data,
                                  iters.ctypes.data, resid.ctypes.data, current_stream(dev))
    assert rc in (nat.GB_OK, nat.GB_NOT_CONVERGED), nat.last_error()
    torch.cuda.synchronize(dev)
    assert np.all(iters > 0)


def test_noalloc_dense_solve_matches_workspace_solve_and_reference():
    L = nat.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    for name, R in CASES:
        D, Tn, bn, want = _dense_inputs(name, R)
        T = torch.from_numpy(Tn).to(dev)
        b = torch.from_numpy(bn).to(dev)
        ref = _solve_workspace(L, dev, D, R, T, b)
        x = torch.full_like(b, complex(np.nan, np.nan))
        _noalloc_call(L, dev, D, R, T, b, x)
        got = x.cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-14 * np.max(np.abs(ref)))
        np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14 * np.max(np.abs(want)))


def test_noalloc_calls_leave_device_memory_unchanged():
    L = nat.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    bufs = []
    for name, R in CASES:   # every input and output exists before the measured calls
        D, Tn, bn, _ = _dense_inputs(name, R)
        b = torch.from_numpy(bn).to(dev)
        bufs.append((D, R, torch.from_numpy(Tn).to(dev), b, torch.empty_like(b)))
    for D, R, T, b, x in bufs:   # warm-up: modules and kernels of both sizes loaded
        _noalloc_call(L, dev, D, R, T, b, x)
    free0, _ = torch.cuda.mem_get_info(dev)
    reserved0 = torch.cuda.memory_reserved(dev)
    for _ in range(2):
        for D, R, T, b, x in bufs:
            _noalloc_call(L, dev, D, R, T, b, x)
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0, f"device free memory changed by {free0 - free1} B"
    assert torch.cuda.memory_reserved(dev) == reserved0


def test_noalloc_rejects_oversize():
    L = nat.lib()
    dev = torch.device("cuda:0")
    z = torch.zeros(1, dtype=torch.complex128, device=dev)
    rc = L.gb_solve_dense_noalloc(8193, 1, nat.ptr(z), nat.ptr(z), nat.ptr(z), 1e-8, 10, None, None, None,
                                  current_stream(dev))
    assert rc == nat.GB_OVER_BUDGET
    assert "limit" in nat.last_error()
