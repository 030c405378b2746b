"""The no-allocation dense solve against the workspace dense solve.

gb_solve_dense_noalloc runs the same FP64 BiCGSTAB as gb_solve_dense in a fixed
device scratch array instead of a caller workspace.  Two calls in a row (of
different sizes, so that the second meets the first one's leftovers in the shared
array) must each agree with gb_solve_dense on the same input within the dense
solve's bar: rtol 1e-10, atol 1e-14 of the largest coefficient.
"""

import numpy as np
import pytest
import torch

from miepy_gb300 import _native as nat
from miepy_gb300.engine import current_stream
from tests import _golden as G

pytestmark = pytest.mark.gpu

EXACT_TOL = 1e-14


def _dense_inputs(name, R):
    g = G.load(name)
    p_src = np.asarray(g["p_src"], dtype=complex)
    D = p_src.size
    T = np.ascontiguousarray(np.asarray(g["agg_tmatrix"], dtype=complex).reshape(D, D))
    b = np.stack([p_src.reshape(-1) * (1.0 + 0.5j * q) for q in range(R)], axis=1)   # [D][R]
    return D, T, np.ascontiguousarray(b)


def _solve_workspace(L, dev, D, R, T, b):
    x = torch.empty_like(b)
    ws = torch.empty(L.gb_solve_dense_workspace_size(D, R), dtype=torch.uint8, device=dev)
    status = np.zeros(R, np.int32)
    rc = L.gb_solve_dense(D, R, nat.ptr(T), nat.ptr(b), nat.ptr(x), EXACT_TOL, 1000, nat.ptr(ws), ws.numel(),
                          status.ctypes.data, None, None, current_stream(dev))
    assert rc in (nat.GB_OK, nat.GB_NOT_CONVERGED), nat.last_error()
    torch.cuda.synchronize(dev)
    return x.cpu().numpy()


def _solve_noalloc(L, dev, D, R, T, b):
    x = torch.full_like(b, complex(np.nan, np.nan))
    status = np.zeros(R, np.int32)
    iters = np.zeros(R, np.int32)
    resid = np.zeros(R)
    rc = L.gb_solve_dense_noalloc(D, R, nat.ptr(T), nat.ptr(b), nat.ptr(x), EXACT_TOL, 1000, status.ctypes.data,
                                  iters.ctypes.data, resid.ctypes.data, current_stream(dev))
    assert rc in (nat.GB_OK, nat.GB_NOT_CONVERGED), nat.last_error()
    torch.cuda.synchronize(dev)
    assert np.all(iters > 0)
    return x.cpu().numpy()


def test_noalloc_dense_solve_matches_workspace_solve():
    L = nat.lib()
    dev = torch.device("cuda:0")
    torch.cuda.set_device(dev)
    # two calls in a row: a larger system with two right-hand sides, then a smaller one
    for name, R in (("dimer_lmax6_exact", 2), ("ag5_lmax2_exact", 1)):
        D, Tn, bn = _dense_inputs(name, R)
        T = torch.from_numpy(Tn).to(dev)
        b = torch.from_numpy(bn).to(dev)
        ref = _solve_workspace(L, dev, D, R, T, b)
        got = _solve_noalloc(L, dev, D, R, T, b)
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-14 * np.max(np.abs(ref)))


def test_noalloc_rejects_oversize():
    L = nat.lib()
    dev = torch.device("cuda:0")
    z = torch.zeros(1, dtype=torch.complex128, device=dev)
    rc = L.gb_solve_dense_noalloc(8193, 1, nat.ptr(z), nat.ptr(z), nat.ptr(z), 1e-8, 10, None, None, None,
                                  current_stream(dev))
    assert rc == nat.GB_OVER_BUDGET
    assert "limit" in nat.last_error()
