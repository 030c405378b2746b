"""The GEMV's bounded waits, made to run out on purpose (no GPU fault involved).

The matrix stream of the packed GEMV lands in shared memory through bulk copies,
each waited for with a bounded mbarrier wait.  gb_set_gemv_wait_limit(0) makes
every consumer wait expire at once: each warp then sets the launch's error flag,
drains its own copies in flight with the default limit, and returns, and the call
reports GB_TIMEOUT.  With the default limit restored, the same batch gives the
oracle's product (complex64 bar 2e-6) and converges in a solve: the context stays
usable after the timeout.
"""

import ctypes

import numpy as np
import pytest
import torch

from miepy_gb300 import _native as nat
from miepy_gb300.engine import ClusterBatch
from oracle import oracle as O

pytestmark = pytest.mark.gpu

nm = 1e-9


def _batch(rng, N=12, lmax=3):
    pos = np.stack([np.arange(N) * 260 * nm, rng.uniform(-40, 40, N) * nm, np.zeros(N)], axis=1)
    mie = (rng.normal(size=(N, 2, lmax)) + 1j * rng.normal(size=(N, 2, lmax))) * 0.2
    k = 2 * np.pi / (600 * nm)
    rmax = lmax * (lmax + 2)
    x = rng.normal(size=(N, 2, rmax, 2)) + 1j * rng.normal(size=(N, 2, rmax, 2))
    return pos, mie, k, x


def test_expired_gemv_wait_reports_timeout_and_context_recovers():
    L = nat.lib()
    rng = np.random.default_rng(3)
    pos, mie, k, x = _batch(rng)
    N = pos.shape[0]
    b = ClusterBatch([dict(position=pos, mie_scat=mie, k=k, p_src=x)], R=2, precision="mixed").assemble()
    xd = torch.from_numpy(x.reshape(-1)).to(b.device)
    prev = ctypes.c_longlong(0)
    nat.check(L.gb_set_gemv_wait_limit(0, ctypes.byref(prev)))
    try:
        assert prev.value > 0
        with pytest.raises(nat.GBError) as ei:
            b.apply(xd, "fp32")
        assert ei.value.code == nat.GB_TIMEOUT
        assert "wait limit" in nat.last_error()
    finally:
        nat.check(L.gb_set_gemv_wait_limit(-1, None))
    cur = ctypes.c_longlong(0)
    nat.check(L.gb_set_gemv_wait_limit(-1, ctypes.byref(cur)))
    assert cur.value == prev.value
    # the context is usable: the same product now matches the oracle, and a solve converges
    T = O.sphere_aggregate_tmatrix(pos, mie.reshape(N, -1), k)
    D = T.shape[0]
    xs = x.reshape(D, 2)
    ref = np.stack([O.gemv(T, xs[:, r]) + xs[:, r] for r in range(2)], axis=1)
    y = b.apply(xd, "fp32").cpu().numpy().reshape(D, 2)
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 2e-6
    b.solve(tol=1e-8, maxiter=500)
    assert np.all(np.asarray(b.status) == 0)
    torch.cuda.synchronize()
