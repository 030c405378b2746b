"""The GEMV's bounded waits, made to run out on purpose (no GPU fault involved).

The matrix stream of the packed GEMV lands in shared memory through bulk copies,
each waited for with a bounded mbarrier wait.  gb_set_gemv_wait_limit(0) makes
every consumer wait expire at once: each warp then sets the launch's error flag,
drains its own copies in flight with the default limit, and returns, and the call
reports GB_TIMEOUT.  With the default limit restored, the same batch gives the
oracle's product (complex64 bar 2e-6) and converges in a solve: the context stays
usable after the timeout (12-sphere cluster of the golden fixtures, two
right-hand sides).
"""

import ctypes

import numpy as np
import pytest
import torch

from miepy_gb300 import _native as nat
from miepy_gb300.engine import ClusterBatch
from oracle import oracle as O
from tests import _golden as G

pytestmark = pytest.mark.gpu



def test_expired_gemv_wait_reports_timeout_and_context_recovers():
    L = nat.lib()
    g = G.load("rand12_lmax3_exact")   # 12 spheres, lmax 3: a physical cluster from the reference
    pos, mie, k = g["position"], g["mie_scat"], float(g["k_b"])
    N = pos.shape[0]
    p_src = np.stack([g["p_src"], g["p_src"] * (1 - 0.5j)], axis=-1)
    b = ClusterBatch([dict(position=pos, mie_scat=mie, k=k, p_src=p_src)], R=2, precision="mixed").assemble()
    xd = b.b.clone()
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
    # the context is usable: the same product now matches the oracle, and a solve
    # reaches the reference's exact solution
    T = O.sphere_aggregate_tmatrix(pos, mie.reshape(N, -1), k)
    D = T.shape[0]
    xs = p_src.reshape(D, 2)
    ref = np.stack([O.gemv(T, xs[:, r]) + xs[:, r] for r in range(2)], axis=1)
    y = b.apply(xd, "fp32").cpu().numpy().reshape(D, 2)
    assert np.max(np.abs(y - ref)) / np.max(np.abs(ref)) < 2e-6
    b.solve(tol=1e-10, maxiter=1000)
    assert np.all(np.asarray(b.status) == 0)
    x = b.cluster_view(0, b.x).cpu().numpy()
    want = np.stack([g["p_inc"], g["p_inc"] * (1 - 0.5j)], axis=-1)
    assert np.max(np.abs(x - want)) / np.max(np.abs(want)) < 1e-8
