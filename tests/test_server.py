"""Continuous-batching solve server.

CPU: admission in arrival order within the HBM budget, over-budget rejection, one
medium per wave, the request generator of the serving workload, and host-side fault
injection through a server whose wave execution is replaced by a fake: a failing
wave re-admits its requests, persistent failure reaches the caller, cancelled
requests are dropped, non-finite inputs are rejected, metrics are streamed.
GPU: every result is the same alone and in the mix (tolerance: C_ext within 1e-8
relative, p_inc within 1e-8 of its largest coefficient, at solve tolerance 1e-10),
with waves overlapping on the device; Gaussian-beam and plane-wave requests mixed.
"""

import collections
import concurrent.futures as cf
import json
import threading
import time

import numpy as np
import pytest

from miepy_gb300 import server as SV


def _bare_server(budget, max_wave_requests=8, precision="mixed", small_bytes=1 << 62, cost_spread=float("inf"),
                 max_wait_s=0.5, max_waves=3):
    s = object.__new__(SV.SolveServer)
    s.budget = budget
    s.max_wave_requests = max_wave_requests
    s.precision = precision
    s.small_bytes, s.cost_spread, s.max_wait_s, s.max_waves = small_bytes, cost_spread, max_wait_s, max_waves
    s._large_running = 0
    s._pending = collections.deque()
    s._in_use = 0
    s.stats = dict(admitted=0, completed=0, rejected=0, waves=0, peak_bytes=0, max_concurrent_waves=0,
                   failed_waves=0, readmitted=0, cancelled=0)
    return s


def _req(N, L, rid, medium=1.0):
    return SV.ClusterRequest(position=np.arange(3 * N, dtype=float).reshape(N, 3) * 1e-6, radius=50e-9,
                             index=1.5, wavelength=600e-9, lmax=L, medium_index=medium, rid=rid)


def test_admission_fifo_budget_and_rejection():
    reqs = [_req(20, 3, 0), _req(30, 4, 1), _req(400, 8, 2), _req(10, 2, 3)]
    need = [SV.request_footprint(r, "mixed") for r in reqs]
    s = _bare_server(budget=need[0] + need[1] + need[3])
    futs = []
    for r in reqs:
        f = cf.Future()
        futs.append(f)
        s._pending.append((r, f, 0.0, 0))
    wave, used, _ = s._take_wave()
    assert [w[0].rid for w in wave] == [0, 1, 3]       # request 2 exceeds the whole budget ...
    assert used == need[0] + need[1] + need[3]
    assert isinstance(futs[2].exception(timeout=0), SV.OverBudget)  # ... and is rejected
    assert s.stats["rejected"] == 1
    assert not s._pending
    s2 = _bare_server(budget=need[0] + need[1])
    for r in (reqs[0], reqs[1], reqs[3]):
        s2._pending.append((r, cf.Future(), 0.0, 0))
    wave, used, _ = s2._take_wave()
    assert [w[0].rid for w in wave] == [0, 1]          # request 3 waits: the budget is used up
    s2._in_use = used - need[0]                         # request 0's wave finished
    wave, used, _ = s2._take_wave()
    assert [w[0].rid for w in wave] == [3]


def test_admission_waits_for_memory_and_splits_media():
    a, b = _req(40, 5, 0), _req(40, 5, 1)
    na = SV.request_footprint(a, "mixed")
    s = _bare_server(budget=int(1.5 * na))
    for r in (a, b):
        s._pending.append((r, cf.Future(), 0.0, 0))
    wave, used, _ = s._take_wave()
    assert [w[0].rid for w in wave] == [0]
    s._in_use = used
    wave, _, _ = s._take_wave()
    assert wave == []                                   # request 1 waits for request 0's memory
    s2 = _bare_server(budget=10 * na)
    for r in (_req(10, 3, 0, 1.0), _req(10, 3, 1, 1.33), _req(10, 3, 2, 1.0)):
        s2._pending.append((r, cf.Future(), 0.0, 0))
    wave, _, _ = s2._take_wave()
    assert [w[0].rid for w in wave] == [0, 2]           # one medium per wave ...
    wave, _, _ = s2._take_wave()
    assert [w[0].rid for w in wave] == [1]              # ... the other one next


def test_admission_size_classes_spread_and_age_bound():
    small, large = _req(10, 3, 0), _req(300, 6, 1)
    ns, nl = SV.request_footprint(small, "mixed"), SV.request_footprint(large, "mixed")
    # classes: a large request (older) and small ones never share a wave
    s = _bare_server(budget=10 * nl, small_bytes=(ns + nl) // 2)
    for r, t in ((large, 0.0), (small, 1.0), (_req(12, 3, 2), 2.0)):
        s._pending.append((r, cf.Future(), t, 0))
    wave, _, cls = s._take_wave()
    assert [w[0].rid for w in wave] == [1] and cls == 1
    wave, _, cls = s._take_wave()
    assert [w[0].rid for w in wave] == [0, 2] and cls == 0
    # large waves keep a slot free for small ones: with max_waves - 1 large waves running,
    # a later small request goes first
    s = _bare_server(budget=10 * nl, small_bytes=(ns + nl) // 2, max_waves=3)
    s._large_running = 2
    for r, t in ((large, 0.0), (small, 1.0)):
        s._pending.append((r, cf.Future(), t, 0))
    wave, _, cls = s._take_wave()
    assert [w[0].rid for w in wave] == [0] and cls == 0
    # cost spread: a request far smaller than the wave's first waits for its own wave
    s = _bare_server(budget=10 * nl, cost_spread=4.0)
    for r, t in ((large, 0.0), (small, 1.0), (_req(280, 6, 3), 2.0)):
        s._pending.append((r, cf.Future(), t, 0))
    wave, _, _ = s._take_wave()
    assert [w[0].rid for w in wave] == [1, 3]
    # skip-ahead: a request that does not fit is passed by a later one that does, until
    # it has waited max_wait_s
    now = SV.time.perf_counter()
    s = _bare_server(budget=nl + ns, max_wait_s=0.5)
    s._in_use = 2 * ns                                # free: nl - ns, too little for the large one
    for r, t in ((large, now), (small, now + 0.001)):
        s._pending.append((r, cf.Future(), t, 0))
    wave, _, _ = s._take_wave()
    assert [w[0].rid for w in wave] == [0]            # the small one passes the young large head
    s = _bare_server(budget=nl + ns, max_wait_s=0.5)
    s._in_use = 2 * ns                                # free: nl - ns, too little for the large one
    for r, t in ((large, now - 1.0), (small, now)):
        s._pending.append((r, cf.Future(), t, 0))
    wave, _, _ = s._take_wave()
    assert wave == []                                 # the old head keeps its place


def test_request_generator():
    rng = np.random.default_rng(4)
    Ns, Ls, beams = [], [], 0
    for i in range(60):
        r = SV.random_request(rng, rid=i, n_range=(2, 60))
        pos, rad = np.asarray(r.position), np.asarray(r.radius)
        d = np.linalg.norm(pos[:, None] - pos[None], axis=-1)
        np.fill_diagonal(d, np.inf)
        assert np.all(d > rad[:, None] + rad[None])
        assert 1.3 <= np.real(r.index) <= 2.5 and 0 <= np.imag(r.index) <= 0.1
        Ns.append(len(rad))
        Ls.append(r.lmax)
        beams += type(r.source).__name__ == "gaussian_beam"
    assert min(Ns) >= 2 and max(Ns) <= 60 and set(Ls) <= set(range(2, 9))
    assert 10 < beams < 50


class FakeServer(SV.SolveServer):
    """The dispatcher, admission and fault handling of SolveServer with the GPU
    work replaced by a fake that answers after a short delay."""

    delay = 0.02

    def _setup_device(self, device, hbm_budget):
        self.device = None
        return hbm_budget

    def _make_streams(self):
        return [None] * self.max_waves

    def _execute(self, wave, sidx):
        time.sleep(self.delay)
        return [SV.ClusterResult(rid=w[0].rid, status=0, passes=1, C_sca=1.0, C_abs=0.0, C_ext=1.0 + w[0].rid,
                                 p_inc=np.zeros((1, 2, 3)), force=np.zeros((1, 3)), torque=np.zeros((1, 3)))
                for w in wave]


def test_failed_wave_readmits_its_requests(tmp_path):
    calls = []

    def hook(wid, reqs):
        calls.append(wid)
        if wid == 0:
            raise MemoryError("injected allocation failure")

    metrics = tmp_path / "metrics.jsonl"
    with FakeServer(hbm_budget=10 ** 12, max_waves=1, max_wave_requests=4, fault_hook=hook,
                    metrics_path=str(metrics)) as srv:
        futs = [srv.submit(_req(5, 2, i)) for i in range(6)]
        res = [f.result(timeout=30) for f in futs]
        stats = dict(srv.stats)
    assert [r.rid for r in res] == list(range(6))
    assert [r.C_ext for r in res] == [1.0 + i for i in range(6)]
    assert stats["failed_waves"] == 1 and stats["readmitted"] >= 1
    assert stats["completed"] == 6 and srv._in_use == 0
    lines = [json.loads(l) for l in metrics.read_text().splitlines()]
    assert sorted(l["rid"] for l in lines) == list(range(6))
    assert all(l["latency_ms"] >= l["wait_ms"] >= 0 for l in lines)


def test_persistent_failure_reaches_the_caller():
    def hook(wid, reqs):
        raise RuntimeError("injected")

    with FakeServer(hbm_budget=10 ** 12, max_waves=2, max_retries=2, fault_hook=hook) as srv:
        f = srv.submit(_req(5, 2, 0))
        with pytest.raises(RuntimeError, match="injected"):
            f.result(timeout=30)
        assert srv.stats["readmitted"] == 2          # two re-admissions, then the error
    assert srv._in_use == 0


def test_cancelled_requests_are_dropped():
    class Slow(FakeServer):
        delay = 0.3

    with Slow(hbm_budget=10 ** 12, max_waves=1, max_wave_requests=1) as srv:
        first = srv.submit(_req(5, 2, 0))
        time.sleep(0.05)                             # request 0 is on the (fake) GPU
        queued = [srv.submit(_req(5, 2, i)) for i in (1, 2)]
        assert queued[0].cancel()
        assert first.result(timeout=30).rid == 0
        assert queued[1].result(timeout=30).rid == 2
        assert queued[0].cancelled()
        assert srv.stats["cancelled"] == 1


def test_non_finite_inputs_rejected_at_submit():
    with FakeServer(hbm_budget=10 ** 12) as srv:
        bad = _req(4, 2, 0)
        bad.position[1, 2] = np.nan
        with pytest.raises(ValueError, match="non-finite position"):
            srv.submit(bad)
        with pytest.raises(ValueError, match="lmax"):
            srv.submit(_req(4, 9, 1))
        r = _req(4, 2, 2)
        r.index = complex(np.inf, 0)
        with pytest.raises(ValueError, match="non-finite index"):
            srv.submit(r)


@pytest.mark.gpu
def test_results_same_alone_and_in_the_mix():
    rng = np.random.default_rng(4)
    reqs = [SV.random_request(rng, rid=i, n_range=(2, 40), lmax_range=(2, 5)) for i in range(12)]
    kw = dict(precision="mixed", tol=1e-10, inner_tol=1e-6)
    with SV.SolveServer(max_waves=3, max_wave_requests=3, **kw) as srv:
        futs = [srv.submit(r) for r in reqs]
        mix = [f.result(timeout=600) for f in futs]
        stats = dict(srv.stats)
    assert stats["admitted"] == stats["completed"] == 12
    assert stats["waves"] >= 4
    alone = []
    with SV.SolveServer(max_waves=1, max_wave_requests=1, **kw) as srv:
        for r in reqs:
            alone.append(srv.submit(r).result(timeout=600))
    for a, m in zip(alone, mix):
        assert a.status == 0 and m.status == 0
        assert abs(a.C_ext - m.C_ext) <= 1e-8 * abs(a.C_ext)
        assert np.max(np.abs(a.p_inc - m.p_inc)) <= 1e-8 * np.max(np.abs(a.p_inc))
        np.testing.assert_allclose(m.force, a.force, rtol=1e-6, atol=1e-6 * np.max(np.abs(a.force)))


@pytest.mark.gpu
def test_server_against_fp64_single_cluster():
    """A served request equals the sphere_cluster FP64 solve of the same cluster."""
    import miepy_gb300 as gb
    rng = np.random.default_rng(5)
    r = SV.random_request(rng, rid=0, n_range=(8, 12), lmax_range=(3, 3))
    with SV.SolveServer(precision="mixed", tol=1e-10) as srv:
        res = srv.submit(r).result(timeout=600)
    c = gb.sphere_cluster(position=r.position, radius=r.radius, material=gb.constant_material(index=r.index),
                          source=r.source, wavelength=r.wavelength, lmax=r.lmax, method=gb.solver.exact)
    C = c.cross_sections()
    assert abs(res.C_ext - C.extinction) <= 1e-8 * abs(C.extinction)
    assert np.max(np.abs(res.p_inc - c.p_inc)) <= 1e-8 * np.max(np.abs(c.p_inc))


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_nan_right_hand_side_reported_per_cluster(precision):
    """A NaN in one cluster's source is reported as that cluster's status (GB_NAN),
    without an error for the call, and its batch-mate still converges."""
    from miepy_gb300 import _native as nat
    from miepy_gb300.engine import ClusterBatch
    rng = np.random.default_rng(6)
    s1 = SV.request_spec(SV.random_request(rng, rid=0, n_range=(6, 8), lmax_range=(3, 3)))
    s2 = SV.request_spec(SV.random_request(rng, rid=1, n_range=(6, 8), lmax_range=(3, 3)))
    s2["p_src"] = np.array(s2["p_src"])
    s2["p_src"][0, 0, 0] = np.nan
    b = ClusterBatch([s1, s2], R=1, precision=precision)
    b.assemble()
    b.solve(tol=1e-8)
    assert b.status[0] == nat.GB_OK
    assert b.status[1] == nat.GB_NAN


@pytest.mark.gpu
def test_ill_conditioned_lmax8_beam_request_converges():
    """Request 16 of the serving stream (seed 4): N=40, lmax 8, Gaussian beam, a
    system on which FP32 BiCGSTAB stalls unless its inner products are accumulated
    beyond FP32 (they cancel as the residual falls).  Mixed must converge and give
    C_ext within 1e-6 of FP64."""
    rng = np.random.default_rng(4)
    reqs = [SV.random_request(rng, rid=i) for i in range(17)]
    r = reqs[16]
    assert (len(r.radius), r.lmax) == (40, 8)
    out = {}
    for prec in ("mixed", "fp64"):
        with SV.SolveServer(precision=prec, tol=1e-8, max_waves=1, max_wave_requests=1) as srv:
            out[prec] = srv.submit(r).result()
    assert out["mixed"].status == 0 and out["fp64"].status == 0
    assert abs(out["mixed"].C_ext - out["fp64"].C_ext) / abs(out["fp64"].C_ext) < 1e-6


def test_priority_level_by_wave_cost():
    lv = SV.SolveServer._priority_level
    # six levels (priorities 0 .. -5): the highest for <= 64 MB, one lower per factor 8
    assert lv(1 << 20, 6) == 5 and lv(64 << 20, 6) == 5
    assert lv((64 << 20) + 1, 6) == 4 and lv(512 << 20, 6) == 4
    assert lv(4 << 30, 6) == 3 and lv(30 << 30, 6) == 2
    assert lv(1 << 50, 6) == 0
    assert lv(1 << 50, 1) == 0 and lv(1, 2) == 1


def test_random_request_source_kind_keeps_the_stream():
    a = [SV.random_request(np.random.default_rng(9), rid=i, n_range=(2, 6)) for i in range(3)]
    g = [SV.random_request(np.random.default_rng(9), rid=i, n_range=(2, 6), source_kind="gaussian") for i in range(3)]
    p = [SV.random_request(np.random.default_rng(9), rid=i, n_range=(2, 6), source_kind="plane") for i in range(3)]
    for x, y, z in zip(a, g, p):
        assert np.array_equal(x.position, y.position) and np.array_equal(x.position, z.position)
        assert x.lmax == y.lmax == z.lmax and x.index == y.index
        assert type(y.source).__name__ == "gaussian_beam" and type(z.source).__name__ == "plane_wave"
