"""Continuous-batching solve server for sphere-cluster requests on one GPU.

Requests (a cluster, a wavelength, an lmax and a source) arrive at any time.  A
dispatcher thread admits waiting requests against an HBM budget (the footprint of
each request's matrices, vectors and solver scratch) and a number of wave slots,
by size class and in arrival order within a class (SolveServer, _take_wave).  Everything admitted together forms a wave: one ragged ClusterBatch
that is assembled, solved (all clusters advance through the same masked kernels;
finished ones drop out) and reduced to observables in one sequence of launches on
the wave's own CUDA stream.  Up to ``max_waves`` waves are on the GPU at once, so
requests that arrive while others are being solved are admitted as soon as memory
and a slot free up, and their work overlaps on the device with the waves already
running.  Each request's result is that of its own cluster: clusters in a batch
share launches, never arithmetic.

The reference has no server; a user would loop over ``sphere_cluster`` objects
(sphere_cluster.py:27-125), one solve at a time.
"""

from __future__ import annotations

import collections
import concurrent.futures as cf
import json
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .engine import ClusterBatch, footprint_bytes, require_cuda
from .materials import constant_material, material_struct
from .mie import mie_coefficients
from .modes import lmax_to_rmax
from .sources import plane_wave


@dataclass
class ClusterRequest:
    position: np.ndarray                 # [N, 3] m
    radius: object                       # [N] or scalar, m
    index: object                        # particle refractive index (complex, [N] or scalar)
    wavelength: float                    # m
    lmax: int
    source: object = None                # plane_wave / gaussian_beam (default: x-polarised plane wave)
    medium_index: float = 1.0            # non-absorbing medium
    rid: int = -1


@dataclass
class ClusterResult:
    rid: int
    status: int
    passes: int                          # refinement passes (mixed) or BiCGSTAB iterations (fp64)
    C_sca: float
    C_abs: float
    C_ext: float
    p_inc: np.ndarray                    # [N, 2, rmax]
    force: np.ndarray                    # [N, 3]
    torque: np.ndarray                   # [N, 3]
    t_submit: float = 0.0
    t_admit: float = 0.0
    t_done: float = 0.0
    wave: int = -1
    wave_size: int = 0

    @property
    def latency(self):
        return self.t_done - self.t_submit


class OverBudget(RuntimeError):
    """A request larger than the whole HBM budget."""


def validate_request(req: ClusterRequest):
    """Rejects requests that the solver could only answer with NaN: non-finite
    positions, radii, indices or wavelength, non-positive sizes, lmax out of 1..8."""
    pos = np.asarray(np.atleast_2d(req.position), float)
    if pos.ndim != 2 or pos.shape[1] != 3 or pos.shape[0] < 1:
        raise ValueError(f"request {req.rid}: position must be [N, 3]")
    arrays = dict(position=pos, radius=np.asarray(req.radius, float), index=np.asarray(req.index, complex),
                  wavelength=np.asarray(req.wavelength, float), medium_index=np.asarray(req.medium_index, float))
    for name, a in arrays.items():
        if not np.all(np.isfinite(a)):
            raise ValueError(f"request {req.rid}: non-finite {name}")
    if np.any(arrays["radius"] <= 0) or req.wavelength <= 0 or req.medium_index <= 0:
        raise ValueError(f"request {req.rid}: radius, wavelength and medium index must be positive")
    if not (1 <= int(req.lmax) <= 8):
        raise ValueError(f"request {req.rid}: lmax must be in 1..8")


def request_spec(req: ClusterRequest):
    """Host inputs of one request: Mie coefficients, wavenumber and p_src."""
    pos = np.asarray(np.atleast_2d(req.position), float)
    N = pos.shape[0]
    radius = np.broadcast_to(np.asarray(req.radius, float), (N,))
    mat = [constant_material(index=complex(i)) for i in np.broadcast_to(np.asarray(req.index, complex), (N,))]
    medium = constant_material(index=float(req.medium_index))
    md = material_struct(np.asarray(mat, dtype=object), medium, wavelength=req.wavelength)
    ms, mi = mie_coefficients(radius, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, int(req.lmax))
    k = float(np.real(md.k_b))
    src = req.source if req.source is not None else plane_wave.from_string("x")
    p_src = src.structure(pos, k, int(req.lmax))
    return dict(position=pos, mie_scat=ms, mie_int=mi, k=k, p_src=p_src, eps_b=float(np.real(md.eps_b)))


def request_footprint(req: ClusterRequest, precision):
    N = np.asarray(np.atleast_2d(req.position)).shape[0]
    return footprint_bytes(N, int(req.lmax), 1, precision)


class SolveServer:
    """Admits, batches and solves cluster requests; ``submit`` returns a Future of
    a ClusterResult."""

    def __init__(self, hbm_budget=None, max_waves=3, max_wave_requests=64, precision="mixed", tol=1e-8,
                 inner_tol=1e-4, maxiter=1000, device=None, max_retries=2, fault_hook=None, metrics_path=None,
                 small_bytes=1 << 30, cost_spread=16.0, max_wait_s=0.5):
        """max_retries: times a request whose wave failed (an exception on the host,
        e.g. an allocation failure) is re-admitted before its Future gets the error.
        fault_hook(wave_id, requests): called at the start of every wave; an exception
        it raises fails that wave (fault injection for tests).  metrics_path: JSONL
        file receiving one line per finished request.

        Admission (see _take_wave): requests of footprint <= small_bytes are small,
        the others large; a wave holds one class, and requests whose footprints lie
        within a factor cost_spread of its first request's, so that no request waits
        on a much larger one in its own wave; large waves hold at most max_waves - 1
        slots, so small requests always find one.  Within a class, requests that do
        not fit the free budget are passed over by later ones, except the class's
        oldest once it has waited max_wait_s: then nothing passes it."""
        self.max_retries = int(max_retries)
        self.fault_hook = fault_hook
        self.metrics_path = metrics_path
        self._metrics_lock = threading.Lock()
        hbm_budget = self._setup_device(device, hbm_budget)
        self.budget = int(hbm_budget)
        self.max_waves = int(max_waves)
        self.max_wave_requests = int(max_wave_requests)
        self.precision = precision
        self.tol, self.inner_tol, self.maxiter = float(tol), float(inner_tol), int(maxiter)
        self.small_bytes, self.cost_spread, self.max_wait_s = int(small_bytes), float(cost_spread), float(max_wait_s)
        self._pending = collections.deque()
        self._cv = threading.Condition()
        self._in_use = 0
        self._waves_running = 0
        self._large_running = 0
        self._wave_counter = 0
        self._closing = False
        self._free_streams = list(range(self.max_waves))
        self._slot_class = {}
        self._slot_cost = {}
        self._streams = self._make_streams()
        # persistent workers: the native library keeps per-thread staging buffers
        # and capture streams, reused wave after wave
        self._pool = cf.ThreadPoolExecutor(max_workers=self.max_waves, thread_name_prefix="miepy-gb300-wave")
        self.stats = dict(admitted=0, completed=0, rejected=0, waves=0, peak_bytes=0, max_concurrent_waves=0,
                          failed_waves=0, readmitted=0, cancelled=0)
        self._dispatcher = threading.Thread(target=self._dispatch, name="miepy-gb300-dispatch", daemon=True)
        self._dispatcher.start()

    def _setup_device(self, device, hbm_budget):
        self.device = require_cuda(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(0.8 * free)
        return hbm_budget

    def _make_streams(self):
        """Per wave slot one stream at every priority the device offers, lowest
        first.  A wave runs on the stream whose priority matches its cost (see
        _priority_level): when waves of different sizes wait for SMs, the CTAs of the
        cheaper one are dispatched first, so a small request is not held behind a
        large one's kernels."""
        lo, hi = torch.cuda.Stream.priority_range() if hasattr(torch.cuda.Stream, "priority_range") else (0, -1)
        step = -1 if hi < lo else 1
        return [[torch.cuda.Stream(device=self.device, priority=p) for p in range(lo, hi + step, step)]
                for _ in range(self.max_waves)]

    @staticmethod
    def _priority_level(cost, levels):
        """Index into a slot's streams (0 = lowest priority) for a wave of cost bytes:
        one level per factor of 8 in footprint, the highest at <= 64 MB."""
        if levels <= 1:
            return 0
        k = 0
        c = 64 << 20
        while cost > c and k < levels - 1:
            c *= 8
            k += 1
        return levels - 1 - k

    # --------------------------------------------------------------- client --
    def submit(self, req: ClusterRequest) -> cf.Future:
        """Queues a request; raises ValueError for inputs that cannot be solved
        (see validate_request).  Cancelling the Future before its wave starts drops
        the request."""
        validate_request(req)
        fut = cf.Future()
        with self._cv:
            if self._closing:
                raise RuntimeError("server is closed")
            self._pending.append((req, fut, time.perf_counter(), 0))
            self._cv.notify_all()
        return fut

    def close(self, wait=True):
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        if wait:
            self._dispatcher.join()
        self._pool.shutdown(wait=wait)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ dispatch --
    def _take_wave(self):
        """Requests for the next wave and their class (0 small, 1 large); caller
        holds the lock.  The class whose oldest request is older goes first (large
        only while it holds fewer than max_waves - 1 running waves).  Its requests
        are taken in arrival order while they fit the free budget, share the first
        one's medium and lie within cost_spread of its footprint; one that does not
        fit is passed over, unless it is the class's oldest and has waited
        max_wait_s."""
        live = []
        for item in self._pending:
            req, fut, t0, tries = item
            if fut.cancelled():
                self.stats["cancelled"] += 1
                continue
            need = request_footprint(req, self.precision)
            if need > self.budget:
                self.stats["rejected"] += 1
                fut.set_exception(OverBudget(f"request {req.rid} needs {need} B, budget {self.budget} B"))
                continue
            live.append((item, need, 0 if need <= self.small_bytes else 1))
        self._pending = collections.deque(item for item, _, _ in live)
        free = self.budget - self._in_use
        now = time.perf_counter()
        oldest = {}
        for item, need, cls in live:
            oldest.setdefault(cls, item[2])
        for cls in sorted(oldest, key=oldest.get):
            if cls == 1 and self.max_waves >= 2 and self._large_running >= self.max_waves - 1:
                continue
            wave, used, taken, anchor = [], 0, set(), None
            first = True
            for item, need, c in live:
                if c != cls:
                    continue
                req, fut, t0, tries = item
                head, first = first, False
                if wave and req.medium_index != wave[0][0].medium_index:
                    continue
                if anchor is not None and not (anchor / self.cost_spread <= need <= anchor * self.cost_spread):
                    continue
                if used + need > free:
                    if head and now - t0 > self.max_wait_s:
                        break   # the class's oldest has waited long enough: nothing passes it
                    continue
                if not fut.running() and not fut.set_running_or_notify_cancel():   # cancelled meanwhile
                    self.stats["cancelled"] += 1
                    taken.add(id(item))
                    continue
                wave.append((req, fut, t0, need, tries))
                taken.add(id(item))
                used += need
                if anchor is None:
                    anchor = need
                if len(wave) >= self.max_wave_requests:
                    break
            if taken:
                self._pending = collections.deque(it for it in self._pending if id(it) not in taken)
            if wave:
                return wave, used, cls
        return [], 0, None

    def _dispatch(self):
        while True:
            with self._cv:
                while True:
                    if self._closing and not self._pending:
                        return
                    if self._pending and self._free_streams:
                        wave, used, cls = self._take_wave()
                        if wave:
                            break
                    self._cv.wait(timeout=0.05)
                self._in_use += used
                self._waves_running += 1
                self._large_running += cls
                self.stats["peak_bytes"] = max(self.stats["peak_bytes"], self._in_use)
                self.stats["max_concurrent_waves"] = max(self.stats["max_concurrent_waves"], self._waves_running)
                self.stats["admitted"] += len(wave)
                self.stats["waves"] += 1
                sidx = self._free_streams.pop()
                self._slot_class[sidx] = cls
                self._slot_cost[sidx] = used
                wid = self._wave_counter
                self._wave_counter += 1
            self._pool.submit(self._run_wave, wave, used, sidx, wid, cls)

    def _run_wave(self, wave, used, sidx, wid, cls=0):
        t_admit = time.perf_counter()
        requeue = []
        try:
            if self.fault_hook is not None:
                self.fault_hook(wid, [w[0] for w in wave])
            results = self._execute(wave, sidx)
            t_done = time.perf_counter()
            for (req, fut, t0, _, _), res in zip(wave, results):
                res.t_submit, res.t_admit, res.t_done = t0, t_admit, t_done
                res.wave, res.wave_size = wid, len(wave)
                self._record(req, res)
                fut.set_result(res)
        except Exception as exc:
            # the wave failed on the host (allocation, a library error): its requests
            # are admitted again, up to max_retries times each, then fail with exc
            for req, fut, t0, _, tries in wave:
                if fut.done():
                    continue
                if tries < self.max_retries:
                    requeue.append((req, fut, t0, tries + 1))
                else:
                    fut.set_exception(exc)
        finally:
            with self._cv:
                self._in_use -= used
                self._waves_running -= 1
                self._large_running -= cls
                self._free_streams.append(sidx)
                if requeue:
                    self.stats["failed_waves"] += 1
                    self.stats["readmitted"] += len(requeue)
                    self._pending.extendleft(reversed(requeue))   # keep arrival order at the head
                self.stats["completed"] += len(wave) - len(requeue)
                self._cv.notify_all()

    def _execute(self, wave, sidx):
        """Solves one wave on its stream: one ragged ClusterBatch, assembled,
        solved and reduced; returns one ClusterResult per request."""
        streams = self._streams[sidx]
        stream = streams[self._priority_level(self._slot_cost.get(sidx, 1 << 62), len(streams))]
        with torch.cuda.device(self.device), torch.cuda.stream(stream):
            specs = [request_spec(w[0]) for w in wave]
            b = ClusterBatch(specs, R=1, precision=self.precision, device=self.device)
            b.assemble()
            b.solve(tol=self.tol, maxiter=self.maxiter, inner_tol=self.inner_tol, max_refine=8)
            b.epilogue(specs[0]["eps_b"])
            # one pinned readback (a copy into pageable memory would share the driver's
            # staging path with the other waves' copies and wait behind their kernels)
            h = b.to_host()
            nobs = b.totals["obs"]
            xs = h["xs"][: nobs * 6 * b.xs_L].reshape(-1, 3, 2 * b.xs_L)
            F = h["F"][: nobs * 3].reshape(-1, 3)
            T = h["T"][: nobs * 3].reshape(-1, 3)
            x = h["x"]
            status, iters = b.status.copy(), b.iters.copy()
            del b
        out = []
        for s, w in enumerate(wave):
            req = w[0]
            l = _layout(specs, s)
            o, N, L = l["obs_off"], l["N"], l["lmax"]
            C = xs[o: o + N, :, : 2 * L].sum(axis=(0, 2))
            out.append(ClusterResult(rid=req.rid, status=int(status[s]), passes=int(iters[s]), C_sca=float(C[0]),
                                     C_abs=float(C[1]), C_ext=float(C[2]),
                                     p_inc=x[l["vec_off"]: l["vec_off"] + l["D"]].reshape(N, 2, l["rmax"]),
                                     force=F[o: o + N].copy(), torque=T[o: o + N].copy()))
        return out

    def _record(self, req, res):
        if not self.metrics_path:
            return
        N = np.asarray(np.atleast_2d(req.position)).shape[0]
        line = dict(rid=req.rid, N=int(N), lmax=int(req.lmax), status=res.status, passes=res.passes,
                    latency_ms=1e3 * res.latency, wait_ms=1e3 * (res.t_admit - res.t_submit), wave=res.wave,
                    wave_size=res.wave_size, footprint_bytes=int(request_footprint(req, self.precision)))
        with self._metrics_lock, open(self.metrics_path, "a") as f:
            f.write(json.dumps(line) + "\n")


def _layout(specs, s):
    """Offsets of cluster s in a ClusterBatch built from specs with R = 1."""
    obs = vec = 0
    for i, sp in enumerate(specs):
        N = np.asarray(sp["position"]).reshape(-1, 3).shape[0]
        L = int(np.asarray(sp["mie_scat"]).shape[-1])
        rmax = lmax_to_rmax(L)
        if i == s:
            return dict(obs_off=obs, vec_off=vec, N=N, lmax=L, rmax=rmax, D=2 * rmax * N)
        obs += N
        vec += 2 * rmax * N
    raise IndexError(s)


# ------------------------------------------------------------ request stream --
_BEAMS = {}                       # one beam object per waist: its far-field projection is cached
_BEAMS_LOCK = threading.Lock()

def random_request(rng, rid=-1, n_range=(2, 500), lmax_range=(2, 8), wavelength=600e-9, beam_width=1e-6,
                   rmin=50e-9, rmax=100e-9, cell=0.5e-6, max_tries=1_000_000, source_kind=None):
    """One request of the serving workload: N log-uniform in n_range, lmax uniform,
    index U[1.3, 2.5] + i U[0, 0.1], radii U[rmin, rmax], centres in a cube of side
    (N cell^3)^(1/3) by rejection sampling; plane wave or Gaussian beam with equal
    probability (source_kind "plane" or "gaussian" fixes it; the draw is made
    either way, so the rest of the stream is unchanged)."""
    from .beams import gaussian_beam
    N = int(round(np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1])))))
    L = int(rng.integers(lmax_range[0], lmax_range[1] + 1))
    index = rng.uniform(1.3, 2.5) + 1j * rng.uniform(0.0, 0.1)
    side = (N * cell ** 3) ** (1 / 3)
    pos = np.zeros((N, 3))
    rad = np.zeros(N)
    n = tries = 0
    while n < N:
        tries += 1
        if tries > max_tries:
            raise RuntimeError("rejection sampling did not place all spheres")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, side, 3)
        if n == 0 or np.all(np.linalg.norm(pos[:n] - c, axis=1) > r + rad[:n]):
            pos[n], rad[n] = c, r
            n += 1
    pos = pos - side / 2
    gauss = rng.uniform() < 0.5
    if source_kind is not None:
        gauss = source_kind == "gaussian"
    if gauss:
        key = float(beam_width)
        with _BEAMS_LOCK:
            if key not in _BEAMS:
                _BEAMS[key] = gaussian_beam(width=beam_width, polarization=[1, 0])
            source = _BEAMS[key]
    else:
        source = plane_wave.from_string("x")
    return ClusterRequest(position=pos, radius=np.array(rad), index=index, wavelength=wavelength, lmax=L,
                          source=source, rid=rid)
