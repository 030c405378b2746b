"""Benchmark: cluster solves per second on the random-cluster workload.

Workload (the metric's configuration): N = 200 non-overlapping spheres, radii
uniform in 50-100 nm, seeded rejection sampling (seed 2) in a 2 um cube,
index 1.5+0.01i, vacuum, lambda = 600 nm, lmax = 4 (D = 9600), two right-hand
sides (x- and y-polarised plane waves along +z).  A step is one complete cluster
solve: assembly of the interaction matrix, BiCGSTAB for both polarisations to a
relative residual of 1e-8, and the epilogue (p_scat, p_int, per-multipole
cross-sections, force and torque of every particle).

  value : mixed-precision solves/s with inputs resident in HBM
  e2e   : the same solve through the public batch API from host buffers, with the
          host->device copy of the inputs and the device->host copy of the results
          inside the timed region
The FP64 (plain complex128) path is timed in the same run (``fp64_solves_per_s``)
and the C_ext error of the mixed path against it is reported.

--impl reference times the CPU path of the reference (its C++ algorithm as
restated by the oracle, OpenMP over all host cores) on the same workload.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NM = 1e-9
TOL = 1e-8
CONC_STREAMS = 2   # concurrent solve streams of the bench's serving-pattern figure
INNER_TOL = 1e-4   # relative residual of each FP32 inner solve of the mixed method
WORKLOAD = "random cluster N=200 lmax=4 R=2 (D=9600), n=1.5+0.01i, vacuum, 600 nm, seed 2"
# DRAM bytes (read + write) of one k_pgemv<Pol32> launch on this workload, from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum); summary and command in
# profiles/k_pgemv_pol32_cluster_n200_lmax4.txt
GEMV_TRAFFIC_BYTES = 375_720_448
GEMV_TRAFFIC_SOURCE = "ncu: dram__bytes_read.sum 367.70 MB + dram__bytes_write.sum 8.02 MB per launch"


# ---------------------------------------------------------------- workload --
def random_cluster(seed=2, N=200, rmin=50 * NM, rmax=100 * NM, box=2000 * NM):
    rng = np.random.default_rng(seed)
    pos, rad = [], []
    tries = 0
    while len(pos) < N:
        tries += 1
        if tries > 10 ** 6:
            raise RuntimeError("rejection sampling failed")
        r = rng.uniform(rmin, rmax)
        c = rng.uniform(0, box, size=3)
        if all(np.linalg.norm(c - p) > r + q for p, q in zip(pos, rad)):
            pos.append(c)
            rad.append(r)
    return np.array(pos), np.array(rad)


def workload_inputs():
    import miepy_gb300 as gb
    pos, rad = random_cluster()
    mat = gb.constant_material(index=1.5 + 0.01j)
    md = gb.material_struct([mat] * len(rad), gb.constant_material(eps=1.0, mu=1.0), wavelength=600 * NM)
    lmax = 4
    mie_scat, mie_int = gb.mie_coefficients(rad, md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, lmax)
    srcs = [gb.plane_wave.from_string("x"), gb.plane_wave.from_string("y")]
    p_src = np.stack([s.structure(pos, md.k_b, lmax) for s in srcs], axis=-1)   # [N, 2, rmax, 2]
    return dict(position=pos, radius=rad, mie_scat=mie_scat, mie_int=mie_int, k=float(np.real(md.k_b)),
                p_src=np.ascontiguousarray(p_src), eps_b=float(np.real(md.eps_b)), lmax=lmax)


# ------------------------------------------------------------------ clocks --
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm_, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm_)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------- GPU arm --
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def nat_lib():
    from miepy_gb300 import _native
    return _native.lib()


def run_gpu(args, rank, world):
    import torch

    import miepy_gb300 as gb
    from miepy_gb300.engine import ClusterBatch

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    W = workload_inputs()
    spec = dict(position=W["position"], mie_scat=W["mie_scat"], mie_int=W["mie_int"], k=W["k"], p_src=W["p_src"])
    N, lmax = W["position"].shape[0], W["lmax"]
    R = 2
    stream = torch.cuda.current_stream()

    def one_solve(batch, precision):
        batch.assemble()
        batch.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8, precision=precision)
        batch.epilogue(W["eps_b"])

    # ---- resident inputs
    batches = {p: ClusterBatch([spec], R=R, precision=p, device=dev) for p in ("mixed", "fp64")}
    # measured GEMV lane shapes (gb_autotune_gemv) before any solve captures its graphs
    gemv_shapes = {p: {str(B): list(v) for B, v in (b.gemv_shapes() if args.no_autotune else b.autotune()).items()}
                   for p, b in batches.items()}
    for p, b in batches.items():
        for _ in range(args.warmup):
            one_solve(b, p)
    torch.cuda.synchronize()

    def timed(precision, steps):
        b = batches[precision]
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        evs[0].record(stream)
        for s in range(steps):
            one_solve(b, precision)
            evs[s + 1].record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        per = np.array([evs[i].elapsed_time(evs[i + 1]) for i in range(steps)])
        return evs[0].elapsed_time(evs[-1]) / 1e3, per

    L = nat_lib()
    # clocks are sampled across all timed regions (mixed, FP64 and end-to-end)
    clocks = ClockSampler(dev.index).start()
    n0 = L.gb_launch_count()
    t_mixed, per_mixed = timed("mixed", args.steps)
    launches = L.gb_launch_count() - n0
    t_fp64, per_fp64 = timed("fp64", max(3, args.steps // 2))

    # accuracy of the mixed path against FP64, C_ext per polarisation
    def cext(b):
        xs = b.xs[: N * R * 6 * lmax].view(N, R, 3, 2, lmax).sum(dim=(0, 3, 4))
        return xs[:, 2].cpu().numpy()

    one_solve(batches["mixed"], "mixed")
    one_solve(batches["fp64"], "fp64")
    ce_m, ce_d = cext(batches["mixed"]), cext(batches["fp64"])
    cext_err = float(np.max(np.abs(ce_m - ce_d) / np.abs(ce_d)))
    iters_fp64 = batches["fp64"].iters.tolist()
    iters_mixed = batches["mixed"].iters.tolist()
    ref_err = dict(mixed=errors_vs_reference(batches["mixed"], N, lmax, R),
                   fp64=errors_vs_reference(batches["fp64"], N, lmax, R))

    # ---- dominant kernel: one packed-operator product (c64, as in the mixed inner solve),
    # and the double-float / FP64 products for reference
    x = torch.randn(batches["mixed"].totals["vec"], dtype=torch.complex128, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def time_apply(b, prec, reps=32, gemv_only=False):
        """Per-launch duration of the operator (or of its matrix pass alone): events
        around calls of k and k + reps back-to-back launches on the stream; the
        difference over reps leaves out each call's fixed cost (host plan build and
        the first full product), so it is the launches' own duration; the median of
        five such differences."""
        def span(n):
            torch.cuda.synchronize()
            e0.record(stream)
            b.apply_repeat(x, prec, reps=n, gemv_only=gemv_only)
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / 1e3
        span(3)
        k = 4
        return float(np.median([(span(k + reps) - span(k)) / reps for _ in range(5)]))

    def time_assemble(b, reps=9):
        """Device time of one assemble (Mie expansion + matrix assembly), median of reps."""
        out_ = []
        for _ in range(reps):
            torch.cuda.synchronize()
            e0.record(stream)
            b.assemble()
            e1.record(stream)
            torch.cuda.synchronize()
            out_.append(e0.elapsed_time(e1) / 1e3)
        return float(np.median(out_))

    def time_assemble_stream(b, reps=8):
        """Device time per assembly in a stream of assemblies (Mie expansion + special
        functions + matrix assembly): events around k and k + reps back-to-back calls,
        the difference over reps (the median of five), so the host's enqueue of one call
        overlaps the device work of the one before, as in the operator timing."""
        def span(n):
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(n):
                b.assemble()
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / 1e3
        span(2)
        return float(np.median([(span(2 + reps) - span(2)) / reps for _ in range(5)]))

    t_asm = {p: time_assemble(b) for p, b in batches.items()}
    t_asm_stream = {p: time_assemble_stream(b) for p, b in batches.items()}
    t_apply64 = time_apply(batches["mixed"], "fp32")
    t_gemv64 = time_apply(batches["mixed"], "fp32", gemv_only=True)
    t_applydf = time_apply(batches["mixed"], "mixed")
    t_apply128 = time_apply(batches["fp64"], "fp64")
    P = N * (N - 1) // 2
    B = 2 * lmax * (lmax + 2)
    mat_bytes_64 = P * B * B * 8
    mat_bytes_128 = P * B * B * 16
    peak, peak_kind = peaks()

    # ---- end to end from host buffers through the public batch API
    host = {k: (np.ascontiguousarray(v) if isinstance(v, np.ndarray) else v) for k, v in spec.items()}

    e2e_batch = []

    def e2e_step():
        # one cluster per step from host buffers: upload (H2D), assemble, solve,
        # epilogue, read back x / cross-sections / force / torque (D2H)
        if not e2e_batch:
            e2e_batch.append(ClusterBatch([host], R=R, precision="mixed", device=dev))
        else:
            e2e_batch[0].load([host])
        bb = e2e_batch[0]
        one_solve(bb, "mixed")
        out = bb.to_host()
        return bb, out

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_steps = max(3, args.steps // 2)
    t0 = time.perf_counter()
    e0.record(stream)
    for _ in range(e2e_steps):
        bb, out = e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = e0.elapsed_time(e1) / 1e3

    # ---- concurrent solves (the serving pattern): CONC_STREAMS host threads, each
    # with its own batch on its own stream, args.steps solves each; one solve's
    # latency-bound phases overlap another's matrix passes.  Device-timed: every
    # stream waits on a start event and the main stream on every stream's end event.
    conc = [batches["mixed"]] + [ClusterBatch([spec], R=R, precision="mixed", device=dev)
                                 for _ in range(CONC_STREAMS - 1)]
    conc_streams = [torch.cuda.Stream(dev) for _ in conc]
    for b, st_ in zip(conc, conc_streams):
        with torch.cuda.stream(st_):
            for _ in range(args.warmup):
                one_solve(b, "mixed")
    torch.cuda.synchronize()
    c_start, c_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ends = [torch.cuda.Event() for _ in conc]
    per_conc = [None] * len(conc)

    def conc_worker(i):
        b, st_ = conc[i], conc_streams[i]
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
        with torch.cuda.stream(st_):
            st_.wait_event(c_start)
            evs[0].record(st_)
            for s_ in range(args.steps):
                one_solve(b, "mixed")
                evs[s_ + 1].record(st_)
            ends[i].record(st_)
        ends[i].synchronize()
        per_conc[i] = [evs[j].elapsed_time(evs[j + 1]) for j in range(args.steps)]

    n_c0 = L.gb_launch_count()
    c_start.record(stream)
    workers = [threading.Thread(target=conc_worker, args=(i,)) for i in range(len(conc))]
    for th in workers:
        th.start()
    for th in workers:
        th.join()
    for ev in ends:
        stream.wait_event(ev)
    c_end.record(stream)
    torch.cuda.synchronize()
    t_conc = c_start.elapsed_time(c_end) / 1e3
    launches_conc = L.gb_launch_count() - n_c0
    per_c = np.concatenate([np.asarray(v) for v in per_conc])
    conc_same = all(torch.equal(b.xs, conc[0].xs) and torch.equal(b.x, conc[0].x) for b in conc[1:])
    clocks_info = clocks.stop()
    h2d = bb.h2d_bytes
    d2h = sum(o.nbytes for o in out.values())

    ts = np.array([t_mixed, t_fp64, t_e2e, t_conc])
    if world > 1:
        tt = torch.tensor(ts, device=dev)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        ts = tt.cpu().numpy()
    t_mixed, t_fp64, t_e2e, t_conc = ts
    res = dict(
        value=world * args.steps / t_mixed,
        ms_per_step=1e3 * t_mixed / args.steps,
        p50_ms=float(np.percentile(per_mixed, 50)), p99_ms=float(np.percentile(per_mixed, 99)),
        fp64_solves_per_s=world * max(3, args.steps // 2) / t_fp64,
        fp64_p50_ms=float(np.percentile(per_fp64, 50)), fp64_p99_ms=float(np.percentile(per_fp64, 99)),
        cext_rel_err_mixed_vs_fp64=cext_err, iterations_fp64=iters_fp64, refinement_passes_mixed=iters_mixed,
        e2e=dict(value=world * e2e_steps / t_e2e, unit="solves/s", h2d_bytes_per_step=int(h2d),
                 d2h_bytes_per_step=int(d2h)),
        gemv_shapes=gemv_shapes,
        concurrent=dict(streams=CONC_STREAMS, solves_per_s=world * CONC_STREAMS * args.steps / t_conc,
                        p50_ms=float(np.percentile(per_c, 50)), p99_ms=float(np.percentile(per_c, 99)),
                        results_identical_across_streams=bool(conc_same), gpu_launches=int(launches_conc),
                        note="mixed solves of the same workload on concurrent streams, inputs resident"),
        roofline=dict(bound="hbm", achieved=mat_bytes_64 / t_gemv64 / 1e9, peak=peak, unit="GB/s",
                      frac=mat_bytes_64 / t_gemv64 / 1e9 / peak, traffic=GEMV_TRAFFIC_BYTES,
                      traffic_source=GEMV_TRAFFIC_SOURCE,
                      kernel="k_pgemv<Pol32> (packed complex64 matrix pass of the inner BiCGSTAB)",
                      algorithmic_bytes_per_launch=int(mat_bytes_64),
                      peak_source=peak_kind + " (MEASURED_PEAKS.json hbm_gbs, copy burst)",
                      ms_per_launch=1e3 * t_gemv64),
        operators=dict(
            c64_fp32=dict(ms=1e3 * t_apply64, matrix_gbs=mat_bytes_64 / t_apply64 / 1e9,
                          gemv_ms=1e3 * t_gemv64),
            double_float_hi_lo=dict(ms=1e3 * t_applydf, matrix_gbs=2 * mat_bytes_64 / t_applydf / 1e9),
            c128_fp64=dict(ms=1e3 * t_apply128, matrix_gbs=mat_bytes_128 / t_apply128 / 1e9)),
        assembly=dict(
            kernel="k_assemble (packed pair blocks; mixed writes complex64 hi + lo, FP64 complex128)",
            mixed_ms=1e3 * t_asm["mixed"], fp64_ms=1e3 * t_asm["fp64"], bytes_written=int(mat_bytes_128),
            write_floor_ms=1e3 * mat_bytes_128 / (peak * 1e9),
            frac_of_floor_mixed=mat_bytes_128 / (peak * 1e9) / t_asm["mixed"],
            frac_of_floor_fp64=mat_bytes_128 / (peak * 1e9) / t_asm["fp64"],
            note="mixed_ms / fp64_ms: one call between events (with the host's launch gaps); *_stream: "
                 "per call in a stream of back-to-back calls",
            mixed_ms_stream=1e3 * t_asm_stream["mixed"], fp64_ms_stream=1e3 * t_asm_stream["fp64"],
            frac_of_floor_mixed_stream=mat_bytes_128 / (peak * 1e9) / t_asm_stream["mixed"],
            frac_of_floor_fp64_stream=mat_bytes_128 / (peak * 1e9) / t_asm_stream["fp64"]),
        gpu_launches_total=int(launches),
        clocks=clocks_info,
        errors_vs_reference=ref_err,
    )
    if not args.no_multi_rhs:
        res["multi_rhs"] = run_multi_rhs(args, W, dev, peak)
    return res


def errors_vs_reference(batch, N, lmax, R):
    """Relative errors of a solved config-2 batch (x and y plane waves) against the
    reference's exact solve of the same cluster (tests/golden/config2_n200_lmax4_exact,
    made by the reference's own sphere_cluster): p_inc, total cross-sections, forces
    and torques."""
    path = os.path.join(ROOT, "tests", "golden", "config2_n200_lmax4_exact.npz")
    if not os.path.exists(path):
        return None
    g = np.load(path)
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    x = batch.cluster_view(0, batch.x).cpu().numpy()
    xs = batch.xs[: N * R * 6 * lmax].view(N, R, 3, 2, lmax).sum(dim=(0, 3, 4)).cpu().numpy()
    F = batch.F[: N * R * 3].view(N, R, 3).cpu().numpy()
    T = batch.T[: N * R * 3].view(N, R, 3).cpu().numpy()
    out = {}
    for q, pol in enumerate(("x", "y")):
        C = g[f"cross_sections_{pol}"]
        out[pol] = dict(p_inc=rel(x[..., q], g[f"p_inc_{pol}"]),
                        C_sca=float(abs(xs[q, 0] - C[0]) / abs(C[0])), C_abs=float(abs(xs[q, 1] - C[1]) / abs(C[1])),
                        C_ext=float(abs(xs[q, 2] - C[2]) / abs(C[2])), force=rel(F[:, q], g[f"force_{pol}"]),
                        torque=rel(T[:, q], g[f"torque_{pol}"]))
    return out


def run_multi_rhs(args, W, dev, peak):
    """Eight sources on the headline cluster (x and y polarisation at four incidence
    directions): R = 8 right-hand sides share every matrix pass.  The FP32 inner
    solves run their products either as one tcgen05 split-BF16x3 pass over the bf16
    tiles (tensor=True) or as four CUDA-core complex64 passes (one per pair of
    right-hand sides).  Reports both passes against the HBM roofline and both mixed
    solves (tolerance 1e-8), with their C_ext error against an FP64 solve."""
    import torch

    import miepy_gb300 as gb
    from miepy_gb300.engine import ClusterBatch
    R = 8
    srcs = []
    for d in range(R // 2):
        th, ph = 0.35 * d, 0.8 * d
        srcs += [gb.plane_wave(polarization=[1, 0], theta=th, phi=ph), gb.plane_wave(polarization=[0, 1], theta=th, phi=ph)]
    pos = W["position"]
    N, lmax = pos.shape[0], W["lmax"]
    p_src = np.stack([s_.structure(pos, W["k"], lmax) for s_ in srcs], axis=-1)
    spec = dict(position=pos, mie_scat=W["mie_scat"], mie_int=W["mie_int"], k=W["k"], p_src=p_src)
    stream = torch.cuda.current_stream()
    bt = ClusterBatch([spec], R=R, precision="mixed", device=dev, tensor=True)
    bc = ClusterBatch([spec], R=R, precision="mixed", device=dev)
    b64 = ClusterBatch([spec], R=R, precision="fp64", device=dev)

    def solve(b, prec="mixed"):
        b.assemble()
        b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8, precision=prec)
        b.epilogue(W["eps_b"])

    for _ in range(max(1, args.warmup)):
        solve(bt)
        solve(bc)
    solve(b64, "fp64")
    torch.cuda.synchronize()
    steps = max(3, args.steps // 2)

    def timed(b):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        torch.cuda.synchronize()
        e[0].record(stream)
        for _ in range(steps):
            solve(b)
        e[1].record(stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]) / 1e3 / steps

    t_tc, t_cc = timed(bt), timed(bc)
    x = torch.randn(bt.totals["vec"], dtype=torch.complex128, device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def span(fn, n):
        torch.cuda.synchronize()
        e0.record(stream)
        fn(n)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3

    def per_pass(fn, reps=24):
        span(fn, 3)
        return float(np.median([(span(fn, 4 + reps) - span(fn, 4)) / reps for _ in range(5)]))

    t_pass_tc = per_pass(lambda n: bt.apply_tc(x, reps=n, gemv_only=True))
    t_pass_cc = per_pass(lambda n: bt.apply_repeat(x, "fp32", reps=n, gemv_only=True))
    cext = lambda b: b.xs[: N * R * 6 * lmax].view(N, R, 3, 2, lmax).sum(dim=(0, 3, 4))[:, 2].cpu().numpy()
    c64 = cext(b64)
    err = lambda b: float(np.max(np.abs(cext(b) - c64) / np.abs(c64)))
    P = N * (N - 1) // 2
    B = 2 * lmax * (lmax + 2)
    tile_bytes = P * 2 * (((B + 7) // 8) * 8) * (((2 * B + 15) // 16) * 16) * 2
    mat64 = P * B * B * 8
    return dict(
        workload=f"{WORKLOAD.split(' R=2')[0]}, R=8 (x/y polarisation at 4 incidence directions)",
        tensor_core=dict(solves_per_s=1.0 / t_tc, source_solves_per_s=R / t_tc, ms_per_step=1e3 * t_tc,
                         cext_rel_err_vs_fp64=err(bt), pass_ms=1e3 * t_pass_tc,
                         roofline=dict(bound="hbm", kernel="k_pgemv_tc<8> (tcgen05 split-BF16x3, one pass for R=8)",
                                       algorithmic_bytes_per_launch=int(tile_bytes),
                                       achieved=tile_bytes / t_pass_tc / 1e9, peak=peak, unit="GB/s",
                                       frac=tile_bytes / t_pass_tc / 1e9 / peak)),
        cuda_core=dict(solves_per_s=1.0 / t_cc, source_solves_per_s=R / t_cc, ms_per_step=1e3 * t_cc,
                       cext_rel_err_vs_fp64=err(bc), pass_ms=1e3 * t_pass_cc,
                       note="k_pgemv<Pol32> once per pair of right-hand sides: 4 matrix passes per product",
                       matrix_gbs_per_product=mat64 / t_pass_cc / 1e9),
        tensor_over_cuda_core=dict(pass_speedup=t_pass_cc / t_pass_tc, solve_speedup=t_cc / t_tc))


# ---------------------------------------------------------- CPU baseline --
def run_cpu_sample(threads=None, gemv_reps=0):
    """One full cluster solve on the host cores with the oracle (OpenMP): assembly,
    BiCGSTAB for both polarisations, cross-sections, forces and torques.  With
    gemv_reps > 0 it also times that many matrix-vector products of the assembled
    matrix alone (the solve's bound: 16 D^2 bytes each)."""
    from oracle import oracle as O
    W = workload_inputs()
    if threads:
        O.set_num_threads(threads)
    n_thr = O.num_threads()
    N, lmax = W["position"].shape[0], W["lmax"]
    t0 = time.perf_counter()
    T = O.sphere_aggregate_tmatrix(W["position"], W["mie_scat"].reshape(N, -1), W["k"])
    t_asm = time.perf_counter() - t0
    xs_all = []
    its = []
    for r in range(2):
        x, it, _ = O.solve_linear_system_profiled(T, W["p_src"][..., r].ravel(), "bicgstab", tol=TOL)
        its.append(it)
        x = x.reshape(N, 2, -1)
        t = W["mie_scat"][:, :, [n - 1 for n in range(1, lmax + 1) for _ in range(2 * n + 1)]]
        ps = x * t
        for i in range(N):
            xs_all.append(O.particle_cross_sections(ps[i], x[i], W["p_src"][i, :, :, r], W["k"]))
        O.force_all(ps, x, W["k"], W["eps_b"])
        O.torque_all(ps, x, W["k"], W["eps_b"])
    total = time.perf_counter() - t0
    out = dict(seconds=total, assembly_s=t_asm, cores=n_thr, iterations=its)
    if gemv_reps:
        D = T.shape[0]
        v = W["p_src"][..., 0].ravel()
        O.gemv(T, v)
        t1 = time.perf_counter()
        for _ in range(gemv_reps):
            O.gemv(T, v)
        dt = (time.perf_counter() - t1) / gemv_reps
        out["gemv_ms"] = 1e3 * dt
        out["gemv_gbs"] = 16.0 * D * D / dt / 1e9
    return out


# ------------------------------------------------------ wavelength sweep --
SWEEP_WORKLOAD = ("wavelength sweep: N=100 Drude spheres (eps_inf 9, wp 9 eV, gamma 0.07 eV; radii 40-80 nm, seed 3, "
                  "2 um cube), 256 wavelengths 400-1000 nm, adaptive lmax 3-7, x-polarised plane wave, vacuum")


def run_sweep(args, rank=0, world=1):
    """One step = the whole 256-wavelength sweep (assembly, mixed solve, epilogue of
    every wavelength) as one ragged batch; value = wavelength solves/s.  On N GPUs
    the wavelengths are split by cost over the ranks (replicas, no collective on the
    data path) and the slowest rank's time counts."""
    import torch
    from miepy_gb300 import replicas as RP
    from miepy_gb300 import sweep as SW
    from miepy_gb300.engine import ClusterBatch
    from miepy_gb300.materials import drude_material
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    pos, rad = SW.drude_cluster(N=100, seed=3)
    wl = np.linspace(400, 1000, 256) * NM
    mine = RP.my_shard([RP.unit_cost(100, L) for L in SW.adaptive_lmax(wl)], rank, world)
    W_total = len(wl)
    specs = SW.sweep_specs(pos, rad, drude_material(9.0, 9.0, 0.07), wl[mine], SW.adaptive_lmax)
    stream = torch.cuda.current_stream()
    L = nat_lib()

    shapes = {}

    def timed(precision, steps, warmup):
        b = ClusterBatch(specs, R=1, precision=precision, device=dev)
        shapes[precision] = {str(B): list(v) for B, v in b.autotune().items()}   # measured GEMV lane shapes
        for _ in range(warmup):
            b.assemble(); b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8); b.epilogue(1.0)
        torch.cuda.synchronize()
        evs = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
        n0 = L.gb_launch_count()
        evs[0].record(stream)
        for k in range(steps):
            b.assemble(); b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8); b.epilogue(1.0)
            evs[k + 1].record(stream)
        torch.cuda.synchronize()
        per = np.array([evs[i].elapsed_time(evs[i + 1]) for i in range(steps)])
        # phase split of one more step (events between the phases)
        ph = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ph[0].record(stream); b.assemble(); ph[1].record(stream)
        b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8); ph[2].record(stream)
        b.epilogue(1.0); ph[3].record(stream)
        torch.cuda.synchronize()
        phases = dict(assemble_ms=ph[0].elapsed_time(ph[1]), solve_ms=ph[1].elapsed_time(ph[2]),
                      epilogue_ms=ph[2].elapsed_time(ph[3]))
        cext = np.array([b.cross_sections(s)[0, 2].item() for s in range(len(specs))])
        out = dict(t=evs[0].elapsed_time(evs[-1]) / 1e3, per=per, launches=L.gb_launch_count() - n0, cext=cext,
                   phases=phases,
                   status=b.status.copy(), iters=b.iters.copy(), mat_bytes=sum(
                       (t.numel() * t.element_size()) for t in (b.mat128, b.mat64, b.mat64lo) if t is not None))
        del b
        torch.cuda.empty_cache()
        return out

    clocks = ClockSampler(dev.index).start()
    m = timed("mixed", args.steps, args.warmup)
    d = timed("fp64", 1, 1)
    clocks_info = clocks.stop()
    W = W_total
    m["t"] = RP.max_over_ranks(m["t"], dev)
    d["t"] = RP.max_over_ranks(d["t"], dev)
    err = RP.max_over_ranks(float(np.max(np.abs(m["cext"] - d["cext"]) / np.abs(d["cext"]))), dev)
    lm = SW.adaptive_lmax(wl)
    return dict(value=W * args.steps / m["t"], ms_per_step=1e3 * m["t"] / args.steps,
                p50_ms=float(np.percentile(m["per"], 50)), p99_ms=float(np.percentile(m["per"], 99)),
                fp64_solves_per_s=W / d["t"], cext_rel_err_mixed_vs_fp64=err,
                all_converged=bool(np.all(m["status"] == 0) and np.all(d["status"] == 0)),
                lmax_histogram={int(l): int(np.sum(lm == l)) for l in np.unique(lm)}, gemv_shapes=shapes,
                resident_matrix_gb=m["mat_bytes"] / 1e9, gpu_launches=int(m["launches"]),
                phases_mixed=m["phases"], phases_fp64=d["phases"], clocks=clocks_info)


# --------------------------------------------------------- serving stream --
SERVE_WAVES = 4           # waves on the GPU at once in the serving stream
SERVE_WORKLOAD = ("serving stream: seeded requests (seed 4), N log-uniform 2-500, lmax uniform 2-8, index "
                  "U[1.3,2.5]+iU[0,0.1], radii 50-100 nm at constant density, 600 nm, vacuum, plane wave or "
                  "Gaussian beam (waist 1 um) 50/50; Poisson arrivals")


def run_serve(args, nreq=None):
    """The serving stream (seed 4): throughput at saturation (all requests queued at
    once) in mixed precision and in FP64 over the same full stream; then Poisson
    arrivals at half the mixed saturation rate, with each request's latency, its
    latency alone on an idle server, and their ratio (the slowdown the mix causes);
    every Poisson result is checked against its alone result."""
    import torch
    from miepy_gb300 import server as SV
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(4)
    nreq = max(8, nreq or args.requests)
    reqs = [SV.random_request(rng, rid=i) for i in range(nreq)]
    L = nat_lib()
    kw = dict(tol=TOL, max_waves=SERVE_WAVES, max_wave_requests=16)

    def saturate(precision, rs):
        with SV.SolveServer(precision=precision, **kw) as srv:
            t0 = time.perf_counter()
            futs = [srv.submit(r) for r in rs]
            out = [f.result() for f in futs]
            t = time.perf_counter() - t0
            stats = dict(srv.stats)
        return t, out, stats

    # warm-up: tables of every lmax, the kernels, and the Gaussian beam's far-field
    # projection at every lmax (one small request per lmax and source kind)
    warm = [SV.random_request(np.random.default_rng(100 + l), rid=-1, n_range=(4, 6), lmax_range=(l, l),
                              source_kind=kind) for l in range(2, 9) for kind in ("plane", "gaussian")]
    for p in ("mixed", "fp64"):
        saturate(p, warm)
    clocks = ClockSampler(dev.index).start()
    n0 = L.gb_launch_count()
    t_sat, res_sat, st_sat = saturate("mixed", reqs)
    launches = L.gb_launch_count() - n0
    t_64, res_64, _ = saturate("fp64", reqs)
    rate = 0.5 * nreq / t_sat
    arr = np.cumsum(np.random.default_rng(44).exponential(1.0 / rate, size=nreq))
    with SV.SolveServer(precision="mixed", **kw) as srv:
        t0 = time.perf_counter()
        futs = []
        for r, ta in zip(reqs, arr):
            dt = t0 + ta - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            futs.append(srv.submit(r))
        res_poi = [f.result() for f in futs]
        t_poi = time.perf_counter() - t0
        st_poi = dict(srv.stats)
    with SV.SolveServer(precision="mixed", **kw) as srv:   # each request alone on an idle server
        res_alone = [srv.submit(r).result() for r in reqs]
    clocks_info = clocks.stop()
    lat = np.array([r.latency for r in res_poi]) * 1e3
    alone = np.array([r.latency for r in res_alone]) * 1e3
    slow = lat / alone
    lat_sat = np.array([r.latency for r in res_sat]) * 1e3
    err = max(abs(a.C_ext - b.C_ext) / abs(b.C_ext) for a, b in zip(res_sat, res_64))
    err_alone = max(abs(a.C_ext - b.C_ext) / abs(b.C_ext) for a, b in zip(res_poi, res_alone))
    sizes = [(len(np.asarray(r.radius)), r.lmax) for r in reqs]
    pct = lambda a, q: float(np.percentile(a, q))
    return dict(value=nreq / t_sat, ms_per_step=1e3 * t_sat / nreq,
                p50_ms=pct(lat, 50), p99_ms=pct(lat, 99),
                poisson=dict(rate_per_s=rate, achieved_solves_per_s=nreq / t_poi, p50_ms=pct(lat, 50),
                             p99_ms=pct(lat, 99), alone_p50_ms=pct(alone, 50), alone_p99_ms=pct(alone, 99),
                             slowdown_p50=pct(slow, 50), slowdown_p99=pct(slow, 99), waves=st_poi["waves"],
                             max_concurrent_waves=st_poi["max_concurrent_waves"],
                             cext_rel_err_vs_alone=float(err_alone)),
                saturation=dict(solves_per_s=nreq / t_sat, p50_ms=pct(lat_sat, 50), p99_ms=pct(lat_sat, 99),
                                waves=st_sat["waves"], max_concurrent_waves=st_sat["max_concurrent_waves"],
                                peak_hbm_gb=st_sat["peak_bytes"] / 1e9),
                fp64_solves_per_s=nreq / t_64, mixed_over_fp64=t_64 / t_sat,
                cext_rel_err_mixed_vs_fp64=float(err),
                all_converged=bool(all(r.status == 0 for r in res_sat + res_poi + res_64 + res_alone)),
                requests=nreq, largest_request=dict(N=int(max(sizes)[0]), lmax=int(max(s[1] for s in sizes))),
                gpu_launches=int(launches), clocks=clocks_info)


# ------------------------------------------------------------ large system --
LARGE_WORKLOAD = ("large system: N=2000 spheres on a jittered hexagonal lattice (pitch 300 nm, jitter +-30 nm, "
                  "seed 5), radius 80 nm, n=2.0, lmax 3 (D=60000), vacuum, 600 nm, x-polarised plane wave; "
                  "E on a 512x512 plane at z=0 over the lattice + 500 nm")


def run_large(args):
    """One step = assembly + mixed solve + epilogue of the 2000-sphere lattice; the
    512 x 512 field map (FP32 exterior sums) is timed separately; the FP64 solve once."""
    import torch
    from miepy_gb300 import large as LG
    from miepy_gb300.engine import ClusterBatch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    pos = LG.hex_lattice()
    spec, md, rad = LG.lattice_spec(pos)
    eps_b = float(np.real(md.eps_b))
    stream = torch.cuda.current_stream()
    L = nat_lib()

    def step(b):
        b.assemble(); b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8); b.epilogue(eps_b)

    clocks = ClockSampler(dev.index).start()
    b = ClusterBatch([spec], R=1, precision="mixed", device=dev)
    for _ in range(args.warmup):
        step(b)
    torch.cuda.synchronize()
    steps = max(1, args.steps)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(steps + 1)]
    n0 = L.gb_launch_count()
    ev[0].record(stream)
    for i in range(steps):
        step(b)
        ev[i + 1].record(stream)
    torch.cuda.synchronize()
    launches = L.gb_launch_count() - n0
    per = np.array([ev[i].elapsed_time(ev[i + 1]) for i in range(steps)])
    t = ev[0].elapsed_time(ev[-1]) / 1e3
    ph = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    ph[0].record(stream); b.assemble(); ph[1].record(stream)
    b.solve(tol=TOL, maxiter=1000, inner_tol=INNER_TOL, max_refine=8); ph[2].record(stream)
    b.epilogue(eps_b); ph[3].record(stream)
    torch.cuda.synchronize()
    phases = dict(assemble_ms=ph[0].elapsed_time(ph[1]), solve_ms=ph[1].elapsed_time(ph[2]),
                  epilogue_ms=ph[2].elapsed_time(ph[3]))
    Cm = b.cross_sections(0)[0].cpu().numpy()
    pts = torch.from_numpy(LG.plane_grid(pos, n=512)).to(dev)
    LG.near_field(b, 0, md, rad, pts[:4096], precision="fp32")
    torch.cuda.synchronize()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    E = LG.near_field(b, 0, md, rad, pts, precision="fp32")
    f1.record(stream)
    torch.cuda.synchronize()
    t_field = f0.elapsed_time(f1) / 1e3
    mat_gb = sum(x.numel() * x.element_size() for x in (b.mat64, b.mat64lo) if x is not None) / 1e9
    del b, E
    torch.cuda.empty_cache()
    b = ClusterBatch([spec], R=1, precision="fp64", device=dev)
    d0, d1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    d0.record(stream)
    step(b)
    d1.record(stream)
    torch.cuda.synchronize()
    t64 = d0.elapsed_time(d1) / 1e3
    Cd = b.cross_sections(0)[0].cpu().numpy()
    clocks_info = clocks.stop()
    Npts, N, rmax = 512 * 512, 2000, 15
    return dict(value=steps / t, ms_per_step=1e3 * t / steps, p50_ms=float(np.percentile(per, 50)),
                p99_ms=float(np.percentile(per, 99)), phases_mixed=phases, fp64_solves_per_s=1.0 / t64,
                cext_rel_err_mixed_vs_fp64=float(abs(Cm[2] - Cd[2]) / abs(Cd[2])),
                resident_matrix_gb=mat_gb,
                field=dict(points=Npts, ms=1e3 * t_field, point_particle_terms_per_s=Npts * N / t_field,
                           tflops_by_40_P_N_rmax=40.0 * Npts * N * rmax / t_field / 1e12,
                           precision="FP32 exterior sums, FP64 interior expansions"),
                gpu_launches=int(launches), clocks=clocks_info)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="cluster", choices=["cluster", "sweep", "serve", "large", "multi_rhs"],
                    help="cluster: the headline N=200 cluster; sweep: the 256-wavelength Drude sweep; "
                         "serve: the request stream through the solve server; multi_rhs: the headline cluster "
                         "with R = 8 right-hand sides, tensor-core and CUDA-core matrix passes")
    ap.add_argument("--requests", type=int, default=48, help="requests in the serving stream")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="leave the serving stream out of the headline run")
    ap.add_argument("--no-multi-rhs", action="store_true", help="leave the R=8 tensor-core leg out of the headline run")
    ap.add_argument("--no-autotune", action="store_true",
                    help="GEMV lane shapes from the model instead of measured ones (for runs under a profiler, "
                         "whose timings would mislead the tuner)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    base = dict(metric="cluster solves/s + p99 latency, mixed vs FP64 GPU, at <=1e-6 rel C_ext err",
                unit="solves/s", n_gpus=world, steps=args.steps, warmup=args.warmup, higher_is_better=True,
                scaling="weak", vs_baseline=None, data="synthetic (seeded random cluster)",
                config=dict(workload=WORKLOAD, solve_tol=TOL, rhs=2, l2="inputs larger than L2 (packed matrix "
                            "367 MB c64 + 733 MB c128)", parallelism=f"replicas x{world}"))

    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as O
        O.build()
        cores = len(os.sched_getaffinity(0))
        for _ in range(args.warmup):
            run_cpu_sample(threads=cores)
        times, info = [], None
        for k in range(args.steps):
            info = run_cpu_sample(threads=cores, gemv_reps=3 if k == 0 else 0)
            if k == 0:
                gemv = dict(ms=info["gemv_ms"], gbs=info["gemv_gbs"])
            times.append(info["seconds"])
        one = run_cpu_sample(threads=1, gemv_reps=1)   # one single-thread solve beside the all-core ones
        O.set_num_threads(cores)
        v = args.steps / sum(times)
        line = dict(base, impl="reference", value=v, ms_per_step=1e3 * sum(times) / args.steps, dtype="c128",
                    cpu_baseline=dict(value=v, unit="solves/s", cores=info["cores"], kind="port",
                                      sample=f"{args.steps} full solves of the workload after {args.warmup} warm-up "
                                             "solves (oracle restatement of the reference's OpenMP C++ path: "
                                             "assembly, BiCGSTAB for both polarisations, cross-sections, forces, "
                                             "torques)",
                                      gemv_ms=gemv["ms"], gemv_gbs=gemv["gbs"],
                                      single_thread=dict(value=1.0 / one["seconds"], unit="solves/s", cores=1,
                                                         gemv_gbs=one["gemv_gbs"])),
                    e2e=dict(value=v, unit="solves/s", h2d_bytes_per_step=0, d2h_bytes_per_step=0),
                    iterations=info["iterations"], p50_ms=1e3 * float(np.percentile(times, 50)),
                    p99_ms=1e3 * float(np.percentile(times, 99)))
        print(json.dumps(line))
        return

    import torch
    if args.config == "large":
        if rank == 0:
            res = run_large(args)
            line = dict(base, metric="large-system solves/s (assembly + mixed solve + epilogue), 512^2 near field",
                        unit="solves/s", impl="gb300", dtype="c64 BiCGSTAB + double-float refinement residual",
                        data="synthetic (seeded jittered lattice)", cpu_baseline=None,
                        config=dict(workload=LARGE_WORKLOAD, solve_tol=TOL, rhs=1), **res)
            print(json.dumps(line))
        return
    if args.config == "multi_rhs":
        if rank == 0:
            dev = torch.device("cuda", 0)
            torch.cuda.set_device(dev)
            res = run_multi_rhs(args, workload_inputs(), dev, peaks()[0])
            line = dict(base, metric="source solves/s (R = 8 right-hand sides per cluster solve)", unit="solves/s",
                        impl="gb300", value=res["tensor_core"]["source_solves_per_s"],
                        dtype="split-bf16x3 tensor-core FP32 inner solves + double-float refinement residual",
                        cpu_baseline=None, config=dict(workload=res["workload"], solve_tol=TOL, rhs=8), **res)
            print(json.dumps(line))
        return
    if args.config == "serve":
        if rank == 0:
            res = run_serve(args)
            line = dict(base, metric="cluster solves/s + p99 latency, mixed vs FP64 GPU, serving stream",
                        unit="solves/s", impl="gb300", dtype="c64 BiCGSTAB + double-float refinement residual",
                        data="synthetic (seeded request stream)", cpu_baseline=None,
                        config=dict(workload=SERVE_WORKLOAD, solve_tol=TOL, rhs=1,
                                    batching=f"continuous (waves admitted by HBM budget and size class, "
                                             f"{SERVE_WAVES} concurrent waves, stream priority by wave cost)"),
                        **res)
            print(json.dumps(line))
        return
    if args.config == "sweep":
        if world > 1:
            torch.distributed.init_process_group("nccl")
        res = run_sweep(args, rank, world)
        if world > 1:
            torch.distributed.destroy_process_group()
        if rank == 0:
            line = dict(base, metric="wavelength solves/s, mixed vs FP64 GPU, at <=1e-6 rel C_ext err",
                        unit="solves/s", impl="gb300", dtype="c64 BiCGSTAB + double-float refinement residual",
                        data="synthetic (seeded Drude cluster)", cpu_baseline=None, scaling="strong",
                        config=dict(workload=SWEEP_WORKLOAD, solve_tol=TOL, rhs=1, batching="one ragged batch",
                                    l2="inputs larger than L2",
                                    parallelism=f"wavelengths split by cost over {world} replica(s)"), **res)
            print(json.dumps(line))
        return
    if world > 1:
        torch.distributed.init_process_group("nccl")
    res = run_gpu(args, rank, world)
    if rank == 0:
        cpu = None
        if not args.no_cpu_baseline and world == 1:
            info = run_cpu_sample(threads=len(os.sched_getaffinity(0)), gemv_reps=3)
            cpu = dict(value=1.0 / info["seconds"], unit="solves/s", cores=info["cores"], kind="port",
                       sample="1 full solve of the workload (assembly + 2 BiCGSTAB solves + epilogue) on the oracle",
                       assembly_s=info["assembly_s"], iterations=info["iterations"], gemv_gbs=info["gemv_gbs"])
        serving = None
        if world == 1 and not args.no_serving:
            sv = run_serve(args)
            serving = dict(workload=SERVE_WORKLOAD, requests=sv["requests"],
                           mixed_solves_per_s=sv["saturation"]["solves_per_s"],
                           fp64_solves_per_s=sv["fp64_solves_per_s"], mixed_over_fp64=sv["mixed_over_fp64"],
                           cext_rel_err_mixed_vs_fp64=sv["cext_rel_err_mixed_vs_fp64"], poisson=sv["poisson"],
                           all_converged=sv["all_converged"], largest_request=sv["largest_request"])
        line = dict(base, impl="gb300", dtype="c64 BiCGSTAB + double-float (c64 hi+lo) refinement residual, "
                                             "c64 incremental residual once |r| <= 2.5e4 tol |b|",
                    gpu_launches=res.pop("gpu_launches_total"), cpu_baseline=cpu, serving=serving, **res)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
