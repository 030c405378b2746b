"""Device-resident batches of sphere clusters.

A ClusterBatch owns, on one GPU, everything a set of independent cluster solves
needs: positions, Mie coefficients, the packed translation matrices (complex128
and/or complex64), right-hand sides, solutions, workspace and observables.  The
single-cluster solver, the wavelength sweep and the solve server all drive this
one class; every step is a call into the CUDA extension.
"""

from __future__ import annotations

import ctypes
import threading

import numpy as np
import torch

from . import _native as nat
from .modes import lmax_to_rmax

PRECISIONS = {"fp64": nat.PREC_FP64, "mixed": nat.PREC_MIXED, "fp32": nat.PREC_FP32,
              "mixed_fp64res": nat.PREC_MIXED_FP64RES}
NEEDS = {"fp64": ("c128",), "mixed": ("hi", "lo"), "fp32": ("hi",), "mixed_fp64res": ("hi", "c128")}


def current_stream(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(device=None) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("miepy_gb300 needs a CUDA device (GB300); no CPU fallback exists")
    nat.lib()
    return torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())


def matrix_elements(N, lmax):
    B = 2 * lmax_to_rmax(lmax)
    return N * (N - 1) // 2 * B * B


def footprint_bytes(N, lmax, R=1, precision="fp64"):
    """HBM bytes a cluster needs inside a batch (matrices + vectors + solver scratch), for admission."""
    el = matrix_elements(N, lmax)
    D = 2 * lmax_to_rmax(lmax) * N
    mat = sum({"c128": 16, "hi": 8, "lo": 8}[m] for m in NEEDS[precision]) * el
    P = N * (N - 1) // 2
    B = 2 * lmax_to_rmax(lmax)
    partials = 16 * (P * B * R + (P + N) * B * R)
    vec = 16 * D * R * 16
    return mat + partials + vec + 4096


def _spec_lmax(spec, N):
    """lmax of a cluster spec: from its Mie coefficients [N,2,lmax], or from its
    T-matrices [N, B, B] / [N, 2, rmax, 2, rmax] (B = 2 lmax (lmax + 2))."""
    if "mie_scat" in spec:
        return int(np.asarray(spec["mie_scat"]).shape[-1])
    T = np.asarray(spec["tmatrix"])
    n = T.shape[0] if N is None else N
    B = int(round(np.sqrt(T.size // n)))
    return int(round(np.sqrt(1 + B // 2) - 1))


_stage_local = threading.local()


def _staging(nbytes):
    """This thread's pinned staging buffer (grown as needed) and the event behind its
    last host->device copy; waits for that copy before handing the buffer out again."""
    st = getattr(_stage_local, "buf", None)
    if st is not None:
        st[1].synchronize()
    if st is None or st[0].numel() < nbytes:
        cap = max(nbytes, 1 << 20)
        st = (torch.empty(cap, dtype=torch.uint8).pin_memory(), torch.cuda.Event())
        _stage_local.buf = st
    return st


class ClusterBatch:
    """Independent clusters sharing launch sequences.

    specs: list of dicts with
        position [N,3] float, mie_scat [N,2,lmax] complex, k float (medium wavenumber),
        p_src [N,2,rmax,R] complex (or [N,2,rmax] when R == 1),
        optional mie_int [N,2,lmax], eps_b float.
    packed=False allocates no packed pair-block matrix: for a batch whose operator is
    formed and solved densely (lmax > 8, an interface, a periodic symmetry), which
    uses the batch only for its inputs, vectors and epilogue.
    """

    def __init__(self, specs, R=1, precision="fp64", device=None, tensor=False, packed=True):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {list(PRECISIONS)}")
        if tensor and (int(R) not in (4, 8) or precision not in ("fp32", "mixed")):
            raise ValueError("tensor=True serves R = 4 or 8 right-hand sides with precision 'fp32' or 'mixed'")
        self.device = require_cuda(device)
        self.R = int(R)
        self.precision = precision
        self._set_layout(specs)
        dev = self.device
        t = self.totals
        # inputs: one device allocation, filled by one host->device copy (see _upload)
        self._parts = [("pos", np.float64, t["pos"]), ("mie_scat", np.complex128, t["mie"]),
                       ("mie_int", np.complex128, t["mie"]), ("b", np.complex128, t["vec"])]
        self._offs, nbytes = {}, 0
        for name, dt, n in self._parts:
            self._offs[name] = nbytes
            nbytes += (np.dtype(dt).itemsize * max(n, 1) + 255) & ~255
        self._inputs = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        tdt = {np.float64: torch.float64, np.complex128: torch.complex128}
        self.pos, self.mie_scat, self.mie_int, self.b = (
            self._inputs[self._offs[name]: self._offs[name] + np.dtype(dt).itemsize * max(n, 1)].view(tdt[dt])
            for name, dt, n in self._parts)
        self.h2d_bytes = 8 * t["pos"] + 16 * (2 * t["mie"] + t["vec"])
        self.tvec = torch.empty(max(t["t"], 1), dtype=torch.complex128, device=dev)
        # outputs in one float64 buffer: x, then per-particle xs, force and torque, so
        # that to_host() reads them back with one copy
        self.xs_L = max(l["lmax"] for l in self.layout)
        nv2 = 2 * max(t["vec"], 1)
        self._n_xs = max(t["obs"] * self.R * 6 * self.xs_L, 1)
        self._n_f = max(t["obs"] * self.R * 3, 1)
        self._out = torch.zeros(nv2 + self._n_xs + 2 * self._n_f, dtype=torch.float64, device=dev)
        self.x = self._out[:nv2].view(torch.complex128)
        self._xs_buf = self._out[nv2: nv2 + self._n_xs]
        self._f_buf = self._out[nv2 + self._n_xs: nv2 + self._n_xs + self._n_f]
        self._t_buf = self._out[nv2 + self._n_xs + self._n_f:]
        self.xs = self.F = self.T = None
        self.packed = bool(packed)
        need = NEEDS[precision] if packed else ()
        mat = max(t["mat"], 1)
        self.mat128 = torch.empty(mat, dtype=torch.complex128, device=dev) if "c128" in need else None
        self.mat64 = torch.empty(mat, dtype=torch.complex64, device=dev) if "hi" in need else None
        self.mat64lo = torch.empty(mat, dtype=torch.complex64, device=dev) if "lo" in need else None
        # bf16 hi/lo tiles of the complex64 matrix for the tensor-core pass of the FP32
        # solves (R = 4 or 8), rebuilt by every assemble
        self.mat_tc = None
        if tensor:
            nb = nat.lib().gb_tc_matrix_bytes(self.nsys, self.sys)
            self.mat_tc = torch.empty(max(int(nb), 16), dtype=torch.uint8, device=dev)
        self._ws = None
        self._host_out = None
        # general particles: per-particle T-matrices [N][B][B] instead of Mie coefficients
        has_t = ["tmatrix" in sp for sp in specs]
        if any(has_t) and not all(has_t):
            raise ValueError("a batch holds either sphere clusters (mie_scat) or T-matrix clusters (tmatrix)")
        self.tmatrix = all(has_t)
        self.tmat128 = self.tmat64 = None
        if self.tmatrix:
            sizes = [l["N"] * (2 * l["rmax"]) ** 2 for l in self.layout]
            self.tm_off = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64)
            n = int(sum(sizes))
            if precision != "fp32":
                self.tmat128 = torch.empty(n, dtype=torch.complex128, device=dev)
            if precision != "fp64":
                self.tmat64 = torch.empty(n, dtype=torch.complex64, device=dev)
        self._upload(specs)

    def _set_layout(self, specs):
        self.specs = specs
        self.nsys = len(specs)
        descs, mie_off, obs_off = [], [], []
        pos_off = mat_off = vec_off = t_off = m_off = o_off = 0
        self.layout = []
        for s in specs:
            pos = np.asarray(s["position"], float).reshape(-1, 3)
            N = pos.shape[0]
            lmax = _spec_lmax(s, N)
            rmax = lmax_to_rmax(lmax)
            D = 2 * rmax * N
            el = matrix_elements(N, lmax)
            descs.append((N, lmax, float(np.real(s["k"])), pos_off, mat_off, vec_off, t_off))
            mie_off.append(m_off)
            obs_off.append(o_off)
            self.layout.append(dict(N=N, lmax=lmax, rmax=rmax, D=D, pos_off=pos_off, mat_off=mat_off, vec_off=vec_off,
                                    t_off=t_off, mie_off=m_off, obs_off=o_off))
            pos_off += 3 * N
            mat_off += el
            vec_off += D * self.R
            t_off += D
            m_off += N * 2 * lmax
            o_off += N
        self.totals = dict(pos=pos_off, mat=mat_off, vec=vec_off, t=t_off, mie=m_off, obs=o_off)
        self.sys = nat.systems_array(descs)
        self.mie_off = np.asarray(mie_off, dtype=np.int64)
        self.obs_off = np.asarray(obs_off, dtype=np.int64)

    def _upload(self, specs):
        """Host inputs of specs -> the device input buffer, through this thread's
        pinned staging buffer, as one asynchronous copy on the current stream."""
        stage, done = _staging(self._inputs.numel())
        hv = stage.numpy()
        n_mie = lambda sp: 2 * np.asarray(sp["position"]).reshape(-1, 3).shape[0] * _spec_lmax(sp, None)
        for name, dt, n in self._parts:
            dst = hv[self._offs[name]: self._offs[name] + np.dtype(dt).itemsize * n].view(dt)
            o = 0
            for sp in specs:
                if name == "pos":
                    a = np.asarray(sp["position"], float).reshape(-1)
                elif name == "mie_scat":
                    a = np.asarray(sp["mie_scat"]).reshape(-1) if "mie_scat" in sp else np.zeros(n_mie(sp), complex)
                elif name == "mie_int":
                    a = np.asarray(sp["mie_int"]).reshape(-1) if "mie_int" in sp else np.zeros(n_mie(sp), complex)
                else:
                    a = np.asarray(sp["p_src"]).reshape(-1)
                dst[o: o + a.size] = a
                o += a.size
        self._inputs.copy_(stage[: self._inputs.numel()], non_blocking=True)
        done.record(torch.cuda.current_stream(self.device))
        if self.tmatrix:   # per-particle T-matrices (a separate, larger upload)
            host = np.concatenate([np.asarray(sp["tmatrix"], complex).reshape(-1) for sp in specs])
            if self.tmat128 is not None:
                self.tmat128.copy_(torch.from_numpy(np.ascontiguousarray(host)))
            if self.tmat64 is not None:
                self.tmat64.copy_(torch.from_numpy(np.ascontiguousarray(host.astype(np.complex64))))
        self.status = self.iters = self.resid = None
        self.assembled = False

    def load(self, specs):
        """New clusters of the same shapes (per cluster N and lmax, same order) into
        this batch's device buffers: positions, Mie coefficients, wavenumbers and
        right-hand sides (and T-matrices of general particles) are uploaded; the
        matrices are rebuilt by the next assemble."""
        old = [(l["N"], l["lmax"]) for l in self.layout]
        new = [(np.asarray(s["position"]).reshape(-1, 3).shape[0], _spec_lmax(s, None)) for s in specs]
        if old != new:
            raise ValueError("load() needs clusters of the batch's shapes (N, lmax per cluster)")
        if any(("tmatrix" in s) != self.tmatrix for s in specs):
            raise ValueError("load() needs clusters of the batch's kind (Mie coefficients or T-matrices)")
        # same shapes, so the same offsets: only the wavenumbers of the descriptors change
        self.specs = specs
        for i, sp in enumerate(specs):
            self.sys[i].k = float(np.real(sp["k"]))
        self._upload(specs)
        return self

    # ---------------------------------------------------------------- steps --
    def assemble(self):
        if not self.packed:
            raise ValueError("this batch was built with packed=False and holds no packed matrix to assemble")
        L = nat.lib()
        st = current_stream(self.device)
        nat.check(L.gb_expand_mie_batch(self.nsys, self.sys, self.mie_off.ctypes.data, nat.ptr(self.mie_scat),
                                        nat.ptr(self.tvec), st), "expand mie")
        if self.totals["mat"] > 0:
            nat.check(L.gb_assemble_batch(self.nsys, self.sys, nat.ptr(self.pos), nat.ptr(self.mat128),
                                          nat.ptr(self.mat64), nat.ptr(self.mat64lo), st), "assemble")
            if self.mat_tc is not None:
                nat.check(L.gb_tc_matrix_build(self.nsys, self.sys, nat.ptr(self.mat64), nat.ptr(self.mat_tc), st),
                          "tensor-core tiles")
        self.assembled = True
        return self

    def workspace(self, prec_code):
        L = nat.lib()
        need = L.gb_solve_workspace_size(self.nsys, self.sys, self.R, prec_code)
        if need == 0:
            raise nat.GBError(nat.GB_BAD_ARG, "workspace query failed: " + nat.last_error())
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._ws

    def solve(self, tol=1e-5, maxiter=1000, inner_tol=1e-4, max_refine=8, precision=None, raise_on_fail=False,
              precondition=False):
        """Solve every cluster and right-hand side.  precondition=True runs the
        BiCGSTAB iterations right-preconditioned by diag(1 / (1 + a_n)) of the Mie
        coefficients (the reference's build_block_preconditioner_sphere,
        src/miepy/interactions.py:9-39, inside solve_linear_system_preconditioned,
        cpp/src/interactions.cpp:321-345); a device complex128 tensor gives the
        diagonal itself (rows at the clusters' t offsets).  Sphere clusters only."""
        if not self.assembled:
            self.assemble()
        precision = precision or self.precision
        code = PRECISIONS[precision]
        L = nat.lib()
        ws = self.workspace(code)
        n = self.nsys * self.R
        status = np.zeros(n, dtype=np.int32)
        iters = np.zeros(n, dtype=np.int32)
        resid = np.zeros(n, dtype=np.float64)
        if self.tmatrix:
            if precondition is not False and precondition is not None:
                raise ValueError("precondition serves sphere clusters (the diagonal of the Mie coefficients)")
            rc = L.gb_solve_batch_tmatrix(self.nsys, self.sys, self.R, code, float(tol), int(maxiter), float(inner_tol),
                                          int(max_refine), nat.ptr(self.mat128), nat.ptr(self.mat64),
                                          nat.ptr(self.mat64lo), nat.ptr(self.tmat128), nat.ptr(self.tmat64),
                                          self.tm_off.ctypes.data, nat.ptr(self.b), nat.ptr(self.x), nat.ptr(ws),
                                          ws.numel(), status.ctypes.data, iters.ctypes.data, resid.ctypes.data,
                                          current_stream(self.device))
        else:
            tc = self.mat_tc if precision in ("fp32", "mixed") else None
            if isinstance(precondition, torch.Tensor):
                if precondition.dtype != torch.complex128 or precondition.numel() < self.totals["t"] or \
                        precondition.device != self.x.device:
                    raise ValueError("a given preconditioner is a device complex128 [rows] array at the t offsets")
                pd = precondition
            else:
                pd = self._preconditioner() if precondition else None
            rc = L.gb_solve_batch_ex(self.nsys, self.sys, self.R, code, float(tol), int(maxiter), float(inner_tol),
                                     int(max_refine), nat.ptr(self.mat128), nat.ptr(self.mat64),
                                     nat.ptr(self.mat64lo), nat.ptr(tc), nat.ptr(pd), nat.ptr(self.tvec),
                                     nat.ptr(self.b), nat.ptr(self.x), nat.ptr(ws), ws.numel(), status.ctypes.data,
                                     iters.ctypes.data, resid.ctypes.data, current_stream(self.device))
        if rc not in (nat.GB_OK, nat.GB_NOT_CONVERGED, nat.GB_BREAKDOWN, nat.GB_NAN) or (raise_on_fail and rc):
            nat.check(rc, "solve")
        self.status, self.iters, self.resid = status, iters, resid
        return status

    def _preconditioner(self):
        """diag(1 / (1 + a_n)) per row at the clusters' t_off, from tvec (current
        after every assemble)."""
        if getattr(self, "pdiag", None) is None:
            self.pdiag = torch.empty_like(self.tvec)
        nat.check(nat.lib().gb_sphere_preconditioner(int(self.totals["t"]), nat.ptr(self.tvec), nat.ptr(self.pdiag),
                                                      current_stream(self.device)), "sphere preconditioner")
        return self.pdiag

    def apply(self, x, precision="fp64"):
        """y = (I + T) x on the packed matrices (x: device complex128 [total_vec]);
        precision "fp64" (complex128 matrix), "fp32" (complex64) or "mixed"
        (double-float hi + lo)."""
        L = nat.lib()
        code = PRECISIONS[precision]
        need = L.gb_apply_workspace_size(self.nsys, self.sys, self.R, code)
        ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        y = torch.empty_like(x)
        nat.check(L.gb_apply_batch(self.nsys, self.sys, self.R, code, nat.ptr(self.mat128), nat.ptr(self.mat64),
                                   nat.ptr(self.mat64lo), nat.ptr(self.tvec), nat.ptr(x), nat.ptr(y), nat.ptr(ws),
                                   ws.numel(), current_stream(self.device)), "apply")
        return y

    def apply_tc(self, x, reps=1, gemv_only=False):
        """y = (I + T) x with the tensor-core pass (x: device complex128 [total_vec],
        rounded to complex64; needs tensor=True); reps > 1 launches it back to back."""
        if self.mat_tc is None:
            raise ValueError("this batch was made without tensor=True")
        L = nat.lib()
        need = L.gb_apply_workspace_size(self.nsys, self.sys, self.R, nat.PREC_FP32)
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        y = torch.empty_like(x)
        nat.check(L.gb_apply_repeat_tc(self.nsys, self.sys, self.R, nat.ptr(self.mat_tc), nat.ptr(self.tvec),
                                       nat.ptr(x), nat.ptr(y), nat.ptr(self._ws), self._ws.numel(), int(reps),
                                       int(bool(gemv_only)), current_stream(self.device)), "apply (tensor cores)")
        return y

    def apply_repeat(self, x, precision="fp32", reps=10, gemv_only=False):
        """Launch the operator product reps times back to back (kernel timing)."""
        L = nat.lib()
        code = PRECISIONS[precision]
        need = L.gb_apply_workspace_size(self.nsys, self.sys, self.R, code)
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        y = torch.empty_like(x)
        nat.check(L.gb_apply_repeat(self.nsys, self.sys, self.R, code, nat.ptr(self.mat128), nat.ptr(self.mat64),
                                    nat.ptr(self.mat64lo), nat.ptr(self.tvec), nat.ptr(x), nat.ptr(y),
                                    nat.ptr(self._ws), self._ws.numel(), int(reps), int(bool(gemv_only)),
                                    current_stream(self.device)), "apply_repeat")
        return y

    def autotune(self, precision=None, reps=5):
        """Measure the GEMV lane shapes of this batch's block sizes (gb_autotune_gemv)
        for the matrix pass of precision (default: the batch's; "fp64" tunes the
        complex128 pass, the others the complex64 one).  Returns {B: (lanes per row,
        columns per lane)}.  Solves captured before keep their shapes."""
        L = nat.lib()
        prec = self.precision if precision is None else precision
        code = PRECISIONS["fp64" if prec == "fp64" else "fp32"]
        if code == PRECISIONS["fp64"] and self.mat128 is None or code != PRECISIONS["fp64"] and self.mat64 is None:
            raise ValueError(f"this batch holds no matrix for {prec}")
        need = L.gb_apply_workspace_size(self.nsys, self.sys, self.R, code)
        ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        x = torch.zeros(max(self.totals["vec"], 1), dtype=torch.complex128, device=self.device)
        y = torch.empty_like(x)
        if self.totals["mat"] == 0:
            return {}
        if not self.assembled:
            self.assemble()
        nat.check(L.gb_autotune_gemv(self.nsys, self.sys, self.R, code, nat.ptr(self.mat128), nat.ptr(self.mat64),
                                     nat.ptr(self.tvec), nat.ptr(x), nat.ptr(y), nat.ptr(ws), ws.numel(), int(reps),
                                     current_stream(self.device)), "autotune")
        return self.gemv_shapes(prec)

    def gemv_shapes(self, precision=None):
        """{B: (lanes per row, columns per lane)}: the GEMV lane shapes the matrix pass of
        precision launches with for this batch's block sizes (measured ones after
        autotune, the model's otherwise)."""
        L = nat.lib()
        prec = self.precision if precision is None else precision
        code = PRECISIONS["fp64" if prec == "fp64" else "fp32"]
        out = {}
        for B in sorted({2 * l["rmax"] for l in self.layout if l["N"] > 1}):
            lpr, cpl = ctypes.c_int(0), ctypes.c_int(0)
            nat.check(L.gb_gemv_shape(B, code, self.R, ctypes.byref(lpr), ctypes.byref(cpl)), "gemv shape")
            out[B] = (lpr.value, cpl.value)
        return out

    def epilogue(self, eps_b, source=True, want_fields=True):
        """p_scat, p_int (device, [total_vec]) and per particle xs [N,R,3,2*Lx]
        (Lx: the batch's largest lmax; a cluster of smaller lmax fills the first
        2*lmax entries, the rest stay zero), force/torque [N,R,3]."""
        L = nat.lib()
        dev = self.device
        n_obs = self.totals["obs"]
        ragged = any(l["lmax"] != self.xs_L for l in self.layout)
        # the batch's own output buffers, rewritten by every epilogue
        if want_fields:
            if getattr(self, "_p_scat_buf", None) is None:
                self._p_scat_buf, self._p_int_buf = torch.empty_like(self.x), torch.empty_like(self.x)
            self.p_scat, self.p_int = self._p_scat_buf, self._p_int_buf
        else:
            self.p_scat = self.p_int = None
        xs, F, T = self._xs_buf, self._f_buf, self._t_buf
        if ragged:   # rows of clusters with a smaller lmax keep zeros past 2 lmax
            xs.zero_()
        if self.tmatrix:   # p_scat = T p_inc; no interior coefficients for general particles
            if self.p_scat is None:
                self.p_scat = torch.empty_like(self.x)
            self.p_int = None
            if self.tmat128 is None:
                self.tmat128 = self.tmat64.to(torch.complex128)
            nat.check(L.gb_tmatrix_epilogue_batch(self.nsys, self.sys, self.R, nat.ptr(self.tmat128),
                                                  self.tm_off.ctypes.data, self.obs_off.ctypes.data, nat.ptr(self.x),
                                                  nat.ptr(self.b), float(np.real(eps_b)), int(bool(source)),
                                                  nat.ptr(self.p_scat), nat.ptr(xs), nat.ptr(F), nat.ptr(T),
                                                  current_stream(dev)), "epilogue")
        else:
            nat.check(L.gb_epilogue_batch(self.nsys, self.sys, self.R, self.mie_off.ctypes.data,
                                          self.obs_off.ctypes.data, nat.ptr(self.mie_scat), nat.ptr(self.mie_int),
                                          nat.ptr(self.x), nat.ptr(self.b), float(np.real(eps_b)), int(bool(source)),
                                          nat.ptr(self.p_scat), nat.ptr(self.p_int), nat.ptr(xs), nat.ptr(F),
                                          nat.ptr(T), current_stream(dev)), "epilogue")
        self.xs, self.F, self.T = xs, F, T
        return self

    def cross_sections(self, s):
        """Total (C_sca, C_abs, C_ext) of cluster s per right-hand side: [R, 3] (device)."""
        l = self.layout[s]
        xs = self.xs[: self.totals["obs"] * self.R * 6 * self.xs_L].view(-1, self.R, 3, 2 * self.xs_L)
        return xs[l["obs_off"]: l["obs_off"] + l["N"], :, :, : 2 * l["lmax"]].sum(dim=(0, 3))

    def to_host(self):
        """x, per-particle cross-sections, force and torque as numpy arrays, read back
        with asynchronous copies into pinned buffers and a single synchronisation."""
        if self._host_out is None or self._host_out.numel() != self._out.numel():
            self._host_out = torch.empty(self._out.numel(), dtype=torch.float64).pin_memory()
        self._host_out.copy_(self._out, non_blocking=True)
        torch.cuda.current_stream(self.device).synchronize()
        h = self._host_out.numpy()
        nv2 = 2 * self.x.numel()
        n_xs, n_f = self._n_xs, self._n_f
        return {"x": h[:nv2].view(np.complex128).copy(), "xs": h[nv2: nv2 + n_xs].copy(),
                "F": h[nv2 + n_xs: nv2 + n_xs + n_f].copy(), "T": h[nv2 + n_xs + n_f:].copy()}

    # ------------------------------------------------------------- accessors --
    def cluster_view(self, s, t):
        """Slice of a [total_vec] device vector for cluster s as [N, 2, rmax, R]."""
        l = self.layout[s]
        return t[l["vec_off"]: l["vec_off"] + l["D"] * self.R].view(l["N"], 2, l["rmax"], self.R)
