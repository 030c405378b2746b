"""Parity at the benchmark's own sizes, against fixtures made by the reference.

The fixtures (tests/golden/make_golden.py large) hold the reference's own
sphere_cluster run with the exact (LU) solve:

- config2_n200_lmax4_exact: the benchmark's cluster (N = 200, lmax 4, D = 9600,
  seed 2), x- and y-polarised plane waves, solved here as one batch with R = 2,
  exactly as the benchmark does;
- sweep_n100_lmax7_400nm_exact: the wavelength sweep's cluster at 400 nm (N = 100
  Drude spheres, lmax 7, D = 12600);
- serve_n300_lmax6_exact: a serving-size request (N = 300, lmax 6, D = 28800).

Bars: the plain FP64 method (BiCGSTAB to 1e-13) holds p_inc, p_scat and p_int to
rtol 1e-10 (atol 1e-14 of the largest coefficient), the total cross-sections to
rtol 1e-9, and per-multipole cross-sections, forces and torques to 1e-9 of their
largest entry.  The mixed method at the benchmark's settings (tolerance 1e-8,
inner FP32 solves to 1e-4) holds C_ext to 1e-6 of the reference; its error in
every reported quantity is printed (run with -s to see it).
"""

import numpy as np
import pytest

from miepy_gb300.engine import ClusterBatch
from tests import _golden as G

pytestmark = pytest.mark.gpu

CASES = ["config2_n200_lmax4_exact", "sweep_n100_lmax7_400nm_exact", "serve_n300_lmax6_exact"]


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(np.asarray(b))), 1e-300))


def _case(name):
    """Inputs and reference outputs with a trailing right-hand-side axis."""
    g = G.load(name)
    pols = ["x", "y"] if "p_src_x" in g else [None]
    key = (lambda k, p: f"{k}_{p}") if pols[0] else (lambda k, p: k)
    ref = {k: np.stack([g[key(k, p)] for p in pols], axis=-1)
           for k in ("p_src", "p_inc", "p_scat", "p_int", "force", "torque", "cross_sections_per_multipole")}
    ref["cross_sections"] = np.stack([g[key("cross_sections", p)] for p in pols], axis=0)   # [R, 3]
    return g, len(pols), ref


def _solve(g, R, ref, precision, tol, inner_tol=1e-4):
    b = ClusterBatch([dict(position=g["position"], mie_scat=g["mie_scat"], mie_int=g["mie_int"], k=float(g["k_b"]),
                           p_src=ref["p_src"])], R=R, precision=precision).assemble()
    b.solve(tol=tol, maxiter=3000, inner_tol=inner_tol)
    assert np.all(np.asarray(b.status) == 0), (b.status, b.iters, b.resid)
    b.epilogue(1.0)   # vacuum (eps_b = 1) in all three cases
    N, L = g["position"].shape[0], int(g["lmax"])
    out = dict(
        p_inc=b.cluster_view(0, b.x).cpu().numpy(),
        p_scat=b.cluster_view(0, b.p_scat).cpu().numpy(),
        p_int=b.cluster_view(0, b.p_int).cpu().numpy(),
        xs=b.xs[: N * R * 6 * L].view(N, R, 3, 2, L).cpu().numpy(),
        F=b.F[: N * R * 3].view(N, R, 3).cpu().numpy(),
        T=b.T[: N * R * 3].view(N, R, 3).cpu().numpy(),
    )
    return out


def _errors(out, ref, R):
    per = np.moveaxis(ref["cross_sections_per_multipole"], -1, 1)    # [N, R, 3, 2, L]
    tot = out["xs"].sum(axis=(0, 3, 4))                               # [R, 3]
    e = {k: rel(out[k], ref[k]) for k in ("p_inc", "p_scat", "p_int")}
    for c, nm in enumerate(("C_sca", "C_abs", "C_ext")):
        e[nm] = float(np.max(np.abs(tot[:, c] - ref["cross_sections"][:, c]) / np.abs(ref["cross_sections"][:, c])))
    e["xs_per_multipole"] = rel(out["xs"], per)
    e["force"] = rel(out["F"], np.moveaxis(ref["force"], -1, 1))
    e["torque"] = rel(out["T"], np.moveaxis(ref["torque"], -1, 1))
    return e


@pytest.mark.parametrize("name", CASES)
def test_fp64_matches_reference_exact_solve(name):
    g, R, ref = _case(name)
    out = _solve(g, R, ref, "fp64", tol=1e-13)
    for k in ("p_inc", "p_scat", "p_int"):
        np.testing.assert_allclose(out[k], ref[k], rtol=1e-10, atol=1e-14 * np.max(np.abs(ref[k])))
    e = _errors(out, ref, R)
    print(f"\n{name} fp64 errors vs reference: " + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
    for k in ("C_sca", "C_abs", "C_ext", "xs_per_multipole", "force", "torque"):
        assert e[k] < 1e-9, (k, e[k])


@pytest.mark.parametrize("name", CASES)
def test_mixed_matches_reference_within_1e6(name):
    g, R, ref = _case(name)
    out = _solve(g, R, ref, "mixed", tol=1e-8)
    e = _errors(out, ref, R)
    print(f"\n{name} mixed errors vs reference: " + ", ".join(f"{k} {v:.2e}" for k, v in e.items()))
    assert e["C_ext"] < 1e-6
    assert e["C_sca"] < 1e-6 and e["C_abs"] < 1e-5
    assert e["p_inc"] < 1e-6
