"""Block-diagonal right preconditioners of the BiCGSTAB solves.

The reference builds M_inv_blocks in src/miepy/interactions.py:9-68 and runs
Eigen's BiCGSTAB with it (solve_linear_system_preconditioned,
cpp/src/interactions.cpp:321-345) or its own profiled variant
(bicgstab_preconditioned_profiled, :230-290).

Pins (CPU): the oracle's two preconditioned iterations against the reference's own
results file for its solver benchmark (15 silver chains, precond_ag_chains fixture):
iteration counts exact, residuals to 1e-5 relative, the Frobenius norm of I + T to
1e-9, the difference of the two solutions to 1e-3 relative; the oracle's builders
against the reference builder's diagonal (bit-exact) and inv(I + T_i).

Bars (GPU): the device diagonal 1 / (1 + a_n) to 1e-15 relative; the packed solve
with the diagonal, in FP64 at the reference's tolerance 1e-5, takes the oracle's
Eigen iteration count and lands within 1e-10 of the oracle's iterate; at tolerance
1e-12 (FP64, mixed) within 1e-10 of the LU solution, FP32 at 1e-5 within 1e-4; the
dense path with the sphere and the per-particle inv(I + T_i) preconditioners
within 1e-10 of the oracle's preconditioned iterate.
"""

import numpy as np
import pytest

from oracle import oracle as O
from tests import _golden as G


def rel(a, b):
    return float(np.max(np.abs(np.asarray(a) - np.asarray(b))) / max(np.max(np.abs(np.asarray(b))), 1e-300))


def chains():
    f = G.load("precond_ag_chains")
    out = []
    for q in range(int(f["count"])):
        out.append(dict(N=int(f[f"N_{q}"]), lmax=int(f[f"lmax_{q}"]), position=f[f"position_{q}"],
                        mie_scat=f[f"mie_scat_{q}"], k=float(f[f"k_b_{q}"]), p_src=f[f"p_src_{q}"],
                        pdiag=f[f"pdiag_{q}"], expected=dict(zip([str(k) for k in f["expected_keys"]],
                                                                 f[f"expected_{q}"]))))
    return out


CHAINS = chains()


def interaction_matrix(c):
    T = O.sphere_aggregate_tmatrix(c["position"], c["mie_scat"].reshape(c["N"], -1), c["k"])
    D = int(round(np.sqrt(T.size)))
    return T.reshape(D, D)


# ------------------------------------------------------------------- CPU --
@pytest.mark.parametrize("q", range(len(CHAINS)))
def test_oracle_reproduces_reference_solver_results(q):
    c = CHAINS[q]
    e = c["expected"]
    T = interaction_matrix(c)
    A = T + np.eye(T.shape[0])
    b = c["p_src"].reshape(-1)
    x, it, res = O.bicgstab(A, b)
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    xp, itp, resp = O.bicgstab_preconditioned(A, b, M, bs)
    assert it == int(e["iterations"]) and itp == int(e["iterations_preconditioned"])
    assert abs(res - e["residual"]) <= 1e-5 * e["residual"]
    assert abs(resp - e["residual_preconditioned"]) <= 1e-5 * e["residual_preconditioned"]
    assert abs(np.linalg.norm(A) - e["frobenius_norm"]) <= 1e-9 * e["frobenius_norm"]
    diff = np.linalg.norm(x - xp) / np.linalg.norm(x)
    assert abs(diff - e["solution_relative_diff"]) <= 1e-3 * e["solution_relative_diff"]


@pytest.mark.parametrize("q", [0, 8, 14])
def test_oracle_sphere_builder_is_the_reference_diagonal(q):
    c = CHAINS[q]
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    rows = np.arange(M.shape[0])
    assert np.array_equal(M[rows, rows % bs], c["pdiag"])
    off = M.copy()
    off[rows, rows % bs] = 0
    assert not np.any(off)


def test_oracle_sphere_builder_clamps_near_singular():
    mie = np.zeros((2, 2, 2), complex)
    mie[0, 1, 0] = -1.0 + 1e-13j      # |1 + a| < 1e-12 -> 1
    mie[1, 0, 1] = 0.5 - 0.5j
    M, bs = O.build_block_preconditioner_sphere(mie, 2)
    rmax = 8
    assert M[0 * bs + rmax + 0, rmax + 0] == 1.0
    assert np.isclose(M[1 * bs + 0 + 3, 3], 1 / (1.5 - 0.5j))


def test_oracle_particle_builder_inverts_blocks():
    f = G.load("tmatrix3_lmax3_exact")
    tm = f["tmatrix"]
    M, bs = O.build_block_preconditioner_particle(tm)
    for i in range(tm.shape[0]):
        blk = np.eye(bs) + tm[i].reshape(bs, bs)
        assert rel(M[i * bs:(i + 1) * bs] @ blk, np.eye(bs)) < 1e-12


def test_oracle_eigen_preconditioned_converges_to_lu():
    c = CHAINS[8]
    T = interaction_matrix(c)
    b = c["p_src"].reshape(-1)
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    x_lu = O.solve_linear_system(T, b, method="exact")
    x, it, res = O.solve_linear_system_precond(T, b, M, bs, tol=1e-12)
    assert res <= 1e-12 and it > 0
    assert rel(x, x_lu) < 1e-10


def test_block_diagonal_detection():
    from miepy_gb300.backend import _block_diagonal
    c = CHAINS[0]
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    D = M.shape[0]
    assert np.array_equal(_block_diagonal(M, bs, D), c["pdiag"])
    M[1, 0] = 1e-3
    assert _block_diagonal(M, bs, D) is None


# ------------------------------------------------------------------- GPU --
def _batch(c, precision="fp64"):
    from miepy_gb300.engine import ClusterBatch
    spec = dict(position=c["position"], mie_scat=c["mie_scat"], k=c["k"], p_src=c["p_src"])
    return ClusterBatch([spec], R=1, precision=precision).assemble()


@pytest.mark.gpu
@pytest.mark.parametrize("q", [0, 8, 14])
def test_device_sphere_diagonal(q):
    c = CHAINS[q]
    b = _batch(c)
    d = b._preconditioner().cpu().numpy()[: c["pdiag"].size]
    assert rel(d, c["pdiag"]) < 1e-15


@pytest.mark.gpu
@pytest.mark.parametrize("q", [0, 4, 8, 12])
def test_packed_preconditioned_matches_oracle_iterate(q):
    c = CHAINS[q]
    T = interaction_matrix(c)
    bvec = c["p_src"].reshape(-1)
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    x_o, it_o, _ = O.solve_linear_system_precond(T, bvec, M, bs, tol=1e-5)
    b = _batch(c)
    b.solve(tol=1e-5, maxiter=1000, precondition=True)
    assert int(b.status[0]) == 0
    assert int(b.iters[0]) == it_o
    x = b.cluster_view(0, b.x)[..., 0].cpu().numpy().reshape(-1)
    assert rel(x, x_o) < 1e-10


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol,bar", [("fp64", 1e-12, 1e-10), ("mixed", 1e-12, 1e-10), ("fp32", 1e-5, 1e-4)])
def test_packed_preconditioned_converges_to_lu(precision, tol, bar):
    c = CHAINS[8]
    T = interaction_matrix(c)
    x_lu = O.solve_linear_system(T, c["p_src"].reshape(-1), method="exact")
    b = _batch(c, precision)
    b.solve(tol=tol, maxiter=1000, precision=precision, precondition=True)
    assert int(b.status[0]) == 0
    x = b.cluster_view(0, b.x)[..., 0].cpu().numpy().reshape(-1)
    assert rel(x, x_lu) < bar


@pytest.mark.gpu
def test_packed_preconditioned_rejects_tmatrix_clusters():
    from miepy_gb300.engine import ClusterBatch
    f = G.load("tmatrix3_lmax3_exact")
    spec = dict(position=f["position"], tmatrix=f["tmatrix"], k=float(f["k_b"]), p_src=f["p_src"])
    b = ClusterBatch([spec], R=1, precision="fp64").assemble()
    with pytest.raises(ValueError):
        b.solve(tol=1e-5, precondition=True)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["sphere", "particle"])
def test_dense_preconditioned_plugin(kind):
    from miepy_gb300 import backend
    if kind == "sphere":
        c = CHAINS[8]
        T = interaction_matrix(c)
        p_src = c["p_src"]
        M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    else:
        f = G.load("tmatrix3_lmax3_exact")
        D = int(round(np.sqrt(f["agg_tmatrix"].size)))
        T = f["agg_tmatrix"].reshape(D, D)
        p_src = f["p_src"]
        M, bs = O.build_block_preconditioner_particle(f["tmatrix"])
    x_o, it_o, _ = O.solve_linear_system_precond(T, p_src.reshape(-1), M, bs, tol=1e-5)
    x = backend.solve_linear_system_jax(T, p_src, "bicgstab", M_inv_blocks=M, block_size=bs)
    assert x.shape == p_src.shape
    assert rel(x.reshape(-1), x_o) < 1e-10


@pytest.mark.gpu
def test_device_aggregate_with_sphere_preconditioner():
    """The plugin's packed aggregate with the reference builder's M: the diagonal is
    folded into the packed solve and reaches the oracle's preconditioned iterate."""
    from miepy_gb300 import backend
    c = CHAINS[12]
    agg = backend.sphere_aggregate_tmatrix_jax(c["position"], c["mie_scat"], c["k"])
    M, bs = O.build_block_preconditioner_sphere(c["mie_scat"], c["lmax"])
    x = backend.solve_linear_system_jax(agg, c["p_src"], "bicgstab", M_inv_blocks=M, block_size=bs)
    x_o, _, _ = O.solve_linear_system_precond(interaction_matrix(c), c["p_src"].reshape(-1), M, bs, tol=1e-5)
    assert rel(x.reshape(-1), x_o) < 1e-10
