"""Large single system: N = 2000 spheres on a jittered hexagonal lattice (pitch
300 nm, radius 80 nm, n = 2.0, seed 5), lmax 3 (D = 60,000), vacuum, 600 nm.

CPU: the lattice (site count, spacing, jitter bound, non-overlap) and the plane grid.
GPU: the mixed-precision solve against the FP64 solve of the same system (C_ext,
C_sca within 1e-6 relative, C_abs of the lossless spheres below 1e-9 C_ext; forces
within 1e-5 of the largest), and the FP32
near-field map against the FP64 field kernel on a sample of its points (within 1e-4
of the largest field magnitude); a small case checks the FP32 kernel against FP64
at every point, interior points included.
"""

import numpy as np
import pytest

from miepy_gb300 import large as LG

nm = 1e-9


def test_hex_lattice():
    pos = LG.hex_lattice()
    assert pos.shape == (2000, 3) and np.all(pos[:, 2] == 0)
    d = np.linalg.norm(pos[:, None, :2] - pos[None, :, :2], axis=-1)
    np.fill_diagonal(d, np.inf)
    nn = d.min(axis=1)
    assert nn.min() > 2 * 80 * nm                         # no overlap
    assert nn.min() > 300 * nm - 2 * np.sqrt(2) * 30 * nm - 1e-12
    assert abs(np.median(nn) - 300 * nm) < 40 * nm
    pts = LG.plane_grid(pos, n=64)
    assert pts.shape == (4096, 3)
    assert pts[:, 0].min() < pos[:, 0].min() - 499 * nm and pts[:, 1].max() > pos[:, 1].max() + 499 * nm


@pytest.mark.gpu
def test_fp32_field_kernel_against_fp64_small():
    import torch
    from miepy_gb300.engine import ClusterBatch
    pos = LG.hex_lattice(N=12, cells=4)
    spec, md, rad = LG.lattice_spec(pos, lmax=4)
    b = ClusterBatch([spec], R=1, precision="fp64")
    b.assemble()
    b.solve(tol=1e-12)
    b.epilogue(float(np.real(md.eps_b)))
    pts = LG.plane_grid(pos, n=40, margin=200 * nm)
    E64 = LG.near_field(b, 0, md, rad, pts, precision="fp64").cpu().numpy()
    E32 = LG.near_field(b, 0, md, rad, pts, precision="fp32").cpu().numpy()
    scale = np.max(np.abs(E64))
    assert np.max(np.abs(E32 - E64)) <= 2e-5 * scale
    H64 = LG.near_field(b, 0, md, rad, pts, precision="fp64", magnetic=True).cpu().numpy()
    H32 = LG.near_field(b, 0, md, rad, pts, precision="fp32", magnetic=True).cpu().numpy()
    assert np.max(np.abs(H32 - H64)) <= 2e-5 * np.max(np.abs(H64))


@pytest.mark.gpu
def test_large_lattice_mixed_vs_fp64_and_field_map():
    import torch
    from miepy_gb300.engine import ClusterBatch
    pos = LG.hex_lattice()
    spec, md, rad = LG.lattice_spec(pos)
    eps_b = float(np.real(md.eps_b))
    res = {}
    for prec in ("mixed", "fp64"):
        b = ClusterBatch([spec], R=1, precision=prec)
        b.assemble()
        b.solve(tol=1e-8, maxiter=1000, inner_tol=1e-5, max_refine=8)
        assert b.status[0] == 0, (prec, b.status, b.resid)
        b.epilogue(eps_b)
        C = b.cross_sections(0)[0].cpu().numpy()
        res[prec] = (C, b.F[: 2000 * 3].view(2000, 3).cpu().numpy())
        if prec == "mixed":
            pts = LG.plane_grid(pos, n=512)
            E32 = LG.near_field(b, 0, md, rad, pts, precision="fp32").cpu().numpy()
            assert E32.shape == (512 * 512, 3) and np.all(np.isfinite(E32))
            sample = np.random.default_rng(0).choice(512 * 512, 1024, replace=False)
            E64 = LG.near_field(b, 0, md, rad, pts[sample], precision="fp64").cpu().numpy()
            assert np.max(np.abs(E32[sample] - E64)) <= 1e-4 * np.max(np.abs(E64))
        del b
        torch.cuda.empty_cache()
    (Cm, Fm), (Cd, Fd) = res["mixed"], res["fp64"]
    # index 2.0 is lossless: C_abs is rounding noise around zero, held to 1e-9 C_ext
    np.testing.assert_allclose(Cm[[0, 2]], Cd[[0, 2]], rtol=1e-6)
    assert abs(Cm[1]) <= 1e-9 * Cd[2] and abs(Cd[1]) <= 1e-9 * Cd[2]
    assert np.max(np.abs(Fm - Fd)) <= 1e-5 * np.max(np.abs(Fd))
