"""Wavelength sweeps as ragged batches (Drude spheres, adaptive lmax 3-7).

CPU: the sweep's per-wavelength inputs (Drude permittivity, adaptive lmax, Mie
coefficients, p_src) against direct evaluation of the same formulas.
GPU: every wavelength of a small sweep against the oracle's exact solve of the same
cluster (mixed precision: C_ext within 1e-6; FP64 batch: p_inc within 1e-10), and the
full-size sweep (N=100, 256 wavelengths) against FP64 solves of one wavelength per
lmax (C_ext within 1e-6).
"""

import numpy as np
import pytest

from miepy_gb300 import sweep as SW
from miepy_gb300.materials import drude_material

nm = 1e-9
DRUDE = dict(eps_inf=9.0, omega_p_ev=9.0, gamma_ev=0.07)


def test_adaptive_lmax_rule():
    wl = np.linspace(400, 1000, 256) * nm
    L = SW.adaptive_lmax(wl)
    assert L[0] == 7 and L[-1] == 3
    assert np.all(np.diff(L) <= 0)
    assert set(L.tolist()) == {3, 4, 5, 6, 7}
    # round(3 + 4 (1000 - lambda) / 600)
    for w, l in zip(wl, L):
        assert l == int(np.clip(np.round(3 + 4 * (1000e-9 - w) / 600e-9), 3, 7))


def test_sweep_specs_match_direct_formulas():
    pos, rad = SW.drude_cluster(N=6, seed=3, box=0.8e-6)
    mat = drude_material(**DRUDE)
    wl = np.array([400, 550, 700, 1000]) * nm
    specs = SW.sweep_specs(pos, rad, mat, wl, SW.adaptive_lmax)
    from miepy_gb300.mie import mie_coefficients
    from miepy_gb300.sources import plane_wave
    for s, w in zip(specs, wl):
        hw = 1239.84193e-9 / w
        eps = 9.0 - 81.0 / (hw ** 2 + 1j * 0.07 * hw)
        ms, mi = mie_coefficients(rad, eps, 1.0, 1.0, 1.0, 2 * np.pi / w, s["lmax"])
        np.testing.assert_allclose(s["mie_scat"], ms, rtol=1e-13)
        np.testing.assert_allclose(s["mie_int"], mi, rtol=1e-13)
        ps = plane_wave.from_string("x").structure(pos, 2 * np.pi / w, s["lmax"])
        np.testing.assert_allclose(s["p_src"][..., 0], ps, rtol=1e-13)
        assert s["p_src"].shape == (6, 2, s["lmax"] * (s["lmax"] + 2), 1)


@pytest.mark.gpu
def test_small_sweep_against_oracle_exact():
    from oracle import oracle as O
    pos, rad = SW.drude_cluster(N=5, seed=3, box=0.6e-6)
    mat = drude_material(**DRUDE)
    wl = np.linspace(400, 1000, 5) * nm                     # lmax 7, 6, 5, 4, 3
    specs = SW.sweep_specs(pos, rad, mat, wl, SW.adaptive_lmax)
    res_m = SW.wavelength_sweep(None, None, None, None, specs=specs, precision="mixed", tol=1e-10)
    res_d = SW.wavelength_sweep(None, None, None, None, specs=specs, precision="fp64", tol=1e-13)
    assert np.all(res_m.status == 0) and np.all(res_d.status == 0)
    assert sorted(set(res_m.lmax.tolist())) == [3, 4, 5, 6, 7]
    for w, s in enumerate(specs):
        T = O.sphere_aggregate_tmatrix(s["position"], s["mie_scat"].reshape(5, -1), s["k"])
        D = T.shape[0]
        p_inc = O.solve_linear_system_profiled(T.reshape(D, D), s["p_src"][..., 0].reshape(-1), "exact")[0]
        p_inc = p_inc.reshape(5, 2, -1)
        L = s["lmax"]
        n = np.array([nn for nn in range(1, L + 1) for _ in range(-nn, nn + 1)])
        p_scat = p_inc * s["mie_scat"][:, :, n - 1]
        k = s["k"]
        cext = 4 * np.pi / k ** 2 * np.sum(np.real(np.conj(s["p_src"][..., 0]) * p_scat))
        assert abs(res_d.C_ext[w, 0] - cext) / abs(cext) < 1e-9
        assert abs(res_m.C_ext[w, 0] - cext) / abs(cext) < 1e-6
    # the batch gives each wavelength what a batch of that wavelength alone gives
    b = res_d.batches[0]
    for w in (0, 4):
        alone = SW.wavelength_sweep(None, None, None, None, specs=[specs[w]], precision="fp64", tol=1e-13)
        np.testing.assert_allclose(res_d.C_ext[w], alone.C_ext[0], rtol=1e-10)
        x_batch = b.cluster_view(w, b.x).cpu().numpy()
        a = alone.batches[0]
        np.testing.assert_allclose(x_batch, a.cluster_view(0, a.x).cpu().numpy(), rtol=1e-9,
                                   atol=1e-12 * np.max(np.abs(x_batch)))


@pytest.mark.gpu
def test_full_sweep_n100_256_wavelengths():
    """Config: N=100 Drude spheres (seed 3), 256 wavelengths 400-1000 nm, adaptive
    lmax 3-7, mixed precision in one ragged batch; FP64 solves of one wavelength per
    lmax as the reference (C_ext within 1e-6)."""
    import torch
    pos, rad = SW.drude_cluster(N=100, seed=3)
    mat = drude_material(**DRUDE)
    wl = np.linspace(400, 1000, 256) * nm
    specs = SW.sweep_specs(pos, rad, mat, wl, SW.adaptive_lmax)
    free = torch.cuda.mem_get_info()[0]
    res = SW.wavelength_sweep(None, None, None, None, specs=specs, precision="mixed", tol=1e-8,
                              max_batch_bytes=int(0.6 * free))
    assert np.all(res.status == 0), res.status
    assert np.all(res.C_ext > 0) and np.all(res.C_abs > 0) and np.all(res.C_sca > 0)
    np.testing.assert_allclose(res.C_sca + res.C_abs, res.C_ext, rtol=1e-12)
    del res
    torch.cuda.empty_cache()
    picks = [int(np.argmax(SW.adaptive_lmax(wl) == L)) for L in (3, 4, 5, 6, 7)]
    sub = [specs[i] for i in picks]
    r64 = SW.wavelength_sweep(None, None, None, None, specs=sub, precision="fp64", tol=1e-10)
    rmx = SW.wavelength_sweep(None, None, None, None, specs=sub, precision="mixed", tol=1e-8)
    assert np.all(r64.status == 0)
    err = np.abs(rmx.C_ext - r64.C_ext) / np.abs(r64.C_ext)
    assert np.max(err) < 1e-6, err
