"""CPU tests: the C-ABI library builds, loads and exports every symbol the header
declares; host-side pieces (materials, Mie coefficients, plane-wave
decomposition, mode indices) match the reference's outputs in the golden
fixtures.  No GPU calls."""

import ctypes
import os
import re

import numpy as np
import pytest

import miepy_gb300 as gb
from miepy_gb300 import _native, build
from tests import _golden as G
from tests.conftest import ROOT

HEADER = os.path.join(ROOT, "include", "miepy_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gb_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # every declared function has a ctypes signature
    assert set(syms) <= set(_native.SIGNATURES), set(syms) - set(_native.SIGNATURES)


def test_version_and_error_plumbing_without_gpu():
    lib = _native.lib()
    assert lib.gb_version() >= 10000
    M = ctypes.c_int(0)
    assert lib.gb_tables_count(4, ctypes.byref(M)) == 0
    assert M.value == 300   # canonical (n, m, v<=n, u) tuples at lmax 4
    assert lib.gb_tables_count(11, ctypes.byref(M)) == _native.GB_BAD_ARG
    assert "lmax" in _native.last_error()


@pytest.mark.parametrize("lmax,expected", [(2, 36), (3, 120), (4, 300), (5, 630), (6, 1176), (7, 2016), (8, 3240)])
def test_tuple_counts(lmax, expected):
    M = ctypes.c_int(0)
    assert _native.lib().gb_tables_count(lmax, ctypes.byref(M)) == 0
    assert M.value == expected


def test_mode_indices_order():
    idx = list(gb.mode_indices(3))
    assert idx[0] == (0, 1, -1) and idx[-1] == (14, 3, 3)
    assert all(r == gb.reduced_index(n, m) for r, n, m in idx)


@pytest.mark.parametrize("name", G.CASES)
def test_host_mie_and_source_match_reference(name):
    g = G.load(name)
    lmax = int(g["lmax"])
    ms, mi = gb.mie_coefficients(g["radius"], g["eps"], g["mu"], g["eps_b"], g["mu_b"], g["k_b"], lmax)
    np.testing.assert_allclose(ms, g["mie_scat"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(mi, g["mie_int"], rtol=1e-12, atol=1e-300)


def test_plane_wave_structure_matches_reference():
    for name, pol in (("dimer_lmax6_exact", "x"), ("ag5_lmax2_exact", "rhc"), ("rand12_lmax3_exact", "y")):
        g = G.load(name)
        src = gb.plane_wave.from_string(polarization=pol)
        p = src.structure(g["position"], g["k_b"], int(g["lmax"]))
        np.testing.assert_allclose(p, g["p_src"], rtol=1e-13, atol=1e-16)


def test_benchmark_inputs_match_reference_at_full_size():
    """The benchmark's cluster (seed 2), Mie coefficients and both plane waves are
    the reference's (config2 fixture); the sweep's Drude cluster at 400 nm and the
    serving-size request reproduce theirs too."""
    import bench

    g = G.load("config2_n200_lmax4_exact")
    w = bench.workload_inputs()
    np.testing.assert_allclose(w["position"], g["position"], rtol=1e-15, atol=0)   # the reference stores them to 1 ulp
    np.testing.assert_allclose(w["radius"], g["radius"], rtol=1e-15, atol=0)
    np.testing.assert_allclose(w["mie_scat"], g["mie_scat"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(w["mie_int"], g["mie_int"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(w["p_src"], np.stack([g["p_src_x"], g["p_src_y"]], axis=-1), rtol=1e-13, atol=1e-16)
    from miepy_gb300 import sweep as SW
    s = G.load("sweep_n100_lmax7_400nm_exact")
    pos, rad = SW.drude_cluster(N=100, seed=3)
    np.testing.assert_allclose(pos, s["position"], rtol=1e-15, atol=0)
    eps = gb.drude_material(9.0, 9.0, 0.07).eps(400e-9)
    np.testing.assert_allclose(eps, s["eps"][0], rtol=1e-14)
    for name in ("sweep_n100_lmax7_400nm_exact", "serve_n300_lmax6_exact"):
        h = G.load(name)
        lmax = int(h["lmax"])
        md = gb.material_struct([gb.constant_material(eps=complex(e)) for e in np.broadcast_to(
            h["eps"] if "eps" in h else (1.9 + 0.05j) ** 2, h["radius"].shape)],
            gb.constant_material(eps=1.0, mu=1.0), wavelength=float(h["wavelength"]))
        ms, mi = gb.mie_coefficients(h["radius"], md.eps, md.mu, md.eps_b, md.mu_b, md.k_b, lmax)
        np.testing.assert_allclose(ms, h["mie_scat"], rtol=1e-11, atol=1e-300)
        np.testing.assert_allclose(mi, h["mie_int"], rtol=1e-11, atol=1e-300)
        p = gb.plane_wave.from_string("x").structure(h["position"], md.k_b, lmax)
        np.testing.assert_allclose(p, h["p_src"], rtol=1e-13, atol=1e-16)


def test_pi_tau_limits_and_interior_values():
    from oracle import oracle as O
    th = np.array([0.0, 0.3, 1.1, 2.0, np.pi])
    for n in range(1, 7):
        for m in range(-n, n + 1):
            np.testing.assert_allclose(gb.special.pi_func(n, m, th), O.pi_func(n, m, th), rtol=1e-12, atol=1e-12)
            np.testing.assert_allclose(gb.special.tau_func(n, m, th), O.tau_func(n, m, th), rtol=1e-12, atol=1e-12)


def test_materials_drude_and_struct():
    d = gb.drude_material(9.0, 9.0, 0.07)
    w = 1239.84193 / 600.0
    assert d.eps(600e-9) == pytest.approx(9.0 - 81.0 / (w ** 2 + 1j * 0.07 * w))
    ms = gb.material_struct([gb.constant_material(index=1.5)], gb.materials.water(), wavelength=500e-9)
    assert ms.k_b == pytest.approx(2 * np.pi * 1.33 / 500e-9)
    assert ms.eps[0] == pytest.approx(2.25)


def test_footprint_grows_with_size():
    a = gb.footprint_bytes(10, 3, 1, "fp64")
    b = gb.footprint_bytes(20, 3, 1, "fp64")
    c = gb.footprint_bytes(20, 3, 1, "mixed_fp64res")
    d = gb.footprint_bytes(20, 3, 1, "fp32")
    assert b > a and c > b > d


def test_no_cpu_fallback_when_cuda_missing():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(RuntimeError, match="CUDA"):
        gb.sphere_cluster(position=[[0, 0, 0], [3e-7, 0, 0]], radius=5e-8, material=gb.constant_material(index=1.5),
                          source=gb.plane_wave.from_string("x"), wavelength=6e-7, lmax=2)


@pytest.mark.parametrize("lmax", range(1, 9))
def test_model_gemv_shapes_stay_within_the_padding(lmax):
    """The GEMV lane shape the launches use without autotuning covers the block, and
    its column overshoot fits the 256 B of shared-memory padding after a warp's last
    stage for complex128 (16 B) elements (host-side shape logic only, no GPU)."""
    lib = _native.lib()
    B = 2 * lmax * (lmax + 2)
    for prec in (0, 2):   # GB_PREC_FP64 (complex128 pass), GB_PREC_FP32 (complex64 pass)
        lpr, cpl = ctypes.c_int(0), ctypes.c_int(0)
        assert lib.gb_gemv_shape(B, prec, 2, ctypes.byref(lpr), ctypes.byref(cpl)) == 0
        cols = lpr.value * cpl.value
        assert cols >= B
        assert (cols - B) * 16 <= 256
