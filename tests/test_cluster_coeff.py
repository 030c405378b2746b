"""Cluster coefficients, cluster cross-sections per multipole and far fields (the
reference's cluster_coefficients, cross_sections_per_multipole, E_angular and
H_angular) against fixtures made by the reference itself.

Tolerances: p_cluster within 1e-10 of its largest coefficient at the cluster's own
lmax and lmax + 1 (the reference's j_n recurrence loses digits for orders above k r,
so the bar is relative to the largest coefficient); far fields within 1e-8 of the
largest component (at the reference's far radius R = 1e6 wavelengths the phase k R
~ 6e6 carries ~1e-9 of rounding in either implementation); cluster cross-sections
within 1e-9.
"""

import numpy as np
import pytest
import torch

import miepy_gb300 as gb
from miepy_gb300 import _native as nat
from tests import _golden as G

pytestmark = pytest.mark.gpu


def _p_cluster(g, lmax_c):
    dev = torch.device("cuda", 0)
    N, L = g["position"].shape[0], int(g["lmax"])
    pos = torch.from_numpy(np.ascontiguousarray(g["position"])).to(dev)
    ps = torch.from_numpy(np.ascontiguousarray(g["p_scat"])).to(dev)
    L_ = nat.lib()
    ws = torch.empty(L_.gb_cluster_coefficients_workspace_size(N, lmax_c), dtype=torch.uint8, device=dev)
    out = torch.empty(2 * lmax_c * (lmax_c + 2), dtype=torch.complex128, device=dev)
    origin = np.zeros(3)
    nat.check(L_.gb_cluster_coefficients(N, L, nat.ptr(pos), nat.ptr(ps), float(g["k_b"]), origin.ctypes.data,
                                         lmax_c, nat.ptr(out), nat.ptr(ws), ws.numel(),
                                         torch.cuda.current_stream().cuda_stream), "cluster coefficients")
    return out.cpu().numpy().reshape(2, -1)


@pytest.mark.parametrize("name", G.CASES)
def test_cluster_coefficients_match_reference(name):
    g = G.load(name)
    L = int(g["lmax"])
    for key, lc in (("p_cluster", L), ("p_cluster_lmax_plus1", min(L + 1, 8))):
        ref = g[key]
        got = _p_cluster(g, lc)
        assert np.max(np.abs(got - ref)) <= 1e-10 * np.max(np.abs(ref)), (name, key)


@pytest.mark.parametrize("name", G.CASES)
def test_far_fields_match_reference(name):
    g = G.load(name)
    dev = torch.device("cuda", 0)
    N, L = g["position"].shape[0], int(g["lmax"])
    k = float(g["k_b"])
    th, ph = g["far_theta"], g["far_phi"]
    R = np.full_like(th, 1e6 * 2 * np.pi / k)
    d = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a).reshape(-1)).to(dev, dtype=dt)
    pos, ps = d(g["position"], torch.float64), d(g["p_scat"], torch.complex128)
    Rt, Tt, Pt = d(R, torch.float64), d(th, torch.float64), d(ph, torch.float64)
    origin = np.zeros(3)
    for key, mag, hfac in (("E_angular", 0, 1.0), ("H_angular", 1, -1j * np.sqrt(complex(g["eps_b"]) / complex(g["mu_b"])))):
        out = torch.empty((th.size, 2), dtype=torch.complex128, device=dev)
        nat.check(nat.lib().gb_far_field(N, L, nat.ptr(pos), nat.ptr(ps), k, origin.ctypes.data, th.size,
                                         nat.ptr(Rt), nat.ptr(Tt), nat.ptr(Pt), mag, float(np.real(hfac)),
                                         float(np.imag(hfac)), nat.ptr(out), torch.cuda.current_stream().cuda_stream),
                  "far field")
        got = out.cpu().numpy().T
        ref = g[key]
        assert np.max(np.abs(got - ref)) <= 1e-8 * np.max(np.abs(ref)), (name, key)


def test_public_api_dimer():
    g = G.load("dimer_lmax6_exact")
    nm = 1e-9
    c = gb.sphere_cluster(position=[[-100 * nm, 0, 0], [100 * nm, 0, 0]], radius=75 * nm,
                          material=gb.constant_material(index=0.2 + 3.0j), source=gb.plane_wave.from_string("x"),
                          wavelength=600 * nm, lmax=6, medium=gb.materials.water(), method=gb.solver.exact)
    C = c.cross_sections_per_multipole()
    np.testing.assert_allclose(np.array([np.asarray(v) for v in C]), g["cluster_xs_per_multipole"], rtol=1e-9,
                               atol=1e-9 * np.max(np.abs(g["cluster_xs_per_multipole"])))
    E = c.E_angular(g["far_theta"], g["far_phi"])
    assert np.max(np.abs(E - g["E_angular"])) <= 1e-8 * np.max(np.abs(g["E_angular"]))
