"""Import the reference's own Python layer on top of the CPU oracle.

TEST INFRASTRUCTURE ONLY, and only in a checkout that has the reference tree
(its ``src/`` directory, located through ``MIEPY_REFERENCE_SRC``).  The
reference package ``miepy`` imports a compiled module ``miepy.cpp`` (pybind11
over Eigen and GSL) that cannot be built without those libraries; this module
registers the oracle (``oracle/oracle.py``) under that name with the same
submodules and function names, plus small stand-ins for four optional third-
party imports (``quaternion``, ``yaml``, ``matplotlib.colors``, ``spherical``).  The reference's
Python files themselves run unmodified; the only run-time adjustment is the
location of the material database, which the reference ships zipped.

It is used to (1) pin the oracle with the reference's own physics tests and
(2) generate the golden fixtures under ``tests/golden/``.
"""

from __future__ import annotations

import enum
import importlib
import os
import sys
import tempfile
import types
import zipfile

import numpy as np

from . import oracle as O

DEFAULT_REF_SRC = os.environ.get("MIEPY_REFERENCE_SRC", "")


# ---------------------------------------------------------------- enums --
class vsh_mode(enum.Enum):   # cpp/src/vsh_functions.hpp:10-15
    outgoing = 0
    ingoing = 1
    incident = 2
    interior = 3


class solver(enum.Enum):   # cpp/src/interactions.hpp:8-11
    bicgstab = 0
    exact = 1


def _method_name(method):
    if isinstance(method, solver):
        return method.name
    return str(method)


# ------------------------------------------------------- miepy.cpp stand-in --
def _module(name, **attrs):
    m = types.ModuleType(name)
    for k, v in attrs.items():
        setattr(m, k, v)
    m.__all__ = [k for k in attrs if not k.startswith("_")]
    return m


def _solve_linear_system(agg_tmatrix, p_src, method=solver.bicgstab, M_inv_blocks=None, block_size=0):
    if M_inv_blocks is not None:
        raise NotImplementedError("block preconditioner is outside the sphere-cluster hot path")
    return O.solve_linear_system(agg_tmatrix, p_src, _method_name(method))


def _bicgstab_profiled(A, b, maxiter=1000, tolerance=1e-5):
    return O.bicgstab(A, b, maxiter, tolerance)


def _not_in_scope(*_a, **_k):
    raise NotImplementedError("not part of the sphere-cluster hot path restated by the oracle")


def _expand_E_cluster(pos, p_expand, mode, x, y, z, k):
    return O.expand_E_cluster(pos, p_expand, mode, x, y, z, k).T


def build_cpp_module():
    special = _module(
        "miepy.cpp.special",
        spherical_jn=O.spherical_jn, spherical_yn=O.spherical_yn, spherical_hn=O.spherical_hn,
        spherical_hn_2=O.spherical_hn_2, riccati_1=O.riccati_1, riccati_2=O.riccati_2, riccati_3=O.riccati_3,
        associated_legendre=O.associated_legendre, pi_func=O.pi_func, tau_func=O.tau_func,
        wigner_3j=O.wigner_3j, a_func=O.a_func, b_func=O.b_func,
    )
    vsh_functions = _module(
        "miepy.cpp.vsh_functions", vsh_mode=vsh_mode, Emn=O.Emn, vsh_electric=O.vsh_electric,
        vsh_magnetic=O.vsh_magnetic, expand_E_cluster=_expand_E_cluster,
    )
    vsh_translation = _module(
        "miepy.cpp.vsh_translation", vsh_translation=O.vsh_translation, vsh_translation_numpy=O.vsh_translation_numpy,
        vsh_translation_eigen=O.vsh_translation_numpy, vsh_translation_lambda_py=O.vsh_translation_numpy,
        create_vsh_cache_map=_not_in_scope,
    )
    interactions = _module(
        "miepy.cpp.interactions", solver=solver, bicgstab=lambda A, b, maxiter, tolerance: O.bicgstab(A, b, maxiter, tolerance)[0],
        bicgstab_profiled=_bicgstab_profiled, bicgstab_preconditioned_profiled=_not_in_scope,
        sphere_aggregate_tmatrix=O.sphere_aggregate_tmatrix, particle_aggregate_tmatrix=O.particle_aggregate_tmatrix,
        reflection_matrix_nia=O.reflection_matrix_nia, solve_linear_system=_solve_linear_system,
    )
    forces = _module("miepy.cpp.forces", force=O.force, torque=O.torque, force_all=O.force_all,
                     torque_all=O.torque_all)

    def _pcs(p_scat, p_inc, p_src, k):
        return O.particle_cross_sections(p_scat, p_inc, p_src, k)

    flux = _module("miepy.cpp.flux", particle_cross_sections=_pcs, cluster_cross_sections=O.cluster_cross_sections)
    decomposition = _module("miepy.cpp.decomposition", trapz=O.trapz, trapz_2d=O.trapz_2d,
                            integrate_phase=O.integrate_phase, grid_interpolate=_not_in_scope)
    tmatrix = _module("miepy.cpp.tmatrix", has_extended_precision=False, compute_spheroid=_not_in_scope,
                      compute_cylinder=_not_in_scope, compute_rounded_cylinder=_not_in_scope,
                      compute_ellipsoid=_not_in_scope, compute_regular_prism=_not_in_scope)
    cpp = _module("miepy.cpp", special=special, vsh_functions=vsh_functions, vsh_translation=vsh_translation,
                  interactions=interactions, forces=forces, flux=flux, decomposition=decomposition, tmatrix=tmatrix)
    cpp.__path__ = []
    subs = {"special": special, "vsh_functions": vsh_functions, "vsh_translation": vsh_translation,
            "interactions": interactions, "forces": forces, "flux": flux, "decomposition": decomposition,
            "tmatrix": tmatrix}
    return cpp, subs


# ----------------------------------------------------- third-party stand-ins --
class _Quat:
    """Quaternion (array-valued components allowed) with the operations the
    reference's sources and coordinate helpers use."""

    def __init__(self, w, x, y, z):
        self.w, self.x, self.y, self.z = (np.asarray(c, dtype=float) for c in (w, x, y, z))

    def __mul__(self, o):
        a1, b1, c1, d1 = self.w, self.x, self.y, self.z
        a2, b2, c2, d2 = o.w, o.x, o.y, o.z
        return _Quat(a1 * a2 - b1 * b2 - c1 * c2 - d1 * d2, a1 * b2 + b1 * a2 + c1 * d2 - d1 * c2,
                     a1 * c2 - b1 * d2 + c1 * a2 + d1 * b2, a1 * d2 + b1 * c2 - c1 * b2 + d1 * a2)

    def inverse(self):
        n = self.w ** 2 + self.x ** 2 + self.y ** 2 + self.z ** 2
        return _Quat(self.w / n, -self.x / n, -self.y / n, -self.z / n)

    def __eq__(self, o):
        return isinstance(o, _Quat) and all(np.array_equal(a, b) for a, b in
                                            zip((self.w, self.x, self.y, self.z), (o.w, o.x, o.y, o.z)))

    def __ne__(self, o):
        return not self.__eq__(o)

    def __hash__(self):
        return hash((float(np.sum(self.w)), float(np.sum(self.x)), float(np.sum(self.y)), float(np.sum(self.z))))

    @property
    def components(self):
        return np.array([self.w, self.x, self.y, self.z])


def _quaternion_module():
    m = types.ModuleType("quaternion")
    m.one = _Quat(1, 0, 0, 0)
    m.quaternion = _Quat

    def from_spherical_coords(theta, phi):   # exp(phi z/2) * exp(theta y/2)
        theta, phi = np.broadcast_arrays(np.asarray(theta, float), np.asarray(phi, float))
        z0 = np.zeros_like(theta)
        qz = _Quat(np.cos(phi / 2), z0, z0, np.sin(phi / 2))
        qy = _Quat(np.cos(theta / 2), z0, np.sin(theta / 2), z0)
        return qz * qy

    def as_rotation_matrix(q):
        n = np.sqrt(q.w ** 2 + q.x ** 2 + q.y ** 2 + q.z ** 2)
        w, x, y, z = q.w / n, q.x / n, q.y / n, q.z / n
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        return np.moveaxis(R, (0, 1), (-2, -1))

    def as_spherical_coords(q):
        th = 2 * np.arctan2(np.sqrt(q.x ** 2 + q.y ** 2), np.sqrt(q.w ** 2 + q.z ** 2))
        ph = np.arctan2(q.z, q.w) + np.arctan2(-q.x, q.y)
        return np.moveaxis(np.array([th, ph]), 0, -1)

    m.from_spherical_coords = from_spherical_coords
    m.as_rotation_matrix = as_rotation_matrix
    m.as_spherical_coords = as_spherical_coords
    return m


def _spherical_module():
    """Stand-in for the ``spherical`` package's wigner_D(R, ell_min, ell_max), the
    only function the reference takes from it (vsh/vsh_rotation.py:8-29).  For the
    rotation R = Rz(alpha) Ry(beta) Rz(gamma) of quaternion components (w, x, y, z)
    it returns, flattened [m', m] per ell, the complex conjugate of the standard
    D-matrix exp(-i m' alpha) d^ell(beta) exp(-i m gamma), with
    d^ell(beta) = exp(-i beta J_y) evaluated as a matrix exponential of the angular
    momentum generator (J_y = (J+ - J-) / 2i on |ell, m>), so that the reference's
    conj(D) (-1)^(m - m') is the standard rotation of its VSH coefficients."""
    from scipy.linalg import expm

    m = types.ModuleType("spherical")

    def euler_zyz(q):
        w, x, y, z = (float(np.ravel(c)[0]) for c in q)
        beta = 2 * np.arctan2(np.hypot(x, y), np.hypot(w, z))
        apc, amc = np.arctan2(z, w), np.arctan2(-x, y)
        return apc + amc, beta, apc - amc

    def d_small(ell, beta):
        ms = np.arange(-ell, ell + 1, dtype=float)
        jp = np.diag(np.sqrt(ell * (ell + 1) - ms[:-1] * (ms[:-1] + 1)), -1)   # <m+1|J+|m>
        jy = (jp - jp.T) / 2j
        return expm(-1j * beta * jy).real

    def wigner_D(R, ell_min, ell_max):
        alpha, beta, gamma = euler_zyz(R)
        out = []
        for ell in range(ell_min, ell_max + 1):
            ms = np.arange(-ell, ell + 1)
            D = np.exp(-1j * ms[:, None] * alpha) * d_small(ell, beta) * np.exp(-1j * ms[None, :] * gamma)
            out.append(np.conj(D).ravel())
        return np.concatenate(out)

    m.wigner_D = wigner_D
    return m


def _yaml_module():
    """Reads the refractiveindex.info-style files of the reference's database."""
    m = types.ModuleType("yaml")

    class SafeLoader:   # noqa: N801 - mirrors the yaml API name
        pass

    def load(f, Loader=None):
        text = f.read() if hasattr(f, "read") else str(f)
        lines = text.splitlines()
        data_lines, inside = [], False
        for ln in lines:
            s = ln.strip()
            if s.startswith("data:"):
                inside = True
                continue
            if inside:
                if not s or s.endswith(":") or s.startswith("-") or ":" in s:
                    if data_lines:
                        break
                    continue
                data_lines.append(s)
        return {"DATA": [{"data": "\n".join(data_lines)}]}

    m.SafeLoader = SafeLoader
    m.load = load
    m.safe_load = lambda f: load(f)
    return m


def _matplotlib_modules():
    mpl = types.ModuleType("matplotlib")
    colors = types.ModuleType("matplotlib.colors")
    mpl.colors = colors
    mpl.__path__ = []
    return mpl, colors


_MATERIAL_DIR = None


def _material_root(ref_src):
    global _MATERIAL_DIR
    if _MATERIAL_DIR is None:
        d = tempfile.mkdtemp(prefix="miepy_materials_")
        with zipfile.ZipFile(os.path.join(ref_src, "miepy", "materials", "database.zip")) as z:
            z.extractall(d)
        _MATERIAL_DIR = d
    return _MATERIAL_DIR


def import_reference(ref_src: str | None = None):
    """Import the reference ``miepy`` package with the oracle as ``miepy.cpp``.

    Raises ImportError when the reference tree is not available."""
    ref_src = ref_src or DEFAULT_REF_SRC
    if not ref_src or not os.path.isdir(os.path.join(ref_src, "miepy")):
        raise ImportError("reference source tree not available (set MIEPY_REFERENCE_SRC)")
    if "miepy" in sys.modules and getattr(sys.modules["miepy"], "_oracle_shim", False):
        return sys.modules["miepy"]

    for name, factory in (("quaternion", _quaternion_module), ("yaml", _yaml_module),
                          ("spherical", _spherical_module)):
        try:
            importlib.import_module(name)
        except ImportError:
            sys.modules[name] = factory()
    try:
        importlib.import_module("matplotlib.colors")
    except ImportError:
        mpl, colors = _matplotlib_modules()
        sys.modules["matplotlib"] = mpl
        sys.modules["matplotlib.colors"] = colors

    cpp, subs = build_cpp_module()
    sys.modules["miepy.cpp"] = cpp
    for k, v in subs.items():
        sys.modules["miepy.cpp." + k] = v
    if ref_src not in sys.path:
        sys.path.insert(0, ref_src)
    miepy = importlib.import_module("miepy")
    miepy._oracle_shim = True

    load = importlib.import_module("miepy.material_functions.load")
    root = None

    def get_filepath(name, author):
        nonlocal root
        if root is None:
            root = _material_root(ref_src)
        for base in (os.path.join(root, "database", "main"), os.path.join(root, "main")):
            p = os.path.join(base, name, f"{author}.yml")
            if os.path.exists(p):
                return p
        return os.path.join(root, "database", "main", name, f"{author}.yml")

    load.get_filepath = get_filepath
    return miepy
