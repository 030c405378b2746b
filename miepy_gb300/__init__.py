"""miepy_gb300: the sphere-cluster aggregate T-matrix path of miepy on GB300.

Public API mirrors the reference's names: sphere_cluster, solver, materials,
constant_material, function_material, dielectric, sources.plane_wave,
mode_indices; plus batched sweeps (sweep) and the solve server (server).
The compute path is the CUDA extension in csrc/, reached through the C ABI of
include/miepy_gb300.h.
"""

from . import backend, beams, materials as _materials_mod, sources, sweep, symmetry
from .beams import gaussian_beam
from .cluster import cross_sections, solver, sphere_cluster
from .interface import interface
from .tmatrix_cluster import cluster, sphere, tmatrix_cluster, tmatrix_sphere
from .engine import ClusterBatch, footprint_bytes
from .materials import (constant_material, dielectric, drude_material, function_material, material_struct,
                        materials)
from .mie import mie_coefficients
from .modes import lmax_to_rmax, mode_indices, reduced_index, rmax_to_lmax
from .sources import plane_wave

sources.gaussian_beam = gaussian_beam

__version__ = "1.0.0"


def install_backend():
    """Make ``miepy.backends.set_backend('gpu')`` use this package."""
    return backend.install()
