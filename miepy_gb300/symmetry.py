"""Periodic lattices for sphere_cluster(symmetry=...) (src/miepy/symmetry.py).

A lattice is a generator of cell offsets: ``generate(N)`` returns the x, y, z arrays
of the lattice vectors (the origin cell excluded) that the periodic aggregate
T-matrix sums over; the reference calls it with N = 5000
(interactions.py:168).  The lattice constant is the argument ``k`` of each
constructor, as in the reference.
"""

import numpy as np


class periodic_lattice:
    def __init__(self, generate_func):
        self.generate_func = generate_func

    def generate(self, N):
        return self.generate_func(N)


def _line(N, a):
    """N // 2 cells on each side of the origin: -a, -2a, ..., then a, 2a, ... (symmetry.py:12-18)."""
    steps = a * np.arange(1, N // 2 + 1, dtype=float)
    return np.concatenate([-steps, steps])


def _translation_1d(axis, a):
    def generate(N):
        line = _line(N, a)
        xyz = [np.zeros_like(line) for _ in range(3)]
        xyz[axis] = line
        return tuple(xyz)

    return periodic_lattice(generate)


def x_translation_1d(k):
    """Cells along x with spacing k (symmetry.py:21-29)."""
    return _translation_1d(0, k)


def y_translation_1d(k):
    """Cells along y with spacing k.  (The reference's version, symmetry.py:32-40,
    reads an unset variable and raises; this one returns the y line.)"""
    return _translation_1d(1, k)


def z_translation_1d(k):
    """Cells along z with spacing k (the reference's symmetry.py:43-51 raises, as for y)."""
    return _translation_1d(2, k)


def square_lattice_2d(k):
    """An odd Nx x Nx square lattice in the xy plane centred on the origin, Nx the
    largest odd number <= sqrt(N) rounded as int(sqrt(N)) // 2 * 2 + 1, cells ordered
    by distance from the origin, the origin removed (symmetry.py:54-78)."""

    def generate(N):
        Nx = int(np.sqrt(N)) // 2 * 2 + 1
        x = np.arange(Nx) * k
        x = x - np.average(x)
        X, Y = np.meshgrid(x, x)
        xs, ys = X.ravel(), Y.ravel()
        order = np.argsort(xs ** 2 + ys ** 2, kind="stable")
        xs, ys = xs[order][1:], ys[order][1:]
        return xs, ys, np.zeros_like(xs)

    return periodic_lattice(generate)
