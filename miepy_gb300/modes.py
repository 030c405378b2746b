"""(n, m) mode indices in the order the reference uses (vsh/mode_indices.py:1-91)."""


def lmax_to_rmax(lmax):
    return lmax * (lmax + 2)


def rmax_to_lmax(rmax):
    return int(-1 + (1 + rmax) ** 0.5)


def reduced_index(n, m):
    return n * (n + 2) - n + m - 1


class mode_indices:
    """Iterates (r, n, m) for n = 1..lmax, m = -n..n; r = n(n+2) - n + m - 1."""

    def __init__(self, lmax):
        self.lmax = int(lmax)

    def __iter__(self):
        r = 0
        for n in range(1, self.lmax + 1):
            for m in range(-n, n + 1):
                yield r, n, m
                r += 1

    def __len__(self):
        return self.lmax

    def __repr__(self):
        return f"mode_indices(lmax={self.lmax})"
