"""Seeded synthetic instances with the shapes and value distributions of the five workloads.

The reference's own instance (SB/CUDA_GPU/WK2000_1.rud, a 2000-spin complete graph) is not
shipped; the N=2000 complete graph with iid +-1 couplings below stands in for it. Seeds are
1234 + instance id. Generators follow the reference's writers in shape (N header, "i j w" lines,
"i i h" field lines as in SA_king/CUDA_GPU/tests/king.py:27-28).
"""
from __future__ import annotations

import numpy as np


def complete_pm1(n: int = 2000, seed: int = 1234) -> np.ndarray:
    """Complete graph, J_ij iid uniform in {-1, +1}, symmetric, zero diagonal."""
    rng = np.random.default_rng(seed)
    up = np.triu(rng.integers(0, 2, size=(n, n), dtype=np.int8) * 2 - 1, 1).astype(np.float32)
    return up + up.T


def gaussian(n: int = 8192, seed: int = 1234, h_var: float = 0.1):
    """Complete graph, J_ij iid N(0, 1/N) (variance), h_i iid N(0, h_var)."""
    rng = np.random.default_rng(seed)
    a = rng.standard_normal((n, n), dtype=np.float32) * np.float32(1.0 / np.sqrt(n))
    up = np.triu(a, 1)
    J = up + up.T
    h = (rng.standard_normal(n) * np.sqrt(h_var)).astype(np.float32)
    return J, h


def erdos_renyi(n: int, density: float, seed: int, jmax: int = 1, allow_zero: bool = False):
    """G(n, p) with integer couplings: +-1 (jmax = 1) or uniform in [-jmax, jmax]."""
    rng = np.random.default_rng(seed)
    mask = np.triu(rng.random((n, n)) < density, 1)
    if jmax == 1 and not allow_zero:
        w = (rng.integers(0, 2, size=(n, n)) * 2 - 1).astype(np.float32)
    else:
        w = rng.integers(-jmax, jmax + 1, size=(n, n)).astype(np.float32)
    up = np.where(mask, w, 0.0).astype(np.float32)
    return up + up.T


def nmfa_fully(n: int = 1024, seed: int = 1234) -> np.ndarray:
    """The NMFA test graph's distribution (NMFA/CUDA_GPU/tests/fully.py:6-15): each pair is an edge
    with probability 1/2, its weight uniform in {-1, 0, +1}; seeded."""
    return erdos_renyi(n, 0.5, seed, jmax=1, allow_zero=True)


def uneven_batch(count: int = 512, nmin: int = 64, nmax: int = 4096, seed: int = 1234):
    """(N, density, seed) of the uneven-size batch: N ~ U[nmin, nmax], density ~ U[0.05, 1]."""
    rng = np.random.default_rng(seed)
    ns = rng.integers(nmin, nmax + 1, size=count)
    dens = rng.uniform(0.05, 1.0, size=count)
    return [(int(ns[k]), float(dens[k]), 1234 + k) for k in range(count)]


def serving_stream(count: int = 2000, rate: float = 200.0, nmin: int = 128, nmax: int = 16384,
                   smin: int = 500, smax: int = 4000, seed: int = 1234):
    """Poisson arrivals: (arrival_s, N, density, steps, seed) per request."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps) - gaps[0]
    ns = np.exp(rng.uniform(np.log(nmin), np.log(nmax), size=count)).astype(int)
    dens = rng.uniform(0.01, 1.0, size=count)
    steps = rng.integers(smin, smax + 1, size=count)
    return [(float(t[k]), int(ns[k]), float(dens[k]), int(steps[k]), 1234 + k)
            for k in range(count)]


def write_graph(path: str, J: np.ndarray, h=None, header_edges: bool = False) -> None:
    """Write the reference's text format: N (optionally 'N E'), then 'i j w' for i < j, 0-based,
    then 'i i h' lines for nonzero fields."""
    n = J.shape[0]
    iu, ju = np.nonzero(np.triu(J, 1))
    w = J[iu, ju]
    with open(path, "w") as f:
        f.write(f"{n} {len(iu)}\n" if header_edges else f"{n}\n")
        integral = np.all(w == np.floor(w))
        fmt = "%d %d %d\n" if integral else "%d %d %.9g\n"
        for a, b, c in zip(iu.tolist(), ju.tolist(), w.tolist()):
            f.write(fmt % (a, b, c))
        if h is not None:
            for i in np.nonzero(h)[0].tolist():
                f.write("%d %d %.9g\n" % (i, i, h[i]))
