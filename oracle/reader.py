"""Restatement of the reference's graph reader — TEST INFRASTRUCTURE ONLY.

SB/CUDA_GPU/m2_opt.cu:111-123: fscanf("%d") reads N (and the program ignores it in favour of
its compile-time N), then "%d%d%d" triples (a, b, w) are stored symmetrically into a dense float
matrix until feof(); a later triple for the same pair overwrites an earlier one. The reference
asserts a != b (no field lines).
"""
from __future__ import annotations

import numpy as np


def read_reference_format(path: str, n: int | None = None):
    toks = open(path).read().split()
    header = int(toks[0])
    n = header if n is None else n
    J = np.zeros((n, n), np.float32)
    vals = toks[1:]
    for k in range(0, len(vals) - len(vals) % 3, 3):
        a, b, w = int(vals[k]), int(vals[k + 1]), int(vals[k + 2])
        assert a != b
        J[a, b] = w
        J[b, a] = w
    return header, J
