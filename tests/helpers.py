"""In-memory stand-ins for ``lattice.preset`` objects (``load(key)[...]``)."""

import numpy as np


class _Data:
    def __init__(self, arr, name):
        self.arr = arr
        self.file = name
        self.sizeInByte = arr.nbytes
        self.timeInSec = 1e-3

    def __getitem__(self, key):
        return np.asarray(self.arr[key]).copy()


class MemGauge:
    def __init__(self, arr):
        self.data = _Data(arr, "memory-gauge")

    def load(self, key):
        return self.data


class MemEigen:
    def __init__(self, arr, Ne):
        self.Ne = Ne
        self.data = _Data(arr, "memory-eigenvector")

    def load(self, key):
        return self.data


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))
