"""mdcraft.data.Atoms (python/mdcraft/data/_data.cxx): a resizable array of
208-byte Atom records (mdcraft/data/atom.h:21-40) exposed as `data`."""
from __future__ import annotations

import numpy as np

_V3 = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8")])
_M3 = np.dtype([(k, "<f8") for k in ("xx", "xy", "xz", "yx", "yy", "yz", "zx", "zy", "zz")])
ATOM = np.dtype({"names": ["r", "v", "f", "V", "m", "rcut", "rns", "Ep", "Em", "nc", "bc", "kind", "uid", "tag"],
                 "formats": [_V3, _V3, _V3, _M3, "<f8", "<f8", "<f8", "<f8", "<f8", "<f8", "<u2", "<u2", "<u4",
                             "<u2"],
                 "offsets": [0, 24, 48, 72, 144, 152, 160, 168, 176, 184, 192, 194, 196, 200],
                 "itemsize": 208})


def _new(n):
    a = np.zeros(n, dtype=ATOM)
    a["tag"] = 0xFFFF  # the reference's default tag
    return a


class Atoms:
    def __init__(self, size: int = 0):
        self._data = _new(size)
        self._device = None

    @property
    def data(self) -> np.ndarray:
        return self._data

    def resize(self, size: int):
        old = self._data
        self._data = _new(size)
        k = min(size, len(old))
        self._data[:k] = old[:k]

    def __len__(self):
        return len(self._data)

    def erase(self, *args):
        if len(args) == 2:
            idx = np.arange(args[0], args[1])
        else:
            idx = np.asarray(args[0], dtype=np.int64)
        keep = np.ones(len(self._data), dtype=bool)
        keep[idx] = False
        self._data = self._data[keep].copy()

    def join(self, other: "Atoms"):
        self._data = np.concatenate([self._data, other._data])
