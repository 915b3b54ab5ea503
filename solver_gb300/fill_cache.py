"""Reuse of the Lp/P generating rows across geometries and runs.

The quasi-static fill (compute_FFT_mutual_coupling_mats.jl:1-33) integrates over the
full voxel lattice, air included (build_centers_Lp_with_air.jl,
build_center_P_Voxels.jl). Its nine generating rows therefore depend only on the grid
extents, the cell sizes, the origin and the two scalings, not on which voxels are
occupied (``peec_fill`` takes nothing else). Geometries that share those values share
the rows: the cache keys on them exactly (the floats by their bit patterns) and, on a
hit, uploads the stored rows instead of filling again.

Entries live in memory (least recently used first out) and, with a directory, as one
``.npz`` per key, so a later run reuses them too. Concurrent misses on one key fill once:
the other threads wait for that fill.
"""
from __future__ import annotations

import hashlib
import os
import struct
import threading
from collections import OrderedDict
from pathlib import Path

import numpy as np

from .operator import ROW_KEYS, row_dims

FORMAT = 1  # bump when the row layout changes; old files are then ignored


def row_key(grid, origin, sx, sy, sz, escal_Lp, escal_P) -> str:
    """Hex digest of the values the rows depend on (exact: floats by their bits)."""
    h = hashlib.sha256()
    h.update(struct.pack("<4q", FORMAT, *(int(v) for v in grid)))
    h.update(struct.pack("<8d", *(float(v) for v in origin), float(sx), float(sy), float(sz),
                         float(escal_Lp), float(escal_P)))
    return h.hexdigest()


class RowCache:
    def __init__(self, directory: str | os.PathLike | None = None, max_entries: int = 8):
        self.dir = Path(directory) if directory is not None else None
        if self.dir is not None:
            self.dir.mkdir(parents=True, exist_ok=True)
        self.max_entries = max(1, int(max_entries))
        self._mem: OrderedDict[str, dict] = OrderedDict()
        self._lock = threading.Lock()
        self._inflight: dict[str, threading.Event] = {}
        self.hits = self.misses = 0

    def _path(self, key):
        return self.dir / f"rows_{key}.npz"

    def _load(self, key, grid):
        if self.dir is None or not self._path(key).exists():
            return None
        with np.load(self._path(key)) as z:
            rows = {k: z[k] for k in z.files}
        dims = row_dims(*grid)
        ok = all(k in rows and rows[k].size == int(np.prod(dims[k]))
                 for k in ROW_KEYS if int(np.prod(dims[k])) > 0)
        return rows if ok else None

    def _store(self, key, rows):
        if self.dir is None:
            return
        tmp = self.dir / f".rows_{key}.{os.getpid()}.{threading.get_ident()}.npz"
        np.savez(tmp, **{k: np.asarray(v) for k, v in rows.items()})
        os.replace(tmp, self._path(key))

    def _remember(self, key, rows):
        self._mem[key] = rows
        self._mem.move_to_end(key)
        while len(self._mem) > self.max_entries:
            self._mem.popitem(last=False)

    def get_or_fill(self, key, grid, fill):
        """The rows of key; fill() -> rows on a miss (called once per key at a time)."""
        while True:
            with self._lock:
                if key in self._mem:
                    self._mem.move_to_end(key)
                    self.hits += 1
                    return self._mem[key], True
                ev = self._inflight.get(key)
                if ev is None:
                    ev = self._inflight[key] = threading.Event()
                    break
            ev.wait()
        try:
            rows = self._load(key, grid)
            hit = rows is not None
            if not hit:
                rows = fill()
                self._store(key, rows)
            with self._lock:
                self._remember(key, rows)
                if hit:
                    self.hits += 1
                else:
                    self.misses += 1
            return rows, hit
        finally:
            with self._lock:
                self._inflight.pop(key).set()


def fill_operator(op, circulant_centers, escalings, cache: RowCache | None = None):
    """The GPU fill of op's rows and spectra, or, with a cache, the stored rows of an
    identical lattice uploaded instead. Returns True when the rows came from the cache."""
    cc, esc = circulant_centers, escalings
    args = (cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"])
    if cache is None:
        op.fill(*args)
        return False
    key = row_key(op.grid, *args)
    rows, hit = cache.get_or_fill(key, op.grid, lambda: op.fill(*args, return_rows=True))
    if hit:
        op.set_rows(rows)
    return hit
