"""CPU: reuse of the generating rows between geometries on the same lattice
(solver_gb300/fill_cache.py), through a stand-in for libpeec_gb300.so whose fill writes
rows that depend on the lattice values and whose set_rows records what it received.

* Two geometries with different occupancy on one lattice fill once; the second context
  gets the first fill's rows through set_rows.
* A different cell size, origin or scaling is another key.
* A directory makes the rows outlive the cache object (a later run loads them).
* Concurrent misses on one key fill once; the cache keeps at most max_entries in memory."""
import ctypes
import threading
import time

import numpy as np
import pytest

from solver_gb300 import _lib, api, configs, fill_cache, mesher
from solver_gb300 import operator as gop


class FillFake:
    def __init__(self):
        self.fills = 0
        self.uploads = []
        self.grid = None

    def peec_last_error(self, ctx):
        return b"stand-in"

    def peec_set_topology(self, h, Nx, Ny, Nz, *rest):
        self.grid = (Nx, Ny, Nz)
        return 0

    def peec_fill(self, h, origin, sx, sy, sz, eLp, eP, arr):
        self.fills += 1
        dims = gop.row_dims(*self.grid)
        for i, k in enumerate(gop.ROW_KEYS):
            n = int(np.prod(dims[k]))
            if n and arr[i]:
                vals = np.arange(n, dtype=np.float64) * sx + i * eLp + eP
                ctypes.memmove(arr[i], vals.ctypes.data, vals.nbytes)
        return 0

    def peec_set_rows(self, h, arr):
        dims = gop.row_dims(*self.grid)
        got = {}
        for i, k in enumerate(gop.ROW_KEYS):
            n = int(np.prod(dims[k]))
            if n and arr[i]:
                got[k] = np.ctypeslib.as_array(ctypes.cast(arr[i], ctypes.POINTER(ctypes.c_double)),
                                               shape=(n,)).copy()
        self.uploads.append(got)
        return 0

    def __getattr__(self, name):
        if not name.startswith("peec_"):
            raise AttributeError(name)
        return lambda *a: 0


@pytest.fixture
def fake(monkeypatch):
    L = FillFake()
    monkeypatch.setattr(_lib, "load", lambda *a, **k: L)
    return L


def _geometry(seed, s=5e-5):
    out, freqs, settings, z0, grid = mesher.parse_request(
        configs.random_copper((10, 8, 6), s=s, p=0.4, seed=seed))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    return gop.GpuOperator(inc, exp, diag["P"]), cc, esc


def test_same_lattice_fills_once(fake, tmp_path):
    cache = fill_cache.RowCache()
    op1, cc1, esc1 = _geometry(1)
    op2, cc2, esc2 = _geometry(2)          # other occupancy, same lattice
    assert op1.m != op2.m                  # genuinely different geometries
    assert fill_cache.fill_operator(op1, cc1, esc1, cache) is False
    assert fill_cache.fill_operator(op2, cc2, esc2, cache) is True
    assert fake.fills == 1 and len(fake.uploads) == 1
    for k, v in op1._rows.items():
        assert np.array_equal(fake.uploads[0][k], v)
    op3, cc3, esc3 = _geometry(3, s=6e-5)  # another cell size: another key
    assert fill_cache.fill_operator(op3, cc3, esc3, cache) is False
    assert fake.fills == 2
    key = fill_cache.row_key(op1.grid, cc1["origin"], cc1["sx"], cc1["sy"], cc1["sz"],
                             esc1["Lp"], esc1["P"])
    shifted = fill_cache.row_key(op1.grid, np.asarray(cc1["origin"]) + 1e-9, cc1["sx"],
                                 cc1["sy"], cc1["sz"], esc1["Lp"], esc1["P"])
    rescaled = fill_cache.row_key(op1.grid, cc1["origin"], cc1["sx"], cc1["sy"], cc1["sz"],
                                  esc1["Lp"], 2 * esc1["P"])
    assert len({key, shifted, rescaled}) == 3
    # without a cache every geometry fills
    fill_cache.fill_operator(op2, cc2, esc2, None)
    assert fake.fills == 3


def test_rows_persist_in_a_directory(fake, tmp_path):
    op1, cc1, esc1 = _geometry(1)
    assert fill_cache.fill_operator(op1, cc1, esc1, fill_cache.RowCache(tmp_path)) is False
    assert len(list(tmp_path.glob("rows_*.npz"))) == 1
    later = fill_cache.RowCache(tmp_path)  # a new run
    op2, cc2, esc2 = _geometry(2)
    assert fill_cache.fill_operator(op2, cc2, esc2, later) is True
    assert fake.fills == 1
    for k, v in op1._rows.items():
        assert np.array_equal(fake.uploads[-1][k], v)


def test_concurrent_misses_fill_once_and_memory_is_bounded():
    cache = fill_cache.RowCache(max_entries=2)
    calls = []
    lock = threading.Lock()

    def fill():
        with lock:
            calls.append(1)
        time.sleep(0.2)
        return {"Lpx": np.ones(3)}

    out = []
    ts = [threading.Thread(target=lambda: out.append(cache.get_or_fill("k", (2, 2, 2), fill)))
          for _ in range(6)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    assert len(calls) == 1 and len(out) == 6
    assert sum(hit for _, hit in out) == 5
    for key in ("a", "b", "c"):
        cache.get_or_fill(key, (2, 2, 2), lambda: {"Lpx": np.zeros(1)})
    assert list(cache._mem) == ["b", "c"]


def test_api_entry_points_take_a_cache():
    import inspect
    assert "row_cache" in inspect.signature(api.sweep_many).parameters
    assert "row_cache" in inspect.signature(api.do_solving_fft).parameters
