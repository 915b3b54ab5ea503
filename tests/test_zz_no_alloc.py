"""Allocation-free batched inner products (peec_multidot_noalloc).

Some callers of this library cannot allocate device memory at the point where
they need the GMRES reductions -- their device memory is owned by their own pool
allocator, or they run a loop that must not take the implicit synchronisation of
cudaMalloc/cudaFree. The allocation-free entry point keeps its partial sums in a
fixed device array inside the library instead. These tests check that it returns
the same result as the context-based peec_multidot on two calls in a row (the
second call must not see anything left over from the first), and that it rejects
a column count beyond its fixed scratch. The file is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_K = 256


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def test_noalloc_matches_context_multidot_twice():
    import torch
    from solver_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(None, L.peec_ctx_create(ctypes.byref(h), 0))
    try:
        rng = np.random.default_rng(2024)
        # two calls in a row with different shapes: the second uses fewer columns and
        # fewer reduction blocks than the first left behind in the shared array
        for N, k in ((700_001, 37), (5_000, 9)):
            U = rng.standard_normal((k, N)) + 1j * rng.standard_normal((k, N))
            v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
            dU, dv = _dev(U), _dev(v)
            ref = torch.zeros(k, dtype=torch.complex128, device="cuda")
            got = torch.full((k,), complex("nan"), dtype=torch.complex128, device="cuda")
            _lib.check(h, L.peec_multidot(h, ctypes.c_void_p(dU.data_ptr()), N,
                                          ctypes.c_void_p(dv.data_ptr()), N, k,
                                          ctypes.c_void_p(ref.data_ptr())))
            stream = torch.cuda.current_stream().cuda_stream
            rc = L.peec_multidot_noalloc(ctypes.c_void_p(dU.data_ptr()), N,
                                         ctypes.c_void_p(dv.data_ptr()), N, k,
                                         ctypes.c_void_p(got.data_ptr()), ctypes.c_void_p(stream))
            assert rc == 0, L.peec_last_error(None)
            r, g = ref.cpu().numpy(), got.cpu().numpy()
            # same tolerance as the multi-dot test against numpy
            assert np.max(np.abs(g - r)) <= 1e-12 * max(np.max(np.abs(r)), 1.0) * np.sqrt(N)
            assert np.max(np.abs(g - np.conj(U) @ v)) <= 1e-12 * max(np.max(np.abs(r)), 1.0) * np.sqrt(N)
    finally:
        L.peec_ctx_destroy(h)


def test_noalloc_rejects_too_many_columns():
    import torch
    from solver_gb300 import _lib
    L = _lib.load()
    N, k = 1000, MAX_K + 1
    dU = torch.zeros((k, N), dtype=torch.complex128, device="cuda")
    dv = torch.zeros(N, dtype=torch.complex128, device="cuda")
    out = torch.zeros(k, dtype=torch.complex128, device="cuda")
    rc = L.peec_multidot_noalloc(ctypes.c_void_p(dU.data_ptr()), N, ctypes.c_void_p(dv.data_ptr()),
                                 N, k, ctypes.c_void_p(out.data_ptr()), None)
    assert rc == -5
    assert b"256" in L.peec_last_error(None)


def test_noalloc_concurrent_threads_get_their_own_results():
    """Four host threads, each on its own CUDA stream with its own vectors, call the entry
    point repeatedly at the same time; the per-device lock gives each call the shared
    scratch alone, so every thread's last result equals its own inner products."""
    import threading

    import torch
    from solver_gb300 import _lib
    L = _lib.load()
    rng = np.random.default_rng(7)
    jobs = []
    for t in range(4):
        N, k = 200_003 + 1_000 * t, 8 + 4 * t
        U = rng.standard_normal((k, N)) + 1j * rng.standard_normal((k, N))
        v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        got = torch.full((k,), complex("nan"), dtype=torch.complex128, device="cuda")
        jobs.append((N, k, U, v, _dev(U), _dev(v), got, torch.cuda.Stream()))
    torch.cuda.synchronize()
    errors = []

    def run(j):
        N, k, U, v, dU, dv, got, s = jobs[j]
        for _ in range(10):
            rc = L.peec_multidot_noalloc(ctypes.c_void_p(dU.data_ptr()), N,
                                         ctypes.c_void_p(dv.data_ptr()), N, k,
                                         ctypes.c_void_p(got.data_ptr()),
                                         ctypes.c_void_p(s.cuda_stream))
            if rc != 0:
                errors.append((j, rc, L.peec_last_error(None)))
                return

    threads = [threading.Thread(target=run, args=(j,)) for j in range(len(jobs))]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    torch.cuda.synchronize()
    for N, k, U, v, dU, dv, got, s in jobs:
        ref = np.conj(U) @ v
        g = got.cpu().numpy()
        assert np.max(np.abs(g - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1.0) * np.sqrt(N)
