"""GPU Krylov building blocks through the C ABI (device buffers from torch)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _ctx():
    from solver_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    _lib.check(None, L.peec_ctx_create(ctypes.byref(h), 0))
    return L, h


@pytest.mark.parametrize("N,k", [(1, 1), (1000, 3), (300_001, 17), (2_000_000, 40)])
def test_multidot_matches_numpy(N, k):
    import torch
    from solver_gb300 import _lib
    L, h = _ctx()
    rng = np.random.default_rng(N + k)
    U = rng.standard_normal((k, N)) + 1j * rng.standard_normal((k, N))
    v = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    dU = torch.from_numpy(U).cuda()
    dv = torch.from_numpy(v).cuda()
    out = torch.zeros(k, dtype=torch.complex128, device="cuda")
    _lib.check(h, L.peec_multidot(h, ctypes.c_void_p(dU.data_ptr()), N,
                                  ctypes.c_void_p(dv.data_ptr()), N, k,
                                  ctypes.c_void_p(out.data_ptr())))
    ref = np.conj(U) @ v
    got = out.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * max(np.max(np.abs(ref)), 1.0) * np.sqrt(N)
    L.peec_ctx_destroy(h)
