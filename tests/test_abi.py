"""The C ABI library builds, loads without a GPU and exports every declared symbol."""
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "peec_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(peec_[a-z0-9_]+)\s*\(", text)))


def test_header_matches_binding():
    from solver_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.EXPORTS)


def test_library_exports_all_symbols(cuda_lib):
    import ctypes
    L = ctypes.CDLL(str(cuda_lib))
    for name in declared_symbols():
        assert hasattr(L, name), name


def test_version_and_error_without_gpu(cuda_lib):
    from solver_gb300 import _lib
    L = _lib.load(build_if_missing=False)
    assert L.peec_version() >= 100
    # creating a context without a GPU fails loudly with a message, never silently
    import ctypes
    import torch
    if torch.cuda.is_available():
        return
    h = ctypes.c_void_p()
    rc = L.peec_ctx_create(ctypes.byref(h), 0)
    assert rc != 0
    assert L.peec_last_error(None)


def test_entry_points_reject_a_null_context_with_their_own_name(cuda_lib):
    """Every guarded entry point answers a null context with PEEC_ERR_BADARG and a message
    that names the exported function (no GPU is touched before the argument check)."""
    from solver_gb300 import _lib
    L = _lib.load(build_if_missing=False)
    calls = {
        "peec_set_pdiag": lambda: L.peec_set_pdiag(None, None),
        "peec_set_rows": lambda: L.peec_set_rows(None, None),
        "peec_matvec": lambda: L.peec_matvec(None, None, None, 0),
        "peec_matvec_dev": lambda: L.peec_matvec_dev(None, None, None, 0),
        "peec_port_rhs": lambda: L.peec_port_rhs(None, 0, 1, 1.0, None),
        "peec_check_wait_limit": lambda: L.peec_check_wait_limit(None),
        "peec_set_residual_precision": lambda: L.peec_set_residual_precision(None, 0),
        "peec_set_lu_component_max": lambda: L.peec_set_lu_component_max(None, 0),
        "peec_profile_matvec": lambda: L.peec_profile_matvec(None, 0, 1, None),
    }
    for name, call in calls.items():
        assert call() == -5, name
        msg = L.peec_last_error(None).decode()
        assert msg.startswith(name + ":"), (name, msg)
    assert L.peec_ctx_create(None, 0) == -5
    assert L.peec_last_error(None).decode().startswith("peec_ctx_create:")
