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
