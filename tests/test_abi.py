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
        "peec_set_incidence": lambda: L.peec_set_incidence(None, 0, 0, 0, None, None, 0, None, 1),
        "peec_set_dense": lambda: L.peec_set_dense(None, None, None, None, None),
        "peec_set_dense_rcc": lambda: L.peec_set_dense_rcc(None, None, None, None, None),
        "peec_set_dense_rcc_frequency": lambda: L.peec_set_dense_rcc_frequency(None, 1.0),
        "peec_ris_fill": lambda: L.peec_ris_fill(None, None, None, None, 1.0, None, None, None,
                                                 1.0, 0, None),
        "peec_dense_get": lambda: L.peec_dense_get(None, 0, 0, None),
        "peec_set_device_loop": lambda: L.peec_set_device_loop(None, 1),
        "peec_set_edge_state": lambda: L.peec_set_edge_state(None, None, None, None, None, None,
                                                             0, 1.0, 1.0),
        "peec_set_frequency_device": lambda: L.peec_set_frequency_device(None, 1.0, 0, None,
                                                                         None, None),
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


def test_header_is_plain_c_and_cpp(cuda_lib, tmp_path):
    """include/peec_gb300.h compiles as strict C99 and C++17 with every warning an error,
    and a C program resolves each declared function from the built library by name
    (what a cgo, JNI or ccall binding does) and calls peec_version."""
    import shutil
    import subprocess
    names = declared_symbols()
    src = tmp_path / "use_abi.c"
    lines = ['#include <dlfcn.h>', '#include <stdio.h>', '#include "peec_gb300.h"',
             'int main(int argc, char** argv) {',
             '  void* h = dlopen(argv[1], RTLD_NOW | RTLD_LOCAL);',
             '  if (!h) { fprintf(stderr, "%s\\n", dlerror()); return 2; }']
    for nm in names:
        lines.append(f'  if (!dlsym(h, "{nm}")) {{ fprintf(stderr, "missing {nm}\\n"); return 3; }}')
    lines += ['  int (*ver)(void);',
              '  *(void**)(&ver) = dlsym(h, "peec_version");  /* the POSIX form */',
              '  printf("%d\\n", ver());',
              '  (void)argc; return 0;', '}']
    src.write_text("\n".join(lines) + "\n")
    inc = str(ROOT / "include")
    gcc, gxx = shutil.which("gcc"), shutil.which("g++")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", inc,
                    "-D_DEFAULT_SOURCE", "-o", str(tmp_path / "use_abi"), str(src), "-ldl"],
                   check=True)
    hdr = tmp_path / "hdr.cpp"
    hdr.write_text('#include "peec_gb300.h"\n'
                   'int main() { int (*f)(void) = &peec_version; (void)f; return 0; }\n')
    subprocess.run([gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", inc,
                    "-fsyntax-only", str(hdr)], check=True)
    r = subprocess.run([str(tmp_path / "use_abi"), str(cuda_lib)], capture_output=True,
                       text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert int(r.stdout.strip()) >= 100
