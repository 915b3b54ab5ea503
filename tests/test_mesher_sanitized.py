"""CPU: the native mesher built with AddressSanitizer and UBSan meshes the reference's
request fixtures and random multi-material grids (several threads) without a report.
Skipped where the compiler has no sanitizer runtime."""
import os
import shutil
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import gzip, json, sys
from pathlib import Path
sys.path.insert(0, sys.argv[1])
import numpy as np
from solver_gb300 import build, configs, mesher
build.LIBDIR = Path(sys.argv[2])          # the sanitized libpeec_mesh.so
G = Path(sys.argv[1]) / "tests" / "golden"
for r in (mesher.load_request(G / "first_run_data.json"),
          mesher.load_request(G / "first_run_data_2_materials.json"),
          json.loads(gzip.open(G / "crossbar.json.gz").read()),
          configs.random_mixed((24, 20, 12), s=5e-5, p=0.35, seed=7, nports=2, freqs=[1e8])):
    mesher.parse_request(r)
rng = np.random.default_rng(5)
for t in range(30):
    shape = tuple(int(v) for v in rng.integers(1, 14, size=3))
    g = np.stack([rng.random(shape) < rng.uniform(0.05, 0.6) for _ in range(int(rng.integers(1, 4)))])
    dom = (rng.random(g.shape[0]) < 0.6).astype(np.uint8)
    mesher._raw_mesh(g, dom, np.where(dom > 0, 5.8e7, 0.0))
maps = open("/proc/self/maps").read()
assert sys.argv[2] in maps, "the sanitized mesher was not the one loaded"
print("clean")
"""


def _runtime(name):
    gcc = shutil.which("gcc")
    if not gcc:
        return None
    p = subprocess.run([gcc, f"-print-file-name={name}"], capture_output=True, text=True)
    path = p.stdout.strip()
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_mesher_under_address_and_ub_sanitizers(tmp_path):
    asan, ubsan = _runtime("libasan.so"), _runtime("libubsan.so")
    gxx = shutil.which("g++")
    if not (asan and ubsan and gxx) or not Path("/proc/self/maps").exists():
        pytest.skip("no g++ sanitizer runtime")
    subprocess.run([gxx, "-O1", "-g", "-std=c++17", "-fPIC", "-fopenmp", "-shared",
                    "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
                    "-fno-sanitize-recover=undefined", "-o", str(tmp_path / "libpeec_mesh.so"),
                    str(ROOT / "solver_gb300" / "csrc" / "mesher.cpp")], check=True)
    env = dict(os.environ, LD_PRELOAD=f"{asan}:{ubsan}", OMP_NUM_THREADS="4",
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=1",
               UBSAN_OPTIONS="print_stacktrace=1:halt_on_error=1")
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT), str(tmp_path)], env=env,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0 and r.stdout.strip().endswith("clean"), r.stderr[-3000:]
