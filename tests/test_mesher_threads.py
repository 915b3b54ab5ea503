"""CPU: the native mesher's output does not depend on its thread count. Its loops run
in parallel (OpenMP), and every numbered sequence (edges, surfaces, nodes) is assembled in
the reference's loop order, so one thread and several threads give the same arrays."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent

SCRIPT = r"""
import hashlib, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from solver_gb300 import configs, mesher
rng = np.random.default_rng(11)
shape = (37, 29, 13)
grids = np.stack([rng.random(shape) < 0.25, rng.random(shape) < 0.2, rng.random(shape) < 0.15])
out = mesher._raw_mesh(grids, [1, 0, 1], [5.8e7, 0.0, 1e7])
h = hashlib.sha256()
for k in sorted(out):
    h.update(k.encode())
    h.update(np.ascontiguousarray(out[k]).tobytes())
print(json.dumps({"hash": h.hexdigest(), "m": int(out["counts"][2] + out["counts"][3] + out["counts"][4])}))
"""


def _run(threads):
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([sys.executable, "-c", SCRIPT, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=300, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_mesher_output_independent_of_thread_count():
    one, four = _run(1), _run(4)
    assert one["m"] > 0
    assert one == four


def test_mesher_rejects_a_mask_of_the_wrong_length():
    import numpy as np
    import pytest
    sys.path.insert(0, str(ROOT))
    from solver_gb300 import mesher
    grids = np.ones((3, 4, 4, 2), dtype=bool)
    with pytest.raises(ValueError):
        mesher._raw_mesh(grids, [0, 2], [5.8e7, 0.0, 1e7])
