"""CPU: the bench's reference arm (the oracle port timed on the host cores) prints one
JSON line with the keys the benchmark contract asks of it, and ranks other than 0 of a
multi-rank launch exit without work or output."""
import json
import os

import pytest
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _bench(*args, env=None):
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], cwd=ROOT,
                          env=dict(os.environ, **(env or {})), capture_output=True, text=True,
                          timeout=900)


def test_reference_arm_line():
    """A small grid keeps the CPU suite short; the arm's code path is the one the
    default 128x128x64 run takes."""
    r = _bench("--impl", "reference", "--steps", "2", "--warmup", "1", "--grid", "10", "10", "6")
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1
    # complete port solves were timed, nothing extrapolated, and the reference arm built
    # its inputs without the product's native mesher
    solves = d["timed"]["solves"]
    assert len(solves) == 2 and all(s["iters"] >= 1 for s in solves)
    assert d["ms_per_step"] == pytest.approx(d["timed"]["elapsed_s"] * 1e3 / 2)
    assert not any("libpeec" in so for so in (d["native_so_loaded"] or []))
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"] and cb["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _bench("--impl", "reference", "--steps", "1", "--warmup", "0", "--grid", "10", "10", "6",
               env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
