"""Regenerates the committed fixtures under tests/golden/.

* ``first_run_data.json`` / ``first_run_data_2_materials.json`` / ``crossbar.json.gz``:
  the reference's own FFT-solver request bodies (inputs only; the reference ships no
  outputs for this path), copied verbatim (the crossbar gzip-compressed) from the
  reference checkout given as argv[1].
* ``oracle_*.npz``: outputs of the CPU oracle (topology from oracle/mesher_ref.py, fill,
  operator and sweep from oracle/peec_oracle.py) on those inputs (the two-material one at
  1 GHz and 3 GHz) and on the 20x20x4 crossbar configuration, kept as regression pins of
  the oracle itself (rows, one matvec on a seeded vector, the port solution and Z).

Usage: python tests/golden/make_fixtures.py /path/to/reference
"""
import json
import shutil
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import mesher_ref as OM  # noqa: E402
from oracle import peec_oracle as O  # noqa: E402
from solver_gb300 import configs  # noqa: E402


def oracle_case(req, tag):
    out, freqs, settings, z0, (Nx, Ny, Nz) = OM.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    rows = O.fill_rows(cc, esc, Nx, Ny, Nz)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, Nx, Ny, Nz)
    st = {"Inner_Iter": settings["Inner_Iter"], "tol": np.full(len(freqs), settings["tol"])}
    res = O.FFT_solver_QS_S_type(freqs, esc, inc, FFTCP, FFTCLp, diag, ports, z0, le, exp, st, Zs)
    fs = O.frequency_setup(2 * np.pi * freqs[0] * esc["freq"], esc, inc, diag, Zs, le, ports, z0)
    N = inc["A"].shape[0] + inc["Gamma"].shape[1] + inc["A"].shape[1]
    rng = np.random.default_rng(1234)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y = O.ComputeMatrixVectorFTT(x, 2 * np.pi * freqs[0] * esc["freq"], inc, FFTCP, FFTCLp,
                                 fs["DZ"], fs["Yle"], exp, fs["invZ"], fs["invP"], fs["F"])
    np.savez_compressed(HERE / f"oracle_{tag}.npz", x=x, y=y, Z=res["Z"], S=res["S"],
                        V=res["Vrest"], **{f"row_{k}": v for k, v in rows.items()})


def main():
    ref = Path(sys.argv[1])
    for name in ("first_run_data.json", "first_run_data_2_materials.json"):
        shutil.copyfile(ref / name, HERE / name)
    # the 57x57x13 crossbar request (2 ports, 7 lumped elements, thin cells whose rows
    # reach the far-field fill branches), gzip-compressed: its voxel grid is 1.4 MB of JSON
    # (no name and mtime 0 in the gzip header, so regenerating gives the same bytes)
    import gzip
    with open(ref / "crossbar.json", "rb") as src, open(HERE / "crossbar.json.gz", "wb") as raw, \
            gzip.GzipFile(filename="", mode="wb", fileobj=raw, mtime=0) as dst:
        shutil.copyfileobj(src, dst)
    oracle_case(json.loads((HERE / "first_run_data.json").read_text()), "first_run_data")
    # the two-material fixture at 1 GHz and 3 GHz: its face rows reach the far-field
    # (suppressed) branches of the P integrals
    req2 = json.loads((HERE / "first_run_data_2_materials.json").read_text())
    req2["solverInput"]["frequencies"] = [1e9, 3e9]
    oracle_case(req2, "first_run_data_2_materials")
    oracle_case(configs.crossbar_20x20x4(), "crossbar_20x20x4")


if __name__ == "__main__":
    main()
