"""ORACLE build recipe (test infrastructure only): compiles ``fill_ref.c`` as a double
and a long double restatement into ``oracle/_build/liboracle_fill.so``.

No FMA contraction and no fast-math, so the double build rounds as the reference's
scalar Julia code does up to libm differences.
"""
from __future__ import annotations

import hashlib
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT_DIR = HERE / "_build"
LIB = OUT_DIR / "liboracle_fill.so"


def build(force: bool = False) -> Path:
    OUT_DIR.mkdir(exist_ok=True)
    src = HERE / "fill_ref.c"
    dig = hashlib.sha256(src.read_bytes()).hexdigest()
    stamp = OUT_DIR / ".stamp"
    if LIB.exists() and stamp.exists() and stamp.read_text() == dig and not force:
        return LIB
    cc = shutil.which("gcc") or "gcc"
    common = ["-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-std=c11"]
    objs = []
    for sfx, defs in (("d", ["-DREAL=double", "-DSFX=_d"]),
                      ("ld", ["-DREAL=long double", "-DSFX=_ld", "-DLONGD"])):
        obj = OUT_DIR / f"fill_{sfx}.o"
        subprocess.run([cc] + common + defs + ["-c", str(src), "-o", str(obj)], check=True)
        objs.append(str(obj))
    subprocess.run([cc, "-shared", "-fopenmp", "-o", str(LIB)] + objs + ["-lm"], check=True)
    stamp.write_text(dig)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
