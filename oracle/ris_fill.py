"""ORACLE -- test infrastructure only. Python access to the dense RIS fill of
oracle/fill_ref.c (calcola_Lp.jl / calcola_P.jl restated in C, double and long double),
used by tests/ and by bench.py's cpu_baseline leg as the checker; never by the product."""
import ctypes

import numpy as np

from oracle import build


def dense_fill(volumi, superfici, mx, my, mz, esc_Lp=1.0, esc_P=1.0, ld=False,
               forms=None):
    """The oracle's dense Lp blocks and P (oracle/fill_ref.c, double or long double) with
    their error scales (the prefactors times the sum of |terms|). forms: a dict that
    receives, per block, the number of collapsed dimensions of each pair."""
    L = ctypes.CDLL(str(build.build()))
    sfx = "_ld" if ld else "_d"
    dp = ctypes.POINTER(ctypes.c_double)
    f_lp = getattr(L, "oracle_ris_lp_block" + sfx)
    f_lp.restype = ctypes.c_int64
    ip = ctypes.POINTER(ctypes.c_int)
    f_lp.argtypes = [dp, dp, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_double, dp, dp,
                     ip]
    f_p = getattr(L, "oracle_ris_p" + sfx)
    f_p.restype = ctypes.c_int64
    f_p.argtypes = [dp, dp, ctypes.c_int64, ctypes.c_double, dp, dp, ip]

    def P_(a):
        return a.ctypes.data_as(dp)
    coords = np.ascontiguousarray(volumi["coordinate"], dtype=np.float64)
    S = np.ascontiguousarray(volumi["S"], dtype=np.float64)
    Lp, scale, bad = {}, {}, 0
    off = 0
    for d, (key, k) in enumerate((("Lp_x", mx), ("Lp_y", my), ("Lp_z", mz))):
        out = np.zeros(k * k)
        sc = np.zeros(k * k)
        fm = np.full(k * k, -1, dtype=np.int32)
        if k:
            bad += f_lp(P_(coords), P_(S), off, k, d + 1, esc_Lp, P_(out), P_(sc),
                        fm.ctypes.data_as(ip))
        if forms is not None:
            forms[key] = fm.reshape(k, k, order="F")
        Lp[key] = out.reshape(k, k, order="F")
        scale[key] = sc.reshape(k, k, order="F")
        off += k
    ends = np.ascontiguousarray(superfici["estremi_celle"], dtype=np.float64)
    A = np.ascontiguousarray(superfici["S"], dtype=np.float64)
    ns = A.size
    out = np.zeros(ns * ns)
    sc = np.zeros(ns * ns)
    fm = np.full(ns * ns, -1, dtype=np.int32)
    if ns:
        bad += f_p(P_(ends), P_(A), ns, esc_P, P_(out), P_(sc), fm.ctypes.data_as(ip))
    if forms is not None:
        forms["P"] = fm.reshape(ns, ns, order="F")
    return Lp, {"P": out.reshape(ns, ns, order="F")}, scale, sc.reshape(ns, ns, order="F"), bad
