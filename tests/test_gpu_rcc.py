"""GPU parity of the retarded (Rcc, QS_Rcc_FW == 2) operator against the oracle's
restatement (oracle/rcc_ref.py).

* The GPU fill of the Rcc rows' quasi-static parts against the oracle's rows: on cubic
  cells the Lp rows equal the GPU's own QS rows bit for bit, and every row is within the
  rounding of its closed forms of the oracle's; an elongated-cell lattice takes the Rcc
  dispatch's own collinear-line formula.
* Shared rows (the oracle's uploaded) and shared LU factors, as in test_gpu_parity.py: the
  Rcc operator at several frequencies within max(1e-10, 20x the problem's rounding
  noise), FP32 within 2e-5; on geometries where the reference's Rcc solve converges, the
  FP64 sweep with the same flags and iteration counts and port impedances within 1e-10,
  and the mixed sweep within 1e-6 of the oracle's FP64 sweep.
* A reference request end to end with solverType 2 (mesher, GPU Rcc fill, sweep) against
  the oracle's own pipeline at the fixture's tolerance."""
import copy

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from oracle import rcc_ref as RR
from solver_gb300 import api, configs, mesher
from solver_gb300.operator import GpuOperator, ROW_KEYS

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def _case(req):
    out, freqs, settings, z0, grid = OM.parse_request(copy.deepcopy(req))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    pe = mesher.parse_request(copy.deepcopy(req))[0]
    prod = dict(esc=pe[0], inc=pe[1], cc=pe[2], diag=pe[3], exp=pe[4], ports=pe[5], le=pe[6],
                Zs=pe[8])
    rL, rP = RR.compute_rows_Rcc_Lp(cc), RR.compute_rows_Rcc_P(cc)
    return dict(esc=esc, inc=inc, cc=cc, diag=diag, exp=exp, ports=ports, le=le, Zs=Zs,
                rL=rL, rP=rP, freqs=freqs, settings=settings, z0=z0, grid=grid, prod=prod)


def _elongated():
    """a bar of 1 mm x 10 um x 13 um cells, 40 long: far along x the cells collapse to
    collinear lines in the Lp integrals"""
    g = np.zeros((40, 3, 3), dtype=bool)
    g[:, 1, 1] = 1
    g[:, 0, 1] = 1
    cell = (1e-3, 1e-5, 1.3e-5)
    ports = [((0, 1, 1), (39, 1, 1))]
    return configs.make_request({"copper": g}, [configs.COPPER], cell, ports, [1e9], 1e-8)


CASES = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_24x20x12": lambda: configs.random_mixed((24, 20, 12), s=5e-5, p=0.35, seed=7,
                                                    nports=2, freqs=[1e8, 3e9], tol=1e-8),
    "first_run_data_2_materials_1GHz": lambda: _at(
        mesher.load_request(GOLDEN / "first_run_data_2_materials.json"), [1e9, 3e9]),
}


def _at(req, freqs):
    req["solverInput"]["frequencies"] = list(freqs)
    return req


# the sweeps run where the reference's Rcc operator converges: on the mixed copper /
# dielectric grid its P rows, filled with the block indices as face types, leave GMRES at a
# relative residual near 1e-2 after 100 iterations (the oracle as the GPU;
# tests/test_oracle_rcc.py::test_reference_rcc_does_not_converge_on_mixed_grids)
SWEEP_CASES = ("crossbar_20x20x4", "first_run_data_2_materials_1GHz")


def _gpu_case(name):
    c = _case(CASES[name]())
    p = c["prod"]
    op = GpuOperator(p["inc"], p["exp"], p["diag"]["P"])
    cc = c["cc"]
    op.set_rows_rcc(RR.rcc_rows_escaled(c["rL"], c["rP"], c["esc"]), cc["origin"], cc["sx"],
                    cc["sy"], cc["sz"])
    c["op"] = op
    c["name"] = name
    return c


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    c = _gpu_case(request.param)
    yield c
    c["op"].close()


@pytest.fixture(scope="module", params=SWEEP_CASES)
def sweep_case(request):
    c = _gpu_case(request.param)
    yield c
    c["op"].close()


def _freq(c, f_hz):
    w = 2 * np.pi * f_hz * c["esc"]["freq"]
    fs = O.frequency_setup(w, c["esc"], c["inc"], c["diag"], c["Zs"], c["le"], c["ports"], c["z0"])
    c["op"].set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
    c["op"].set_rcc_frequency(f_hz)
    FL = RR.compute_Circulant_Lp_Rcc(c["rL"], c["esc"], f_hz, *c["grid"])
    FP = RR.compute_Circulant_P_sup_Rcc(c["rP"], c["esc"], f_hz, *c["grid"])
    return w, fs, FL, FP


def _oracle_mv(c, w, fs, FL, FP, single=False):
    def mv(x):
        saved = O.precond_3_3_vector
        if single:
            def one(F, invZ, invP, A_, G_, w_, X1, X2, X3):
                Mv = F(A_.T @ (invZ @ X1) - 1j * w_ * (G_ @ (invP @ X2)) + X3)
                return np.concatenate([invZ @ (X1 - A_ @ Mv), invP @ (X2 + G_.T @ Mv), Mv])
            O.precond_3_3_vector = one
        try:
            return O.ComputeMatrixVectorFTT(x, w, c["inc"], FP, FL, fs["DZ"], fs["Yle"],
                                            c["exp"], fs["invZ"], fs["invP"], fs["F"])
        finally:
            O.precond_3_3_vector = saved
    return mv


def _fill_case(req):
    c = _case(req)
    p = c["prod"]
    op = GpuOperator(p["inc"], p["exp"], p["diag"]["P"])
    cc = c["cc"]
    try:
        got = op.fill_rcc(cc["origin"], cc["sx"], cc["sy"], cc["sz"], c["esc"]["Lp"],
                          c["esc"]["P"])
        qs = op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], c["esc"]["Lp"], c["esc"]["P"],
                     return_rows=True)
    finally:
        op.close()
    return c, got, qs


@pytest.mark.parametrize("name", ["crossbar_20x20x4", "elongated_40x3x3"])
def test_rcc_fill_matches_oracle(name):
    req = configs.crossbar_20x20x4() if name == "crossbar_20x20x4" else _elongated()
    c, got, qs = _fill_case(req)
    want = RR.rcc_rows_escaled(c["rL"], c["rP"], c["esc"])
    scale = RR.rcc_row_scales(c["cc"], c["esc"])
    eps = np.finfo(float).eps
    for k in ROW_KEYS:
        if k not in want or want[k].size == 0:
            continue
        g, w = got[k], want[k]
        # the same closed forms in FP64 without contraction on both sides: within the
        # rounding of the terms each entry sums (as the QS fill, test_gpu_fill_far.py)
        assert np.all(np.isfinite(g)), k
        err = np.abs(g - w)
        bound = 64 * eps * scale[k] + 1e-300
        assert np.all(err <= bound), (k, float(np.max(err / bound)))
    if name == "crossbar_20x20x4":
        # cubic cells: the Rcc Lp dispatch takes the QS fill's formulas everywhere
        for k in ("Lpx", "Lpy", "Lpz", "p12_se"):
            assert np.array_equal(got[k], qs[k]), k
    else:
        # the collinear-line entries differ from the QS rows, as in the oracle
        dq = np.nonzero(got["Lpx"] != qs["Lpx"])[0]
        assert dq.size > 0
        o = O.lp_row(1, np.asarray(c["cc"]["Lpx"]), c["cc"]["sx"], c["cc"]["sy"], c["cc"]["sz"])
        o[0] = 0
        assert np.array_equal(dq, np.nonzero(c["rL"]["Lpx"][0] != o)[0])


def test_rcc_matvec(case):
    rng = np.random.default_rng(11)
    N = case["op"].N
    for f in (1e8, 1e9, 5e9):
        w, fs, FL, FP = _freq(case, f)
        x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
        y_ref = _oracle_mv(case, w, fs, FL, FP)(x)
        noise = _rel(_oracle_mv(case, w, fs, FL, FP, single=True)(x), y_ref)
        e64 = _rel(case["op"].matvec(x, 0), y_ref)
        assert e64 < max(1e-10, 20 * noise), (case["name"], f, e64, noise)
        assert _rel(case["op"].matvec(x, 2), y_ref) < max(1e-10, 20 * noise), (case["name"], f)
        assert _rel(case["op"].matvec(x, 1), y_ref) < 2e-5, (case["name"], f)


def test_rcc_sweep(sweep_case):
    c = sweep_case
    freqs = np.array([1e8, 1e9, 3e9])
    st = {"Inner_Iter": c["settings"]["Inner_Iter"], "tol": np.full(freqs.size, 1e-8)}
    ref = RR.FFT_solver_Rcc(freqs, c["esc"], c["inc"], c["rP"], c["rL"], c["diag"], c["ports"],
                            c["z0"], c["le"], c["exp"], st, c["Zs"], c["grid"])
    p = c["prod"]
    p["exp"]["gpu_ctx"] = c["op"]
    h = api.RccRows(c["op"])
    try:
        got = api.FFT_solver_QS_S_type(freqs, p["esc"], p["inc"], h, h, p["diag"], p["ports"],
                                       c["z0"], p["le"], p["exp"], st, p["Zs"], QS_Rcc_FW=2)
        assert [r["niter"] for r in got["info"]] == [len(r["resvec"]) - 1 for r in ref["info"]]
        assert [r["flag"] for r in got["info"]] == [r["flag"] for r in ref["info"]]
        assert _rel(got["Z"], ref["Z"]) < 1e-10
        # mixed precision (2 lanes where there are two ports) against the FP64 oracle
        st10 = {"Inner_Iter": c["settings"]["Inner_Iter"], "tol": np.full(freqs.size, 1e-10)}
        ref10 = RR.FFT_solver_Rcc(freqs, c["esc"], c["inc"], c["rP"], c["rL"], c["diag"],
                                  c["ports"], c["z0"], c["le"], c["exp"], st10, c["Zs"], c["grid"])
        npt = len(np.asarray(c["ports"]["port_nodes"]).reshape(-1, 2))
        mx = api.FFT_solver_QS_S_type(freqs, p["esc"], p["inc"], h, h, p["diag"], p["ports"],
                                      c["z0"], p["le"], p["exp"], st10, p["Zs"], QS_Rcc_FW=2,
                                      mode="mixed", lanes=min(2, npt))
        assert all(r["flag"] == 0 for r in mx["info"])
        assert _rel(mx["Z"], ref10["Z"]) < 1e-6
    finally:
        p["exp"].pop("gpu_ctx", None)


def test_rcc_request_end_to_end():
    """solverType 2 through api.do_solving_fft (product mesher, GPU Rcc fill, sweep)
    against the oracle's pipeline (its mesher, its Rcc rows, its sweep)."""
    req = _at(mesher.load_request(GOLDEN / "first_run_data.json"), [1e9, 3e9])
    req["solverType"] = 2
    c = _case(req)
    st = {"Inner_Iter": c["settings"]["Inner_Iter"],
          "tol": np.full(len(c["freqs"]), c["settings"]["tol"])}
    ref = RR.FFT_solver_Rcc(c["freqs"], c["esc"], c["inc"], c["rP"], c["rL"], c["diag"],
                            c["ports"], c["z0"], c["le"], c["exp"], st, c["Zs"], c["grid"])
    got = api.do_solving_fft(copy.deepcopy(req), mode="fp64")
    assert [r["niter"] for r in got["info"]] == [len(r["resvec"]) - 1 for r in ref["info"]]
    assert _rel(got["Z"], ref["Z"]) < 1e-8
    # and it is not the quasi-static answer
    req["solverType"] = 1
    qs = api.do_solving_fft(copy.deepcopy(req), mode="fp64")
    assert _rel(qs["Z"], ref["Z"]) > 1e-6
