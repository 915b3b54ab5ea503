"""GPU: the dense RIS solver (solver_gb300/ris.py, peec_set_incidence, peec_set_dense)
against the RIS oracle (oracle/ris_ref.py), on dense problems written out from voxel
cases (tests/ris_cases.py):

* the dense operator (FP64, FP32 copy, float-float requests take FP64) against
  ComputeMatrixVectorRis, and against the voxel path's circulant operator on the GPU for
  the same problem;
* GMRES on it: the oracle's flag and iteration counts, x within 1e-10;
* the RIS frequency x port loop (FP64 and mixed, host and device factorisation of SS)
  against the oracle's S parameters;
* a context without voxel lattices refuses the circulant entry points."""
import numpy as np
import pytest

from oracle import peec_oracle as O
from oracle import ris_ref as RO
from solver_gb300 import _lib, configs
from tests import ris_cases

pytestmark = pytest.mark.gpu

CASES = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_16x12x8": lambda: configs.random_mixed((16, 12, 8), s=5e-5, p=0.35, seed=9,
                                                   nports=2, freqs=[1e8, 3e9], tol=1e-8),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    from solver_gb300.ris import DenseOperator
    c = ris_cases.voxel_case(CASES[request.param]())
    c["Lp_data"], c["P_data"] = ris_cases.dense_blocks(c)
    c["volumi"] = ris_cases.volumi_of(c, seed=1)
    c["op"] = DenseOperator(c["inc"], c["Lp_data"], c["P_data"])
    c["name"] = request.param
    yield c
    c["op"].close()


def _ris_state(c, f, use_zs=True):
    w = 2 * np.pi * f * c["esc"]["freq"]
    st = RO.frequency_setup(w, c["esc"], c["inc"], c["P_data"], c["Lp_data"], c["ports"], {},
                            c["volumi"], use_zs, 50.0)
    return w, st


def _ris_mv(c, w, st):
    return lambda x: RO.ComputeMatrixVectorRis(x, w, c["inc"], st["P"], st["Lp"], st["Z_self"],
                                               st["Yle"], st["invZ"], st["invP"], st["F"])


def _noise(c, w, st, x):
    """Rounding noise of the oracle's operator at this frequency: its preconditioner's
    three LU solves taken as one (what the library does), relative to max |y| (about 4e-11
    at 100 MHz on the crossbar, where SS is least well conditioned)."""
    A, G = c["inc"]["A"], c["inc"]["Gamma"]
    saved = RO.precond_3_3_vector

    def one(F, invZ, invP, A_, G_, w_, X1, X2, X3):
        M = F(A_.T @ (invZ @ X1) - 1j * w_ * (G_ @ (invP @ X2)) + X3)
        return np.concatenate([invZ @ (X1 - A_ @ M), invP @ (X2 + G_.T @ M), M])
    RO.precond_3_3_vector = one
    try:
        y1 = _ris_mv(c, w, st)(x)
    finally:
        RO.precond_3_3_vector = saved
    return _rel(y1, _ris_mv(c, w, st)(x))


def _install(c, w, st):
    DZ = st["Z_self"] + 1j * w * st["diag_Lp"]
    c["op"].set_frequency(w, DZ, st["Yle"], st["lu"])


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("f", [1e8, 2e9])
def test_dense_operator_matches_the_oracle(case, f):
    w, st = _ris_state(case, f)
    _install(case, w, st)
    rng = np.random.default_rng(4)
    x = rng.standard_normal(case["op"].N) + 1j * rng.standard_normal(case["op"].N)
    y_ref = _ris_mv(case, w, st)(x)
    y64 = case["op"].matvec(x, _lib.PREC_FP64)
    tol = max(1e-11, 4 * _noise(case, w, st, x))
    assert _rel(y64, y_ref) < tol, (case["name"], f, _rel(y64, y_ref), tol)
    assert np.array_equal(case["op"].matvec(x, _lib.PREC_FF), y64)  # FF requests take FP64
    y32 = case["op"].matvec(x, _lib.PREC_FP32)
    assert _rel(y32, y_ref) < 2e-5, (case["name"], f, _rel(y32, y_ref))


def test_dense_operator_equals_the_circulant_operator(case):
    """The dense blocks are the circulant ones written out: with Z_self = DZ - jw diag(Lp)
    the RIS operator is the voxel operator, so the GPU's dense and circulant products
    agree (different arithmetic: dense sums against FFTs)."""
    from solver_gb300.operator import GpuOperator
    c = case
    import copy as _copy
    from solver_gb300 import mesher
    req = CASES[c["name"]]()
    pe = mesher.parse_request(_copy.deepcopy(req))[0]
    vox = GpuOperator(pe[1], pe[4], pe[3]["P"])
    try:
        vox.set_rows(c["rows"])
        w = 2 * np.pi * 1e9 * c["esc"]["freq"]
        fs = O.frequency_setup(w, c["esc"], c["inc"], c["diag"], c["Zs"], c["le"], c["ports"],
                               c["z0"])
        vox.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
        c["op"].set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
        rng = np.random.default_rng(8)
        x = rng.standard_normal(vox.N) + 1j * rng.standard_normal(vox.N)
        a, b = c["op"].matvec(x, 0), vox.matvec(x, 0)
        assert _rel(a, b) < 1e-9, _rel(a, b)
    finally:
        vox.close()


def test_gmres_parity(case):
    w, st = _ris_state(case, 1e9)
    _install(case, w, st)
    pn = np.asarray(case["ports"]["port_nodes"]).reshape(-1, 2)
    tn = case["op"].port_rhs(pn[0, 0], pn[0, 1], case["esc"]["Is"])
    isv = np.zeros(case["op"].n)
    isv[pn[0, 0]], isv[pn[0, 1]] = case["esc"]["Is"], -case["esc"]["Is"]
    tn_ref = RO.precond_3_3_Kt_S(st["F"], st["invZ"], st["invP"], case["inc"]["A"],
                                 case["inc"]["Gamma"], case["op"].m, case["op"].ns, isv)
    assert _rel(tn, tn_ref) < 1e-10  # device triangular solves against SuperLU's
    x_ref, f_ref, rr_ref, it_ref, _ = O.gmres_custom(tn_ref, False, 1e-8, 200, None,
                                                     _ris_mv(case, w, st))
    x, f, rr, it, _ = case["op"].gmres(tn, None, 1e-8, 200)
    assert f == f_ref and list(it) == list(it_ref), (f, f_ref, it, it_ref)
    assert _rel(x, x_ref) < 1e-10, _rel(x, x_ref)


@pytest.mark.parametrize("mode,lu", [("fp64", "host"), ("fp64", "device"), ("mixed", "device")])
def test_ris_solver_matches_the_oracle(case, mode, lu):
    from solver_gb300 import ris
    c = case
    freqs = [1e8, 1e9, 3e9]
    gs = {"Inner_Iter": 200, "tol": [1e-8] * len(freqs)}
    ref = RO.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], c["P_data"], c["Lp_data"],
                                   c["ports"], {}, gs, c["volumi"], True, 1, 50.0)
    out = ris.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], c["P_data"], c["Lp_data"],
                                    c["ports"], {}, gs, c["volumi"], True, 1, 50.0, mode=mode,
                                    op=c["op"], lu=lu)
    assert all(r["flag"] == 0 for r in out["info"]), out["info"]
    tol = 1e-7 if mode == "fp64" else 1e-6
    for k in range(len(freqs)):
        assert _rel(out["S"][:, :, k], ref["S"][:, :, k]) < tol, (mode, lu, k)
    if mode == "fp64" and lu == "host":
        assert [r["iter"] for r in out["info"]] == [r["iter"] for r in ref["info"]]


def test_incidence_context_refuses_circulant_calls(case):
    import ctypes
    op = case["op"]
    rows = (ctypes.c_void_p * 9)()
    with pytest.raises(_lib.PeecError, match="no voxel lattice"):
        _lib.check(op.h, op.L.peec_set_rows(op.h, rows))
    # the context still applies its dense operator afterwards
    w, st = _ris_state(case, 1e9)
    _install(case, w, st)
    x = np.ones(op.N, dtype=np.complex128)
    assert _rel(op.matvec(x, 0), _ris_mv(case, w, st)(x)) < max(1e-11, 4 * _noise(case, w, st, x))


@pytest.mark.parametrize("f", [3e8, 1e10])
def test_retarded_dense_operator_matches_the_oracle(case, f):
    """QS_Rcc_FW == 2: the blocks times exp(-j beta R), formed on the device per frequency,
    against the oracle's rebuilt blocks (iter_solver_QS_S_type.jl:39-59)."""
    c = case
    Lp, P = ris_cases.with_distances(c, c["Lp_data"], c["P_data"])
    op = c["op"]
    op.set_rcc(Lp, P)
    try:
        w = 2 * np.pi * f * c["esc"]["freq"]
        st = RO.frequency_setup(w, c["esc"], c["inc"], P, Lp, c["ports"], {}, c["volumi"], True,
                                50.0, QS_Rcc_FW=2, freq_unscaled=f)
        op.set_rcc_frequency(f)
        _install(c, w, st)
        rng = np.random.default_rng(12)
        x = rng.standard_normal(op.N) + 1j * rng.standard_normal(op.N)
        y_ref = _ris_mv(c, w, st)(x)
        y64 = op.matvec(x, _lib.PREC_FP64)
        tol = max(1e-11, 4 * _noise(c, w, st, x))
        assert _rel(y64, y_ref) < tol, (c["name"], f, _rel(y64, y_ref), tol)
        assert _rel(op.matvec(x, _lib.PREC_FP32), y_ref) < 2e-5
        # the phases matter at this size: the quasi-static blocks give another operator
        op.set_rcc(None, None)
        assert _rel(op.matvec(x, _lib.PREC_FP64), y_ref) > 100 * tol
    finally:
        op.set_rcc(None, None)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_retarded_ris_solver_matches_the_oracle(case, mode):
    from solver_gb300 import ris
    c = case
    Lp, P = ris_cases.with_distances(c, c["Lp_data"], c["P_data"])
    freqs = [1e8, 3e9, 1e10]
    gs = {"Inner_Iter": 200, "tol": [1e-8] * len(freqs)}
    ref = RO.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], P, Lp, c["ports"], {}, gs,
                                   c["volumi"], True, 2, 50.0)
    out = ris.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], P, Lp, c["ports"], {}, gs,
                                    c["volumi"], True, 2, 50.0, mode=mode, op=c["op"], lu="host")
    assert all(r["flag"] == 0 for r in out["info"]), out["info"]
    tol = 1e-7 if mode == "fp64" else 1e-6
    for k in range(len(freqs)):
        assert _rel(out["S"][:, :, k], ref["S"][:, :, k]) < tol, (mode, k)
    # the context is back on the quasi-static blocks afterwards
    w, st = _ris_state(c, 1e9)
    _install(c, w, st)
    x = np.ones(c["op"].N, dtype=np.complex128)
    assert _rel(c["op"].matvec(x, 0), _ris_mv(c, w, st)(x)) < max(1e-11, 4 * _noise(c, w, st, x))
