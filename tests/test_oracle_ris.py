"""CPU: the RIS oracle (oracle/ris_ref.py) and the RIS host logic of the product
(solver_gb300/ris.py).

* The reference's RIS preconditioner takes three LU solves; one solve of their sum gives
  the same vector (what the library does on both paths).
* A dense RIS problem written out from a voxel case's circulant blocks (tests/ris_cases.py)
  has the voxel operator's products: the two restatements agree to rounding.
* The product's Yle, Z_self and lumped admittances equal the oracle's; the RIS cascade
  of a type-2 element differs from the voxel path's in its fifth network, as in the
  reference.
* The dense C-ABI entry points reject a null context (no GPU is touched)."""
import numpy as np
import pytest

from oracle import peec_oracle as O
from oracle import ris_ref as RO
from solver_gb300 import configs, ris
from tests import ris_cases


@pytest.fixture(scope="module")
def crossbar():
    c = ris_cases.voxel_case(configs.crossbar_20x20x4())
    c["Lp_data"], c["P_data"] = ris_cases.dense_blocks(c)
    return c


def _state(c, f):
    w = 2 * np.pi * f * c["esc"]["freq"]
    return w, O.frequency_setup(w, c["esc"], c["inc"], c["diag"], c["Zs"], c["le"], c["ports"],
                                c["z0"])


def test_one_lu_solve_equals_three(crossbar):
    c = crossbar
    w, fs = _state(c, 1e9)
    A, G = c["inc"]["A"], c["inc"]["Gamma"]
    rng = np.random.default_rng(3)
    X1, X2, X3 = (rng.standard_normal(k) + 1j * rng.standard_normal(k)
                  for k in (A.shape[0], G.shape[1], A.shape[1]))
    y3 = RO.precond_3_3_vector(fs["F"], fs["invZ"], fs["invP"], A, G, w, X1, X2, X3)
    M = fs["F"](A.T @ (fs["invZ"] @ X1) - 1j * w * (G @ (fs["invP"] @ X2)) + X3)
    y1 = np.concatenate([fs["invZ"] @ (X1 - A @ M), fs["invP"] @ (X2 + G.T @ M), M])
    assert np.max(np.abs(y1 - y3)) <= 1e-12 * np.max(np.abs(y3))


@pytest.mark.parametrize("f", [1e8, 1e9, 3e9])
def test_dense_ris_operator_equals_the_voxel_operator(crossbar, f):
    c = crossbar
    w, fs = _state(c, f)
    inc = c["inc"]
    N = inc["A"].shape[0] + inc["Gamma"].shape[1] + inc["A"].shape[1]
    rng = np.random.default_rng(11)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    y_vox = O.ComputeMatrixVectorFTT(x, w, inc, c["FFTCP"], c["FFTCLp"], fs["DZ"], fs["Yle"],
                                     c["exp"], fs["invZ"], fs["invP"], fs["F"])
    z_self = fs["DZ"] - 1j * w * np.asarray(c["diag"]["Lp"]).ravel()
    y_ris = RO.ComputeMatrixVectorRis(x, w, inc, c["P_data"], c["Lp_data"], z_self, fs["Yle"],
                                      fs["invZ"], fs["invP"], fs["F"])
    # the rounding noise of the voxel operator itself: the same vector with its
    # preconditioner's three LU solves taken as one (3.8e-11 of max|y| at 100 MHz, where SS
    # is least well conditioned)
    A, G = inc["A"], inc["Gamma"]
    saved = O.precond_3_3_vector

    def one(F, invZ, invP, A_, G_, w_, X1, X2, X3):
        M = F(A_.T @ (invZ @ X1) - 1j * w_ * (G_ @ (invP @ X2)) + X3)
        return np.concatenate([invZ @ (X1 - A_ @ M), invP @ (X2 + G_.T @ M), M])
    O.precond_3_3_vector = one
    try:
        y_one = O.ComputeMatrixVectorFTT(x, w, inc, c["FFTCP"], c["FFTCLp"], fs["DZ"], fs["Yle"],
                                         c["exp"], fs["invZ"], fs["invP"], fs["F"])
    finally:
        O.precond_3_3_vector = saved
    ymax = np.max(np.abs(y_vox))
    noise = np.max(np.abs(y_one - y_vox)) / ymax
    assert np.max(np.abs(y_ris - y_vox)) / ymax <= max(1e-11, 4 * noise)


def test_product_host_state_matches_the_oracle(crossbar):
    c = crossbar
    n = c["inc"]["A"].shape[1]
    le = {"le_nodes": [[0, 5], [3, 9], [7, 2], [11, 4], [8, 1]], "type": [1, 2, 3, 4, 5],
          "R": [10.0, 5.0, 0.0, 50.0, 1e3], "L": [1e-9, 0.0, 2e-9, 1e-8, 0.0],
          "C": [1e-12, 2e-12, 0.0, 1e-13, 5e-12]}
    ports = {"port_nodes": np.asarray(c["ports"]["port_nodes"]).reshape(-1, 2)}
    for f in (1e6, 1e9):
        w = 2 * np.pi * f
        Yp = ris.build_yle_s(le, [3], ports, c["esc"], n, w, 50.0)
        Yo = RO.build_Yle_S(le, [3], ports, c["esc"], n, w, 50.0)
        assert abs(Yp - Yo).max() <= 1e-15 * abs(Yo).max()
    vol = ris_cases.volumi_of(c, seed=5)
    for use_zs in (True, False):
        for f in (1e7, 2e9):
            w = 2 * np.pi * f * c["esc"]["freq"]
            assert np.array_equal(ris.z_self(vol, w, use_zs), RO.z_self(vol, w, use_zs))


@pytest.mark.parametrize("typ", [1, 2, 3, 4, 5])
def test_lumped_admittance_cascade(typ):
    """Every (R, L, C) combination of zero, finite and infinite values: the product's
    cascade equals the oracle's statement for statement (both take IEEE divisions)."""
    vals = (0.0, 1.0, 3e-9, np.inf)
    for R in vals:
        for L in vals:
            for C in vals:
                for w in (0.0, 2 * np.pi * 1e9):
                    a = ris.lumped_admittance_S(typ, R, L, C, w)
                    b = RO.lumped_admittance_S(typ, R, L, C, w)
                    assert (a == b) or (np.isnan(a) and np.isnan(b)), (typ, R, L, C, w, a, b)


def test_ris_type2_cascade_differs_from_the_voxel_one():
    """R = L = 0, C > 0: the first four networks of a type-2 element are not finite; the
    RIS solver's fifth is 1/(1/(jwC)) + jwC = 2jwC (build_Yle_S.jl:86), the voxel path's
    1/(jwL) + jwC is not finite either and its sixth gives jwC."""
    w, C = 2 * np.pi * 1e9, 1e-12
    assert RO.lumped_admittance_S(2, 0.0, 0.0, C, w) == pytest.approx(2j * w * C)
    assert O.lumped_admittance(2, 0.0, 0.0, C, w) == pytest.approx(1j * w * C)


def test_dense_entry_points_reject_a_null_context():
    from solver_gb300 import _lib
    try:
        L = _lib.load(build_if_missing=False)
    except Exception:
        pytest.skip("library not built")
    assert L.peec_set_incidence(None, 0, 0, 0, None, None, 0, None, 1) == -5
    assert L.peec_set_dense(None, None, None, None, None) == -5


def test_retarded_blocks_reduce_to_the_quasi_static_ones_at_zero_phase(crossbar):
    """QS_Rcc_FW == 2 rebuilds the blocks as Lp exp(-j beta R) (iter_solver_QS_S_type.jl:
    39-59): with zero distances they are the quasi-static blocks, and with the case's
    distances the phases grow with frequency while the diagonals (R = 0) stay real."""
    c = crossbar
    Lp, P = ris_cases.with_distances(c, c["Lp_data"], c["P_data"])
    vol = ris_cases.volumi_of(c, seed=2)
    w = 2 * np.pi * 1e9 * c["esc"]["freq"]
    zero = dict(Lp, Rx=0 * Lp["Rx"], Ry=0 * Lp["Ry"], Rz=0 * Lp["Rz"])
    zp = dict(P, R_cc=0 * P["R_cc"])
    st0 = RO.frequency_setup(w, c["esc"], c["inc"], zp, zero, c["ports"], {}, vol, True, 50.0,
                             QS_Rcc_FW=2, freq_unscaled=1e9)
    stq = RO.frequency_setup(w, c["esc"], c["inc"], P, Lp, c["ports"], {}, vol, True, 50.0)
    assert np.array_equal(st0["Lp"]["Lp_x"].real, stq["Lp"]["Lp_x"])
    assert not np.any(st0["Lp"]["Lp_x"].imag)
    st = RO.frequency_setup(w, c["esc"], c["inc"], P, Lp, c["ports"], {}, vol, True, 50.0,
                            QS_Rcc_FW=2, freq_unscaled=1e9)
    assert np.any(st["P"]["P"].imag) and not np.any(np.diag(st["P"]["P"]).imag)
    assert np.array_equal(st["diag_Lp"], stq["diag_Lp"])
