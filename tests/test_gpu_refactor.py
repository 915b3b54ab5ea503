"""GPU: SS factorised on the device at later frequencies, in the pattern and pivot order
of one host factorisation (peec_lu_refactor_setup, peec_set_frequency_refactor), against
the oracle, which factorises every frequency with SuperLU as the reference does with
UMFPACK (FFT_solver_QS_S_type.jl:118-119):

* the set-up installs the device's factors at the host factors' frequency, giving the
  same operator to rounding, bit-identical when repeated;
* at every frequency the device factors solve SS with the backward error of a stable
  factorisation (1e-13), as the host factors do;
* frequency sweeps through api with lu="device" (host factors at the first frequency
  only) converge with iteration counts within two of the oracle's and Z within 1e-6
  (FP64, both at 1e-8), and within 1e-6 of the oracle's FP64 sweep at 1e-10 in mixed
  precision on two port lanes."""
import copy

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from solver_gb300 import api, configs, mesher
from solver_gb300.operator import GpuOperator

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


CASES = {
    "crossbar_20x20x4": lambda: configs.crossbar_20x20x4(),
    "random_24x20x12": lambda: configs.random_mixed((24, 20, 12), s=5e-5, p=0.35, seed=7,
                                                    nports=2, freqs=[1e8, 1e9, 3e9], tol=1e-8),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    req = CASES[request.param]()
    out, freqs, settings, z0, grid = OM.parse_request(copy.deepcopy(req))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    pe = mesher.parse_request(copy.deepcopy(req))[0]
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    op = GpuOperator(pe[1], pe[4], pe[3]["P"])
    op.set_rows(rows)
    c = dict(esc=esc, inc=inc, diag=diag, exp=exp, ports=ports, le=le, Zs=Zs, z0=z0,
             FFTCP=FFTCP, FFTCLp=FFTCLp, settings=settings, op=op, name=request.param,
             prod=dict(esc=pe[0], inc=pe[1], diag=pe[3], exp=pe[4], ports=pe[5], le=pe[6],
                       Zs=pe[8]))
    yield c
    op.close()


def _state(c, f):
    w = 2 * np.pi * f * c["esc"]["freq"]
    return w, O.frequency_setup(w, c["esc"], c["inc"], c["diag"], c["Zs"], c["le"], c["ports"],
                                c["z0"])


def _mv(c, w, fs, single=False):
    def mv(x):
        saved = O.precond_3_3_vector
        if single:
            def one(F, invZ, invP, A_, G_, w_, X1, X2, X3):
                Mv = F(A_.T @ (invZ @ X1) - 1j * w_ * (G_ @ (invP @ X2)) + X3)
                return np.concatenate([invZ @ (X1 - A_ @ Mv), invP @ (X2 + G_.T @ Mv), Mv])
            O.precond_3_3_vector = one
        try:
            return O.ComputeMatrixVectorFTT(x, w, c["inc"], c["FFTCP"], c["FFTCLp"], fs["DZ"],
                                            fs["Yle"], c["exp"], fs["invZ"], fs["invP"], fs["F"])
        finally:
            O.precond_3_3_vector = saved
    return mv


def _setup(c, f0):
    w0, fs0 = _state(c, f0)
    c["op"].set_frequency(w0, fs0["DZ"], fs0["Yle"], fs0["lu"])
    c["op"].enable_refactor(fs0["Yle"])
    return w0, fs0


def test_refactor_at_the_setup_frequency(case):
    """The set-up installs the device's own factors at the host factors' frequency: the
    same operator to rounding (different summation orders; 3e-11 on the crossbar, whose SS
    is the least well conditioned), and a repeated device factorisation is bit-identical."""
    c = case
    w0, fs0 = _state(c, 1e9)
    c["op"].set_frequency(w0, fs0["DZ"], fs0["Yle"], fs0["lu"])
    rng = np.random.default_rng(31)
    x = rng.standard_normal(c["op"].N) + 1j * rng.standard_normal(c["op"].N)
    y_host = c["op"].matvec(x, 0)
    c["op"].enable_refactor(fs0["Yle"])
    y_dev = c["op"].matvec(x, 0)
    assert _rel(y_dev, y_host) < 1e-10
    c["op"].set_frequency_refactor(w0, fs0["DZ"], fs0["Yle"])
    assert np.array_equal(c["op"].matvec(x, 0), y_dev)


def test_refactor_backward_error(case):
    """The device factors solve SS with the backward error of a stable factorisation at
    every frequency (the solve read from the port right-hand side, whose node block is
    SS \\ is, FFT_solver_QS_S_type.jl:237-262): |SS x - is| <= 1e-13 (|SS| |x| + |is|), as
    for the host factors. Their operator is not compared with the oracle's entry for entry:
    where SS is ill-conditioned (low frequencies) two valid factorisations of it differ by
    about cond(SS) eps (the device factors keep the first frequency's pivot order, SuperLU
    pivots again)."""
    c = case
    _setup(c, 1e9)
    m, ns = c["op"].m, c["op"].ns
    pn = np.asarray(c["ports"]["port_nodes"], dtype=np.int64).reshape(-1, 2)
    Is = c["esc"]["Is"]
    for f in (1e7, 1e8, 1e9, 3e9):
        w, fs = _state(c, f)
        SS = fs["SS"]
        isv = np.zeros(SS.shape[0])
        isv[pn[0, 0]], isv[pn[0, 1]] = Is, -Is
        scale = abs(SS).max()
        for dev in (True, False):
            if dev:
                c["op"].set_frequency_refactor(w, fs["DZ"], fs["Yle"])
            else:
                c["op"].set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
                c["op"].enable_refactor(fs["Yle"])  # back to device factors for the next f
                c["op"].set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
            x3 = c["op"].port_rhs(pn[0, 0], pn[0, 1], Is)[m + ns:]
            r = SS @ x3 - isv
            be = np.max(np.abs(r)) / (scale * np.max(np.abs(x3)) + Is)
            assert be < 1e-13, (c["name"], f, dev, be)
        c["op"].enable_refactor(fs["Yle"])


def test_refactor_rejects_another_yle_pattern(case):
    c = case
    w0, fs0 = _setup(c, 1e9)
    import scipy.sparse as sp
    Y = sp.lil_matrix(fs0["Yle"].shape, dtype=np.complex128)
    Y[0, 0] = 1.0
    from solver_gb300 import _lib
    with pytest.raises(_lib.PeecError):
        c["op"].set_frequency_refactor(w0, fs0["DZ"], Y.tocsr())


def test_graphs_kept_across_device_factorised_frequencies(case):
    """A frequency change with SS factorised on the device writes DZ, Yle, w and the
    factors in place and keeps the context's captured graphs (operator applications and
    the device GMRES loop). Solves through kept graphs equal, bit for bit, those of a
    context that captures its graphs afresh at that frequency."""
    c = case
    w0, fs0 = _setup(c, 1e9)
    pn = np.asarray(c["ports"]["port_nodes"], dtype=np.int64).reshape(-1, 2)
    tn0 = c["op"].port_rhs(pn[0, 0], pn[0, 1], c["esc"]["Is"])
    c["op"].solve_mixed(tn0, None, 1e-8)
    c["op"].gmres(tn0, None, 1e-8, 60)  # graphs of both kinds captured at 1 GHz
    w1, fs1 = _state(c, 3e8)
    other = c["op"].clone()
    try:
        other.set_frequency(w0, fs0["DZ"], fs0["Yle"], fs0["lu"])
        other.enable_refactor(fs0["Yle"])
        for op in (c["op"], other):
            op.set_frequency_refactor(w1, fs1["DZ"], fs1["Yle"])
        tn1 = c["op"].port_rhs(pn[0, 0], pn[0, 1], c["esc"]["Is"])
        assert np.array_equal(tn1, other.port_rhs(pn[0, 0], pn[0, 1], c["esc"]["Is"]))
        g0 = c["op"].device_loop_stats()[0]
        xa = c["op"].solve_mixed(tn1, None, 1e-8)
        ya = c["op"].gmres(tn1, None, 1e-8, 60)
        assert c["op"].device_loop_stats()[0] > g0
        xb = other.solve_mixed(tn1, None, 1e-8)
        yb = other.gmres(tn1, None, 1e-8, 60)
        assert xa[1:] == xb[1:] and np.array_equal(xa[0], xb[0])
        assert (ya[1], list(ya[3])) == (yb[1], list(yb[3])) and np.array_equal(ya[0], yb[0])
        # and the kept graphs solve the new frequency's system
        r = tn1 - _mv(c, w1, fs1)(xa[0])
        assert np.linalg.norm(r) <= 1e-6 * np.linalg.norm(tn1)
    finally:
        other.close()


def test_device_formed_state_matches_the_host_state(case):
    """peec_set_frequency_device forms DZ on the device from the edge data (Z_self of the
    four edge halves, the surface-impedance selection on surface edges, jw Lp_self), as
    frequency.FrequencyState does on the host: the operators agree to the last bits of DZ
    (division orders), and a sweep through device-formed states gives the same port
    impedances as one through host states."""
    from solver_gb300.frequency import DeviceFrequencyState, FrequencyState
    c = case
    p = c["prod"]
    _setup(c, 1e9)
    op = c["op"]
    op.set_edge_state(p["diag"], p["Zs"], p["esc"])
    rng = np.random.default_rng(17)
    x = rng.standard_normal(op.N) + 1j * rng.standard_normal(op.N)
    n = p["inc"]["A"].shape[1]
    for f in (1e7, 3e8, 1e9, 5e9):
        w = 2 * np.pi * f * p["esc"]["freq"]
        hs = FrequencyState(w, p["esc"], p["inc"], p["diag"], p["Zs"], p["le"], p["ports"],
                            c["z0"], factor=False)
        op.set_frequency_refactor(w, hs.DZ, hs.Yle)
        y_host = op.matvec(x, 0)
        ds = DeviceFrequencyState(w, p["esc"], n, p["le"], p["ports"], c["z0"])
        op.set_frequency_device(w, ds.Yle)
        y_dev = op.matvec(x, 0)
        assert _rel(y_dev, y_host) < 1e-12, (c["name"], f, _rel(y_dev, y_host))
    # a refused call leaves a clear error: no edge data on a fresh context
    other = op.clone()
    try:
        from solver_gb300 import _lib
        with pytest.raises(_lib.PeecError, match="edge data"):
            other.set_frequency_device(w, ds.Yle)
    finally:
        other.close()
