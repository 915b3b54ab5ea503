"""CPU: known-answer checks of the oracle (oracle/peec_oracle.py, oracle/fill_ref.c).
The reference ships no outputs for this path, so the oracle is held to what physics and
the reference's own closed forms fix:

* the fill's coincident-cell Lp integral equals the closed-form bar self inductance of
  compute_diagonals.jl:136-155, and its P integral equals the mesher's face self terms
  (mesher_FFT.jl:114-138);
* far apart, Lp -> mu0 l^2 / (4 pi R) and P -> 1 / (4 pi eps0 R), with the quadrupole
  error falling as 1/R^2;
* the port operator is reciprocal: port 2's solution gives the same S12 as port 1's
  (FFT_solver_QS_S_type.jl:206 fills S symmetrically by assuming it);
* the oracle reproduces its committed regression outputs (tests/golden/oracle_*.npz,
  written by tests/golden/make_fixtures.py)."""
import math

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from solver_gb300 import configs, mesher

MU0 = 4 * math.pi * 1e-7
EPS0 = 8.854187812813e-12
CELL = (1e-4, 2e-4, 5e-5)


def _line(n, axis, step):
    c = np.zeros((n, 3))
    c[:, axis] = np.arange(n) * step
    return c


@pytest.mark.parametrize("dc", [1, 2, 3])
def test_lp_self_matches_closed_form(dc):
    sx, sy, sz = CELL
    l = CELL[dc - 1]
    W, T = [(sy, sz), (sx, sz), (sy, sx)][dc - 1]
    row = O.lp_row(dc, _line(2, 0, 10 * sx), sx, sy, sz)
    assert row[0] == pytest.approx(mesher._lp_self(l, W, T), rel=1e-12)


def test_p_self_matches_mesher_self_terms():
    sx, sy, sz = CELL
    want = mesher.p_self_terms(sx, sy, sz)
    for k, caser in enumerate((1, 3, 5)):
        row = O.p_row(caser, caser, _line(2, 2, 10 * sz), sx, sy, sz, mesher.ESCALINGS["P"])
        assert row[0] == pytest.approx(want[k], rel=1e-12)


# centre distances stay below 200 x the smallest cell edge, where the reference switches
# to its lower-dimensional (suppressed) integrals
FAR = np.array([10, 20, 40])


@pytest.mark.parametrize("dc", [1, 2, 3])
def test_lp_far_field(dc):
    sx, sy, sz = CELL
    l = CELL[dc - 1]
    step = max(CELL)
    row = O.lp_row(dc, _line(41, dc % 3, step), sx, sy, sz)
    err = np.abs(row[FAR] * (FAR * step) / (MU0 / (4 * math.pi) * l * l) - 1)
    assert np.all(err * FAR**2 < 2.0) and err[-1] < 1e-3, err


@pytest.mark.parametrize("caser", [1, 3, 5])
def test_p_far_field(caser):
    sx, sy, sz = CELL
    step = max(CELL)
    row = O.p_row(caser, caser, _line(41, 2 if caser != 5 else 0, step), sx, sy, sz, 1.0)
    err = np.abs(row[FAR] * (FAR * step) * 4 * math.pi * EPS0 - 1)
    assert np.all(err * FAR**2 < 2.0) and err[-1] < 1e-3, err


def test_port_operator_is_reciprocal():
    req = configs.random_mixed(shape=(10, 10, 4), p=0.45, seed=3, nports=2,
                               freqs=[1e8, 3e9], tol=1e-10)
    out, freqs, _settings, z0, (Nx, Ny, Nz) = OM.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, _li, Zs = out
    FFTCP, FFTCLp = O.spectra_from_rows(O.fill_rows(cc, esc, Nx, Ny, Nz), Nx, Ny, Nz)
    m, n = inc["A"].shape
    ns = inc["Gamma"].shape[1]
    pn = np.asarray(ports["port_nodes"])
    sols = {}
    O.FFT_solver_QS_S_type(freqs, esc, inc, FFTCP, FFTCLp, diag, ports, z0, le, exp,
                           {"Inner_Iter": 200, "tol": np.full(len(freqs), 1e-12)}, Zs,
                           callback=lambda k, p, V: sols.__setitem__((k, p), V.copy()))
    for k in range(len(freqs)):
        v = lambda p, q: 2 * (sols[(k, p)][m + ns + pn[q][0]] - sols[(k, p)][m + ns + pn[q][1]])
        s12, s21 = v(0, 1), v(1, 0)
        assert abs(s12 - s21) <= 1e-7 * max(abs(s12), 1e-3 * abs(v(0, 0))), (k, s12, s21)


def _case(tag):
    from pathlib import Path
    g = Path(__file__).resolve().parent / "golden"
    if tag == "crossbar_20x20x4":
        req = configs.crossbar_20x20x4()
    else:
        req = mesher.load_request(g / f"{tag}.json")
        if tag == "first_run_data_2_materials":
            req["solverInput"]["frequencies"] = [1e9, 3e9]
    return req, np.load(g / f"oracle_{tag}.npz")


@pytest.mark.parametrize("tag", ["first_run_data", "first_run_data_2_materials",
                                 "crossbar_20x20x4"])
def test_oracle_matches_its_regression_pins(tag):
    req, pin = _case(tag)
    out, freqs, settings, z0, (Nx, Ny, Nz) = OM.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, _li, Zs = out
    rows = O.fill_rows(cc, esc, Nx, Ny, Nz)
    for key, row in rows.items():
        np.testing.assert_allclose(row, pin[f"row_{key}"], rtol=1e-13, atol=0)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, Nx, Ny, Nz)
    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    y = O.ComputeMatrixVectorFTT(pin["x"], w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp,
                                 fs["invZ"], fs["invP"], fs["F"])
    np.testing.assert_allclose(y, pin["y"], rtol=0, atol=1e-9 * np.max(np.abs(pin["y"])))
    st = {"Inner_Iter": settings["Inner_Iter"], "tol": np.full(len(freqs), settings["tol"])}
    res = O.FFT_solver_QS_S_type(freqs, esc, inc, FFTCP, FFTCLp, diag, ports, z0, le, exp, st, Zs)
    np.testing.assert_allclose(res["Z"], pin["Z"], rtol=1e-8)


# grids whose rows reach the far-field (suppressed) branches of the reference's integral
# dispatch: (shape, cell edges)
FAR_GRIDS = {
    "cubic_232x3x2": ((232, 3, 2), (5e-5, 5e-5, 5e-5)),
    "thin_40x40x3": ((40, 40, 3), (1e-4, 1e-4, 1e-6)),
    "needle_60x4x4": ((60, 4, 4), (1e-3, 1e-5, 1e-5)),
    "aniso_120x48x4": ((120, 48, 4), (1e-4, 2e-4, 5e-5)),
}


@pytest.mark.parametrize("name", sorted(FAR_GRIDS))
def test_far_field_branches_reach_the_point_limit(name):
    """Every distant entry (centre distance R > 30 x the longest edge; on cubic voxels
    R > 205 edges, past the switch, since the double near-field form itself loses
    ~1e-3 to cancellation just before it) is within 3 (edge/R)^2 of the point-point
    value -- except collinear pairs that reach the line-line branch: the reference's
    integ_line_line_sp_fft / _P (compute_Lp_Voxels.jl:514-529,
    compute_row_P_sup.jl:461-476) evaluate those in absolute coordinates, and the
    oracle (like the GPU fill) keeps that."""
    shape, cell = FAR_GRIDS[name]
    cu = np.zeros(shape, dtype=bool)
    cu[0:3, 0, 0] = True
    req = configs.make_request({"copper": cu}, [dict(configs.COPPER)], cell,
                               [((0, 0, 0), (2, 0, 0))], [1e9], 1e-8)
    out, _f, _s, _z, _grid = OM.parse_request(req)
    cc = out[2]
    sx, sy, sz = cc["sx"], cc["sy"], cc["sz"]
    edge = max(sx, sy, sz)
    cut = 205 * edge if name.startswith("cubic") else 30 * edge
    V = sx * sy * sz
    rows = [(dc, key, None) for dc, key in ((1, "Lpx"), (2, "Lpy"), (3, "Lpz"))]
    rows += [(None, key, cs) for key, cs in (("p12_se", 1), ("p34_se", 3), ("p56_se", 5))]
    collinear_seen = far_total = 0
    for dc, key, cs in rows:
        c = np.asarray(cc[key])
        if dc:
            S = [(sy * sz) ** 2, (sx * sz) ** 2, (sx * sy) ** 2][dc - 1]
            (row, far) = O.lp_row(dc, c, sx, sy, sz, count_far=True)
            point = lambda R: 1e-7 / S * V * V / R
        else:
            (row, far) = O.p_row(cs, cs, c, sx, sy, sz, 1.0, count_far=True)
            point = lambda R: 1 / (4 * math.pi * 8.854187816997944e-12 * R)
        d = c - c[0]
        R = np.linalg.norm(d, axis=1)
        sel = np.flatnonzero(R > cut)
        far_total += far
        collinear = np.sum(np.abs(d[sel]) < 1e-12 * edge, axis=1) >= 2
        rel = np.abs(row[sel] - point(R[sel])) / point(R[sel])
        ok = rel <= 3 * (edge / R[sel]) ** 2
        assert np.all(ok | collinear), (key, float(rel[~(ok | collinear)].max()))
        collinear_seen += int(np.sum(~ok & collinear))
    assert far_total > 0
    if name == "needle_60x4x4":
        assert collinear_seen > 0


def test_s_to_z_and_y_follow_the_reference():
    """s2z_fft / s2y_fft (FFT_solver_QS_S_type.jl:265-285): Z = z0 (I - S)^-1 (I + S) and
    Y = z0 (I + S)^-1 (I - S). The reference scales Y by z0 rather than 1/z0, so Z Y =
    z0^2 I; the restatement (oracle and solver_gb300.api) keeps that."""
    from solver_gb300 import api
    rng = np.random.default_rng(4)
    S = (rng.standard_normal((3, 3, 2)) + 1j * rng.standard_normal((3, 3, 2))) * 0.2
    S = 0.5 * (S + S.transpose(1, 0, 2))
    z0 = 50.0
    for f in (O.s2z, api.s2z_fft):
        Z = f(S, z0)
        assert np.allclose(Z[:, :, 1] @ (np.eye(3) - S[:, :, 1]) / z0, np.eye(3) + S[:, :, 1])
    Y = api.s2y_fft(S, z0)
    np.testing.assert_allclose(O.s2y(S, z0), Y, rtol=1e-14)
    for k in range(2):
        np.testing.assert_allclose(api.s2z_fft(S, z0)[:, :, k] @ Y[:, :, k], z0 ** 2 * np.eye(3),
                                   atol=1e-9 * z0 ** 2)


def test_oracle_gmres_matches_a_dense_solve():
    """The oracle's Householder GMRES (gmres_custom.jl restated) on the crossbar operator
    against a dense LU solve of the explicitly assembled operator: at relative residual
    1e-11 the solutions agree to ~10x that (the operator's condition number is ~3e6, and
    the recursion's residual tracks the true one)."""
    req = configs.crossbar_20x20x4()
    out, freqs, _settings, z0, grid = OM.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, _li, Zs = out
    FFTCP, FFTCLp = O.spectra_from_rows(O.fill_rows(cc, esc, *grid), *grid)
    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    mv = lambda v: O.ComputeMatrixVectorFTT(v, w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp,
                                            fs["invZ"], fs["invP"], fs["F"])
    m, n = inc["A"].shape
    ns = inc["Gamma"].shape[1]
    n1, n2 = ports["port_nodes"][0]
    i_s = np.zeros(n)
    i_s[n1], i_s[n2] = esc["Is"], -esc["Is"]
    tn = O.precond_3_3_Kt_fft(fs["F"], fs["invZ"], fs["invP"], inc["A"], inc["Gamma"], m, ns, i_s)
    x, flag, relres, it, rv = O.gmres_custom(tn, False, 1e-11, 200, None, mv)
    assert flag == 0 and relres <= 1e-11
    x_dense = np.linalg.solve(O.dense_operator(mv, m + ns + n), tn)
    assert np.max(np.abs(x - x_dense)) <= 1e-9 * np.max(np.abs(x_dense))


def _dense(A):
    A = np.asarray(A, dtype=np.complex128)
    return lambda v: A @ v


def test_oracle_gmres_control_flow_known_answers():
    """The oracle GMRES on small dense systems with known answers, following the
    MATLAB semantics of gmres_custom.jl:
    * a zero right-hand side returns x = 0, flag 0, relres 0, iter [0, 0] (:20-28);
    * an initial guess that already meets the tolerance returns unchanged with iter [0, 0]
      and resvec = [|r0|] (:47-55);
    * the identity converges in one inner step;
    * a diagonal operator with k distinct eigenvalues converges in k inner steps (the
      Krylov space holds the solution after k steps);
    * maxit is clamped to the system size (:12-16): with maxit 100 a 6 x 6 system
      converges within 6 steps;
    * a budget too small ends with flag 1 at the smallest residual seen."""
    rng = np.random.default_rng(3)
    n = 6
    b = rng.standard_normal(n) + 1j * rng.standard_normal(n)

    x, flag, relres, it, rv = O.gmres_custom(np.zeros(n), False, 1e-10, 5, None, _dense(np.eye(n)))
    assert flag == 0 and relres == 0.0 and list(it) == [0, 0] and not np.any(x)
    assert list(rv) == [0.0]

    A = np.diag([1.0, 2.0, 3.0, 4.0, 5.0, 6.0]) + 0j
    xs = np.linalg.solve(A, b)
    x, flag, relres, it, rv = O.gmres_custom(b, False, 1e-8, 5, xs, _dense(A))
    assert flag == 0 and list(it) == [0, 0] and np.array_equal(x, xs)
    assert len(rv) == 1 and rv[0] == np.linalg.norm(b - A @ xs)

    x, flag, relres, it, rv = O.gmres_custom(b, False, 1e-12, 5, None, _dense(np.eye(n)))
    assert flag == 0 and list(it) == [1, 1] and np.allclose(x, b, rtol=0, atol=1e-14)

    D = np.diag([2.0, 2.0, 5.0, 5.0, 5.0, -1.0]) + 0j    # three distinct eigenvalues
    x, flag, relres, it, rv = O.gmres_custom(b, False, 1e-10, 6, None, _dense(D))
    assert flag == 0 and list(it) == [1, 3]
    assert np.allclose(x, np.linalg.solve(D, b), rtol=1e-9, atol=0)

    M = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n)) + 4 * np.eye(n)
    x, flag, relres, it, rv = O.gmres_custom(b, False, 1e-12, 100, None, _dense(M))
    assert flag == 0 and it[0] == 1 and it[1] <= n
    assert np.linalg.norm(b - M @ x) <= 1e-11 * np.linalg.norm(b)

    x, flag, relres, it, rv = O.gmres_custom(b, False, 1e-14, 2, None, _dense(M))
    assert flag == 1 and list(it) == [1, 2]
    assert np.isclose(relres, np.min(rv) / np.linalg.norm(b), rtol=1e-8)
    assert np.isclose(np.linalg.norm(b - M @ x) / np.linalg.norm(b), relres, rtol=1e-8)


def test_lumped_element_admittances():
    """Lumped element types 1..5 (build_Yle_FFT.jl:128-209): the element network for
    generic values, the reference's fallbacks when an element vanishes, and the product's
    table-driven form against the oracle's statement-by-statement one on random corners."""
    from solver_gb300.frequency import lumped_admittance as product
    w = 2 * np.pi * 1.3e9
    jw = 1j * w
    R, L, C = 37.0, 2.2e-9, 0.8e-12
    par = lambda *ys: sum(ys)   # admittances of parallel branches add
    ser = lambda *zs: sum(zs)   # impedances of series elements add
    want = {1: 1 / ser(R, jw * L, 1 / (jw * C)),
            2: par(1 / ser(R, jw * L), jw * C),
            3: par(1 / ser(R, 1 / (jw * C)), 1 / (jw * L)),
            4: par(1 / R, jw * C, 1 / (jw * L)),
            5: par(1 / R, 1 / ser(jw * L, 1 / (jw * C)))}
    for t, y in want.items():
        assert abs(O.lumped_admittance(t, R, L, C, w) - y) <= 1e-14 * abs(y), t
    # a vanishing element is dropped from the network
    assert O.lumped_admittance(1, R, L, 0.0, w) == pytest.approx(1 / (R + jw * L), rel=1e-14)
    assert O.lumped_admittance(2, 0.0, 0.0, C, w) == pytest.approx(jw * C, rel=1e-14)
    assert O.lumped_admittance(3, R, 0.0, C, w) == pytest.approx(1 / (R + 1 / (jw * C)), rel=1e-14)
    assert O.lumped_admittance(4, R, 0.0, C, w) == pytest.approx(1 / R + jw * C, rel=1e-14)
    assert O.lumped_admittance(4, 0.0, L, C, w) == pytest.approx(jw * C + 1 / (jw * L), rel=1e-14)
    assert O.lumped_admittance(5, R, L, 0.0, w) == pytest.approx(1 / R + 1 / (jw * L), rel=1e-14)
    assert O.lumped_admittance(5, 0.0, L, C, w) == pytest.approx(1 / (jw * L + 1 / (jw * C)), rel=1e-14)
    # nothing finite left: 0
    assert O.lumped_admittance(1, 0.0, 0.0, 0.0, w) == 0.0
    assert O.lumped_admittance(4, 0.0, 0.0, 0.0, w) == 0.0
    rng = np.random.default_rng(12)
    for _ in range(400):
        t = int(rng.integers(1, 6))
        vals = [v if rng.random() < 0.7 else 0.0 for v in (rng.uniform(1e-3, 1e3),
                                                            rng.uniform(1e-12, 1e-8),
                                                            rng.uniform(1e-15, 1e-11))]
        ww = 2 * np.pi * 10 ** rng.uniform(6, 10)
        a, b = product(t, *vals, ww), O.lumped_admittance(t, *vals, ww)
        assert a == b or abs(a - b) <= 1e-15 * abs(b), (t, vals, ww, a, b)
    with pytest.raises(ValueError):
        product(6, R, L, C, w)


def test_yle_stamps_lumped_elements_and_ports():
    """Yle (build_Yle_FFT.jl:1-126): each element's admittance y between its two nodes as
    [[y, -y], [-y, y]], each port's 1/z0 the same way, all times the Yle scaling."""
    from solver_gb300.frequency import lumped_admittance, yle_matrix
    w = 2 * np.pi * 5e8
    le = {"le_nodes": [[0, 3], [2, 3]], "type": [2, 5], "R_value": [10.0, 75.0],
          "L_value": [1e-9, 3e-9], "C_value": [1e-12, 0.0]}
    ports = {"port_nodes": [[1, 4]]}
    Y = yle_matrix(le, ports, 5, w, 50.0, 2.5).toarray()
    want = np.zeros((5, 5), complex)
    for (a, b), y in (((0, 3), lumped_admittance(2, 10.0, 1e-9, 1e-12, w)),
                      ((2, 3), lumped_admittance(5, 75.0, 3e-9, 0.0, w)), ((1, 4), 1 / 50.0)):
        want[a, a] += y
        want[b, b] += y
        want[a, b] -= y
        want[b, a] -= y
    assert np.allclose(Y, 2.5 * want, rtol=1e-15, atol=0)
