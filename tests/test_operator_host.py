"""CPU: the host half of GpuOperator (the conversion of the reference's data structures
into the C ABI's flat arrays, and its argument checks), run against a stand-in for
libpeec_gb300.so that records each call's arguments and returns success.

* The topology arrays handed to peec_set_topology agree with the incidence matrices
  (edge n1/n2 are the -1/+1 columns of A's rows; surface nodes are Gamma's rows).
* Every parity geometry's genuine frequency state (Yle, SuperLU factors, DZ) passes the
  wrapper's length checks, and the exported LU parts are CSR of size n.
* Vectors of the wrong length, a short diagP and a wrong-sized Yle are rejected before any
  library call."""
import ctypes

import numpy as np
import pytest

from oracle import peec_oracle as O
from solver_gb300 import _lib, configs, mesher
from solver_gb300 import operator as gop


class FakeLib:
    """Arrays are read during the call, as the library copies them before it returns."""

    def __init__(self):
        self.calls = {}

    def peec_last_error(self, ctx):
        return b"stand-in"

    def peec_set_topology(self, h, Nx, Ny, Nz, mx, my, mz, ecell, n1, n2, ns, fam, scell,
                          snode, n):
        m = mx + my + mz
        self.n = n
        self.calls.setdefault("peec_set_topology", []).append(dict(
            grid=(Nx, Ny, Nz), m=m, ns=ns, n=n, ecell=_arr(ecell, m, np.int64),
            n1=_arr(n1, m, np.int64), n2=_arr(n2, m, np.int64), fam=_arr(fam, ns, np.int32),
            scell=_arr(scell, ns, np.int64), snode=_arr(snode, ns, np.int64)))
        return 0

    def peec_set_frequency(self, h, w, DZ, nnz, yr, yc, yv, Lp, Lc, Lv, Up, Uc, Uv, pr, pc,
                           extra):
        self.calls.setdefault("peec_set_frequency", []).append(dict(
            Lp=_arr(Lp, self.n + 1, np.int64), Up=_arr(Up, self.n + 1, np.int64),
            pr=_arr(pr, self.n, np.int64), pc=_arr(pc, self.n, np.int64)))
        return 0

    def __getattr__(self, name):
        if not name.startswith("peec_"):
            raise AttributeError(name)

        def call(*args):
            self.calls.setdefault(name, []).append(args)
            return 0
        return call


def _arr(p, n, dtype):
    """Reads n values of dtype behind a ctypes pointer argument (c_void_p)."""
    addr = p.value if isinstance(p, ctypes.c_void_p) else p
    return np.ctypeslib.as_array(ctypes.cast(addr, ctypes.POINTER(np.ctypeslib.as_ctypes_type(
        dtype))), shape=(n,)).copy()


@pytest.fixture
def fake(monkeypatch):
    L = FakeLib()
    monkeypatch.setattr(_lib, "load", lambda *a, **k: L)
    return L


CASES = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_12x10x6": lambda: configs.random_mixed((12, 10, 6), s=5e-5, p=0.35, seed=7,
                                                   nports=2, freqs=[1e8], tol=1e-8),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_topology_and_frequency_arguments(fake, name):
    out, freqs, settings, z0, grid = mesher.parse_request(CASES[name]())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = gop.GpuOperator(inc, exp, diag["P"])
    (t,) = fake.calls["peec_set_topology"]
    m, ns, n = t["m"], t["ns"], t["n"]
    assert t["grid"] == tuple(grid) and (m, ns, n) == (op.m, op.ns, op.n)
    A = inc["A"].tocsr()
    rows = np.arange(m)
    assert np.all(A[rows, t["n1"]].A1 == -1) and np.all(A[rows, t["n2"]].A1 == 1)
    Gm = inc["Gamma"].tocsc()
    assert np.array_equal(t["snode"], Gm.indices)
    assert set(np.unique(t["fam"])) <= {0, 1, 2}
    assert t["ecell"].min() >= 0 and t["scell"].min() >= 0
    assert np.bincount(t["fam"], minlength=3).sum() == ns

    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    op.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
    (f,) = fake.calls["peec_set_frequency"]
    for ptr in (f["Lp"], f["Up"]):
        assert ptr[0] == 0 and np.all(np.diff(ptr) >= 1)   # a diagonal entry in every row
    assert np.array_equal(np.sort(f["pr"]), np.arange(n))
    assert np.array_equal(np.sort(f["pc"]), np.arange(n))

    x, flag, relres, it, rv = op.gmres(np.ones(op.N), None, 1e-8, 10)
    assert x.shape == (op.N,)
    x, flag, relres, outer, inner = op.solve_mixed(np.ones(op.N), None, 1e-8)
    assert x.shape == (op.N,)

    with pytest.raises(ValueError):
        op.gmres(np.ones(op.N - 1), None, 1e-8, 10)
    with pytest.raises(ValueError):
        op.solve_mixed(np.ones(op.N), np.ones(op.N + 1), 1e-8)
    with pytest.raises(ValueError):
        op.matvec(np.ones(op.N + 1))
    with pytest.raises(ValueError):
        op.set_frequency(w, fs["DZ"][:-1], fs["Yle"], fs["lu"])
    import scipy.sparse as sp
    with pytest.raises(ValueError):
        op.set_frequency(w, fs["DZ"], sp.eye(op.n + 1, format="csr"), fs["lu"])
    with pytest.raises(ValueError):
        gop.GpuOperator(inc, exp, np.asarray(diag["P"]).ravel()[:-1])


def test_cached_state_is_keyed_by_the_objects_themselves(fake):
    """api's frequency and spectra caches hold the host objects they were built from and
    compare them by identity: an equal but new object uploads again, the same object does
    not, and new device rows invalidate the spectra cache."""
    from solver_gb300 import api
    out, freqs, settings, z0, grid = mesher.parse_request(configs.crossbar_20x20x4())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = gop.GpuOperator(inc, exp, diag["P"])
    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    n_set = lambda: len(fake.calls.get("peec_set_frequency", []))
    api._set_freq(op, w, fs["DZ"], fs["Yle"], fs["lu"])
    api._set_freq(op, w, fs["DZ"], fs["Yle"], fs["lu"])
    assert n_set() == 1
    api._set_freq(op, w, fs["DZ"].copy(), fs["Yle"], fs["lu"])
    assert n_set() == 2
    api._set_freq(op, w * 2, fs["DZ"], fs["Yle"], fs["lu"])
    assert n_set() == 3
    op.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])          # unkeyed: always uploads
    api._set_freq(op, w, fs["DZ"], fs["Yle"], fs["lu"])
    assert n_set() == 5

    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    n_rows = lambda: len(fake.calls.get("peec_set_rows", []))
    api._ensure_spectra(op, FFTCP, FFTCLp)
    api._ensure_spectra(op, FFTCP, FFTCLp)
    assert n_rows() == 1
    op.set_rows(rows)                                            # other rows on the device
    api._ensure_spectra(op, FFTCP, FFTCLp)
    assert n_rows() == 3


def test_library_error_codes_reach_the_caller(monkeypatch):
    """A failing library call raises PeecError carrying the code and the library's message
    (here a host allocation failure, PEEC_ERR_OOM, as the exception guard returns it); a
    cancelled solve (PEEC_ERR_CANCELLED) comes back as the reference's flag 99."""
    class Failing(FakeLib):
        def __init__(self, codes):
            super().__init__()
            self.codes = codes

        def peec_last_error(self, ctx):
            return b"peec_set_topology: host memory allocation failed"

        def peec_set_topology(self, *args):
            return self.codes.get("peec_set_topology", 0)

        def __getattr__(self, name):
            if not name.startswith("peec_"):
                raise AttributeError(name)
            return lambda *a: self.codes.get(name, 0)

    out, freqs, settings, z0, grid = mesher.parse_request(configs.crossbar_20x20x4())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    L = Failing({"peec_set_topology": -2})
    monkeypatch.setattr(_lib, "load", lambda *a, **k: L)
    with pytest.raises(_lib.PeecError) as ei:
        gop.GpuOperator(inc, exp, diag["P"])
    assert ei.value.code == -2 and "allocation failed" in str(ei.value)
    assert "PEEC_ERR_OOM" in str(ei.value)

    L = Failing({"peec_gmres": -3, "peec_solve_mixed": -3})
    monkeypatch.setattr(_lib, "load", lambda *a, **k: L)
    op = gop.GpuOperator(inc, exp, diag["P"])
    b = np.ones(op.N)
    assert op.gmres(b, None, 1e-8, 10)[1] == 99
    assert op.solve_mixed(b, None, 1e-8)[1] == 99


def test_single_layer_grid(fake):
    """A planar trace (Nz = 1): the z edge family is empty (mz = 0, no Lpz row), the host
    wrapper passes a consistent topology, and the oracle solves the port to flag 0 with an
    inductive impedance (a copper strip at 1 GHz)."""
    cu = np.zeros((16, 8, 1), bool)
    cu[1:15, 3:5, 0] = True
    req = configs.make_request({"copper": cu}, [dict(configs.COPPER)], (1e-4,) * 3,
                               [((1, 3, 0), (14, 4, 0))], [1e9], 1e-8)
    out, freqs, settings, z0, grid = mesher.parse_request(req)
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    assert grid == (16, 8, 1) and int(inc["mz"]) == 0
    op = gop.GpuOperator(inc, exp, diag["P"])
    (t,) = fake.calls["peec_set_topology"]
    assert t["grid"] == (16, 8, 1) and t["m"] == int(inc["mx"]) + int(inc["my"])
    rows = O.fill_rows(cc, esc, *grid)
    assert "Lpz" not in rows or np.asarray(rows["Lpz"]).size == 0
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    res = O.FFT_solver_QS_S_type(freqs, esc, inc, FFTCP, FFTCLp, diag, ports, z0, le, exp,
                                 {"Inner_Iter": 100, "tol": np.full(1, 1e-8)}, Zs)
    Z = res["Z"][0, 0, 0]
    assert np.isfinite(Z) and Z.real > 0 and Z.imag > 0


@pytest.mark.parametrize("shape,seed", [((9, 7, 5), 3), ((6, 2, 5), 4), ((8, 6, 1), 5)])
def test_rows_recovered_from_reference_spectra(shape, seed):
    """The drop-in API accepts the reference's own spectra (FFTCP / FFTCLp at the 2N
    extents, store_circulant_fft) and recovers the generating rows on the host; the
    recovered rows equal the rows the spectra were built from."""
    from solver_gb300 import api
    out, freqs, settings, z0, grid = mesher.parse_request(
        configs.random_copper(shape, p=0.5, seed=seed))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    got = api.rows_from_reference_spectra(FFTCP, FFTCLp, grid)
    for k, v in rows.items():
        v = np.asarray(v).ravel()
        if v.size == 0:
            continue
        assert np.max(np.abs(got[k] - v)) <= 1e-12 * np.max(np.abs(v)), k


def _fixture_requests():
    import gzip
    import json
    from pathlib import Path
    G = Path(__file__).resolve().parent / "golden"
    r2 = mesher.load_request(G / "first_run_data_2_materials.json")
    r2["solverInput"]["frequencies"] = [1e9, 3e9]
    return {"first_run_data": mesher.load_request(G / "first_run_data.json"),
            "first_run_data_2_materials": r2,
            "crossbar_57x57x13": json.loads(gzip.open(G / "crossbar.json.gz").read()),
            "crossbar_20x20x4": configs.crossbar_20x20x4()}


@pytest.mark.parametrize("name", ["first_run_data", "first_run_data_2_materials",
                                  "crossbar_57x57x13", "crossbar_20x20x4"])
def test_product_frequency_state_matches_the_oracle(name):
    """The product's per-frequency host state (frequency.FrequencyState: edge impedances
    with the surface-impedance switch, lumped and port admittances, SS) equals the
    oracle's restatement of FFT_solver_QS_S_type.jl:102-119 at every frequency of the
    reference's fixtures, and the product's S-to-Z/Y conversions equal the oracle's."""
    from solver_gb300 import api
    from solver_gb300 import frequency as fq
    out, freqs, settings, z0, grid = mesher.parse_request(_fixture_requests()[name])
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    for f in freqs:
        w = 2 * np.pi * f * esc["freq"]
        st = fq.FrequencyState(w, esc, inc, diag, Zs, le, ports, z0)
        fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
        assert np.max(np.abs(st.DZ - fs["DZ"])) <= 1e-15 * np.max(np.abs(fs["DZ"]))
        assert abs(st.Yle - fs["Yle"]).max() <= 1e-15 * max(abs(fs["Yle"]).max(), 1e-300)
        SSo = (fs["Yle"] + inc["A"].T @ (fs["invZ"] @ inc["A"])
               + 1j * w * ((inc["Gamma"] @ fs["invP"]) @ inc["Gamma"].T))
        assert abs(st.SS - SSo).max() <= 1e-14 * abs(SSo).max()
    rng = np.random.default_rng(8)
    S = 0.3 * (rng.standard_normal((3, 3, 4)) + 1j * rng.standard_normal((3, 3, 4)))
    S = 0.5 * (S + S.transpose(1, 0, 2))
    assert np.allclose(api.s2z_fft(S, 50.0), O.s2z(S, 50.0), rtol=1e-13, atol=0)
    assert np.allclose(api.s2y_fft(S, 50.0), O.s2y(S, 50.0), rtol=1e-13, atol=0)
