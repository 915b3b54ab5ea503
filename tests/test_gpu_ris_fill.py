"""GPU: the dense RIS fill on the device (peec_ris_fill: calcola_Lp.jl / calcola_P.jl)
against the oracle's restatement of the same case trees (oracle/fill_ref.c), and the RIS
solver running on device-filled matrices:

* every entry of the Lp blocks and of P within 64 eps of its sum of |terms| on seeded
  bodies that take every branch of both trees, the same non-finite entries;
* the centre distances equal numpy's;
* the frequency x port loop on the device-filled operator (quasi-static and retarded,
  the distances kept on the device) gives the S parameters of the host-filled one;
* calcola_Lp / calcola_P return the oracle's matrices."""
import numpy as np
import pytest

from oracle import ris_ref as RO
from solver_gb300 import configs, ris
from tests import ris_cases

pytestmark = pytest.mark.gpu

EPS = np.finfo(np.float64).eps


def _fill_op(vol, surf, mx, my, mz, esc, rcc=1):
    inc = ris._sizes_only(mx, my, mz, len(surf["S"]))
    return ris.DenseOperator.from_geometry(inc, vol, surf, esc, rcc)


def _close(dev, ref, scale):
    fin = np.isfinite(ref)
    assert np.array_equal(np.isfinite(dev), fin)
    err = np.abs(dev - ref)[fin]
    lim = 64 * EPS * scale[fin] + 1e-300
    assert np.all(err <= lim), float(np.max(err / lim))


@pytest.mark.parametrize("seed", [7, 8])
def test_device_fill_matches_the_oracle(seed):
    dims = (70, 50, 40, 90)
    vol, surf = ris_cases.random_bodies(seed, *dims)
    esc = {"Lp": 1e6, "P": 1e-12}
    Lr, Pr, sL, sP, bad = ris_cases.oracle_dense_fill(vol, surf, *dims[:3], esc["Lp"], esc["P"])
    op = _fill_op(vol, surf, *dims[:3], esc)
    try:
        Lp, P = op.dense_data()
        for k in ("Lp_x", "Lp_y", "Lp_z"):
            _close(Lp[k], Lr[k], sL[k])
        _close(P["P"], Pr["P"], sP)
        assert op.nonfinite == bad
        assert np.array_equal(op.diag_P, np.diag(P["P"]))
        assert np.array_equal(op.diag_Lp, np.concatenate([np.diag(Lp[k]) for k in
                                                          ("Lp_x", "Lp_y", "Lp_z")]))
    finally:
        op.close()


def test_device_distances_equal_numpy():
    dims = (30, 20, 10, 40)
    vol, surf = ris_cases.random_bodies(3, *dims)
    op = _fill_op(vol, surf, *dims[:3], {"Lp": 1.0, "P": 1.0}, rcc=2)
    try:
        Lp, P = op.dense_data()
        off = 0
        for k, n in zip(("Rx", "Ry", "Rz"), dims[:3]):
            c = np.asarray(vol["centri"])[off:off + n]
            d = c[:, None, :] - c[None, :, :]
            ref = np.sqrt(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])
            assert np.array_equal(Lp[k], ref)
            off += n
        c = np.asarray(surf["centri"])
        d = c[:, None, :] - c[None, :, :]
        ref = np.sqrt(d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])
        assert np.array_equal(P["R_cc"], ref)
    finally:
        op.close()


def test_calcola_functions_return_the_oracle_matrices():
    dims = (25, 15, 20, 30)
    vol, surf = ris_cases.random_bodies(11, *dims)
    esc = {"Lp": 1e6, "P": 1e-12}
    Lr, Pr, sL, sP, _ = ris_cases.oracle_dense_fill(vol, surf, *dims[:3], esc["Lp"], esc["P"])
    inc = {"mx": dims[0], "my": dims[1], "mz": dims[2]}
    Lp = ris.calcola_Lp(vol, inc, esc, 2)
    P = ris.calcola_P(surf, esc, 2)
    for k in ("Lp_x", "Lp_y", "Lp_z"):
        _close(Lp[k], Lr[k], sL[k])
    _close(P["P"], Pr["P"], sP)
    assert set(Lp) >= {"Rx", "Ry", "Rz"} and "R_cc" in P
    assert "Rx" not in ris.calcola_Lp(vol, inc, esc, 1)


CASES = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_16x12x8": lambda: configs.random_mixed((16, 12, 8), s=5e-5, p=0.35, seed=9,
                                                   nports=2, freqs=[1e8, 3e9], tol=1e-8),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    c = ris_cases.voxel_case(CASES[request.param]())
    vol, surf = ris_cases.ris_geometry(c)
    vol.update(ris_cases.volumi_of(c, seed=1))
    c["volumi"], c["superfici"] = vol, surf
    inc = c["inc"]
    Lr, Pr, _, _, bad = ris_cases.oracle_dense_fill(vol, surf, inc["mx"], inc["my"], inc["mz"],
                                                    c["esc"]["Lp"], c["esc"]["P"])
    assert bad == 0
    c["Lp_data"], c["P_data"] = Lr, Pr
    return c


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("QS_Rcc_FW", [1, 2])
def test_ris_solver_on_device_filled_matrices(case, QS_Rcc_FW):
    c = case
    freqs = [1e8, 1e9, 3e9]
    gs = {"Inner_Iter": 200, "tol": [1e-8] * len(freqs)}
    Lp, P = c["Lp_data"], c["P_data"]
    if QS_Rcc_FW == 2:
        Lp, P = dict(Lp), dict(P)
        for k, b in zip(("Rx", "Ry", "Rz", "R_cc"), (0, 1, 2, 3)):
            cc = np.asarray((c["volumi"]["centri"] if b < 3 else c["superfici"]["centri"]))
            inc = c["inc"]
            lo = (0, inc["mx"], inc["mx"] + inc["my"], 0)[b]
            n = (inc["mx"], inc["my"], inc["mz"], len(c["superfici"]["S"]))[b]
            d = cc[lo:lo + n, None, :] - cc[None, lo:lo + n, :]
            (Lp if b < 3 else P)[k] = np.sqrt((d ** 2).sum(-1))
    ref = RO.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], P, Lp, c["ports"], {}, gs,
                                   c["volumi"], True, QS_Rcc_FW, 50.0)
    op = ris.DenseOperator.from_geometry(c["inc"], c["volumi"], c["superfici"], c["esc"],
                                         QS_Rcc_FW)
    try:
        assert op.nonfinite == 0
        out = ris.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], None, None, c["ports"], {},
                                        gs, c["volumi"], True, QS_Rcc_FW, 50.0, op=op)
        assert all(r["flag"] == 0 for r in out["info"]), out["info"]
        for k in range(len(freqs)):
            assert _rel(out["S"][:, :, k], ref["S"][:, :, k]) < 1e-7, k
        if QS_Rcc_FW == 2:
            # back on the quasi-static blocks after the loop, and a second retarded run
            # takes the distances from the device again
            out2 = ris.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], None, None, c["ports"],
                                             {}, gs, c["volumi"], True, 2, 50.0, op=op)
            assert np.array_equal(out2["S"], out["S"])
    finally:
        op.close()


def test_device_fill_reproduces_the_reference_nan():
    """The point-surface form's 0/0 (a point in a surface's plane, on an edge's line) is NaN
    on the device as in the oracle, and counted."""
    from tests.test_oracle_ris_fill import _nan_case
    vol = _nan_case()
    surf = {"estremi_celle": np.zeros((0, 12)), "S": np.zeros(0)}
    op = _fill_op(vol, surf, 2, 0, 0, {"Lp": 1.0, "P": 1.0})
    try:
        Lp, _ = op.dense_data()
        assert np.isnan(Lp["Lp_x"][0, 1]) and np.isnan(Lp["Lp_x"][1, 0])
        assert np.isfinite(np.diag(Lp["Lp_x"])).all()
        assert op.nonfinite == 1
    finally:
        op.close()


def test_do_solving_ris_end_to_end(case):
    """doSolvingRis without its service parts: ports given by coordinates are mapped back to
    the mesh's nodes, the matrices filled on the device, the loop run; its S parameters
    match the oracle's loop on the oracle's matrices."""
    c = case
    n = c["inc"]["A"].shape[1]
    k = np.arange(n)
    nodi = np.stack([k * 1e-3, (k % 7) * 1e-3, np.zeros(n)], axis=1)  # distinct nodes
    pn = np.asarray(c["ports"]["port_nodes"]).reshape(-1, 2)
    freqs = [1e8, 1e9, 3e9]
    si = {"unit": "m", "frequencies": freqs, "lumped_elements": [],
          "ports": [{"inputElement": nodi[a].tolist(), "outputElement": nodi[b].tolist()}
                    for a, b in pn]}
    algo = {"innerIteration": 200, "outerIteration": 1, "convergenceThreshold": 1e-8}
    out = ris.do_solving_ris(c["inc"], c["volumi"], c["superfici"], nodi, c["esc"], si, algo, 1)
    gs = {"Inner_Iter": 200, "tol": [1e-8] * len(freqs)}
    ref = RO.iter_solver_QS_S_type(freqs, c["esc"], c["inc"], c["P_data"], c["Lp_data"],
                                   c["ports"], {}, gs, c["volumi"], True, 1, 50.0)
    assert all(r["flag"] == 0 for r in out["info"])
    for q in range(len(freqs)):
        assert _rel(out["S"][:, :, q], ref["S"][:, :, q]) < 1e-7, q
