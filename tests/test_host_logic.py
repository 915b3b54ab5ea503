"""CPU: host-side logic of the sweep API with stand-in contexts (no GPU).

* PortLanes.sweep gives every port its own lane (port c on lane c % lanes), walks each
  lane through the whole frequency sequence in order with warm starts from that lane's
  own previous solutions, releases a frequency state once every lane has set it (and
  not while a later position still needs it), and stops on the stop flag.
* dump_json_data writes the reference's results layout
  (format_input_output_solver_functions.jl:1-31).
* do_solving_fft refuses the solver types it does not implement."""
import ctypes
import json
import threading

import numpy as np
import pytest

from solver_gb300 import api


class FakeOp:
    """Stands in for a GpuOperator: records the calls; the 'solution' of port c at
    frequency w is x0 + (w + c), so warm starts are visible in the results."""

    def __init__(self, name, log):
        self.name, self.log, self.w = name, log, None

    def set_frequency(self, w, DZ, Yle, lu, key=None):
        self.w = w
        self.log.append((self.name, "set", w))

    def port_rhs(self, n1, n2, Is):
        return np.array([n1, n2, Is], dtype=np.complex128)

    def solve_mixed(self, tn, x0, tol, **kw):
        self.log.append((self.name, "solve", self.w, int(tn[0].real)))
        return x0 + (self.w + tn[0].real), 0, tol / 2, 1, 5


    def gmres(self, tn, x0, tol, maxit):
        self.log.append((self.name, "gmres", self.w, int(tn[0].real), maxit))
        return x0 + (self.w + tn[0].real), 0, tol / 2, [1, 7], np.zeros(8)


class FakeLanes(api.PortLanes):
    def __init__(self, nlanes, log):
        from concurrent.futures import ThreadPoolExecutor
        self.ops = [FakeOp(i, log) for i in range(nlanes)]
        self._pool = ThreadPoolExecutor(max_workers=nlanes)

    def close(self):
        self._pool.shutdown(wait=True)


class State:
    def __init__(self, w):
        self.w, self.DZ, self.Yle, self.lu = w, None, None, None


@pytest.mark.parametrize("nlanes,nports", [(2, 4), (3, 2), (1, 3)])
def test_lanes_sweep_schedule_warm_starts_and_release(nlanes, nports):
    log, released, recs = [], [], []
    lock = threading.Lock()
    lanes = FakeLanes(nlanes, log)
    seq = [0, 1, 2, 1]  # a repeated key must not be released before its last use
    pn = np.array([[10 * c, 10 * c + 1] for c in range(nports)])
    V = np.zeros((3, nports), dtype=np.complex128)

    def record(pos, k, c, Vc, flag, relres, outer, inner):
        with lock:
            recs.append((pos, k, c, Vc.copy()))

    def rel(k):
        with lock:
            released.append(k)

    try:
        ok = lanes.sweep(seq, lambda k, pos: State(float(k)), rel, pn, 1.0, V,
                         lambda k: 1e-8, {}, record)
    finally:
        lanes.close()
    assert ok
    assert len(recs) == len(seq) * nports
    # each lane walks the sequence in order and solves only its own ports
    for lane in range(min(nlanes, nports)):
        mine = [e for e in log if e[0] == lane]
        sets = [e[2] for e in mine if e[1] == "set"]
        assert sets == [float(k) for k in seq]
        solved = {e[3] // 10 for e in mine if e[1] == "solve"}
        assert solved == {c for c in range(nports) if c % nlanes == lane}
    # warm starts: port c's final solution accumulates (w + 10c) over the sequence
    for c in range(nports):
        assert V[0, c] == sum(float(k) + 10 * c for k in seq)
    # every key released exactly once, after its last position
    assert sorted(released) == sorted(set(seq))


def test_lanes_sweep_stops_on_flag():
    log = []
    lanes = FakeLanes(2, log)
    stop = ctypes.c_int(1)
    try:
        ok = lanes.sweep([0, 1], lambda k, pos: State(float(k)), lambda k: None,
                         np.array([[0, 1], [2, 3]]), 1.0, np.zeros((3, 2), complex),
                         lambda k: 1e-8, {}, lambda *a: None, stop_flag=stop)
    finally:
        lanes.close()
    assert ok is False and log == []


def test_dump_json_data_layout():
    Z = np.arange(2 * 2 * 3).reshape(2, 2, 3) * (1 + 1j)
    out = api.dump_json_data(Z, Z * 2, Z * 3, 2, "job7", partial=True, freqIndex=4)
    assert (out["id"], out["partial"], out["freqIndex"], out["isStopped"]) == ("job7", True, 4, False)
    mz = json.loads(out["matrices"]["matrix_Z"])
    assert len(mz) == 4  # port pairs, i outer, j inner
    for idx, (i, j) in enumerate([(0, 0), (0, 1), (1, 0), (1, 1)]):
        assert mz[idx] == [[[float(v.real), float(v.imag)] for v in Z[i, j, :]]]
    assert json.loads(out["matrices"]["matrix_S"])[1][0][2] == [float((Z[0, 1, 2] * 2).real),
                                                                float((Z[0, 1, 2] * 2).imag)]


def test_do_solving_fft_rejects_other_solver_types():
    # 1 (quasi-static) and 2 (Rcc) are built; the reference comments out Taylor (3)
    for t in (0, 3):
        with pytest.raises(NotImplementedError):
            api.do_solving_fft({"solverType": t})


def test_operator_rejects_vectors_of_the_wrong_length():
    """The C library reads N entries from every vector it is given, so the host wrapper
    checks lengths before any call (no GPU needed: the check comes first)."""
    import numpy as np
    import pytest
    from solver_gb300.operator import GpuOperator

    op = GpuOperator.__new__(GpuOperator)
    op.N = 10
    with pytest.raises(ValueError):
        op._vectors(np.zeros(9), None)
    with pytest.raises(ValueError):
        op._vectors(np.zeros(10), np.zeros(11))
    b, x = op._vectors(np.ones(10), None)
    assert b.dtype == np.complex128 and x.shape == (10,) and not x.any()


def test_lanes_sweep_failure_in_one_lane_stops_the_others():
    """A lane whose solve raises (a failed library call, say) stops the other lanes before
    their next frequency or port, and the exception reaches the caller."""
    log = []
    lanes = FakeLanes(2, log)

    def boom(tn, x0, tol, **kw):
        raise RuntimeError("lane 0 failed")
    lanes.ops[0].solve_mixed = boom
    seq = list(range(50))
    try:
        with pytest.raises(RuntimeError, match="lane 0 failed"):
            lanes.sweep(seq, lambda k, pos: State(float(k)), lambda k: None,
                        np.array([[0, 1], [2, 3]]), 1.0, np.zeros((3, 2), complex),
                        lambda k: 1e-8, {}, lambda *a: None)
    finally:
        lanes.close()
    solves = [e for e in log if e[1] == "solve"]
    assert len(solves) < len(seq)  # lane 1 did not run the whole sweep


def test_request_parser_rejects_inconsistent_grids():
    """Malformed solve requests fail with a message before the mesher runs: material grids
    of different shapes, grids that disagree with n_cells, an empty geometry, and a grid
    whose material is not listed."""
    import copy

    from solver_gb300 import configs, mesher
    base = configs.crossbar_20x20x4()
    mesher.parse_request(copy.deepcopy(base))  # the well-formed request parses

    r = copy.deepcopy(base)
    r["mesherOutput"]["n_cells"]["n_cells_x"] = 21
    with pytest.raises(ValueError, match="n_cells"):
        mesher.parse_request(r)

    r = copy.deepcopy(base)
    r["mesherOutput"]["mesher_matrices"]["copper"] = [
        [[False] * 4 for _ in range(20)] for _ in range(20)]
    with pytest.raises(ValueError, match="no occupied voxel"):
        mesher.parse_request(r)

    r = copy.deepcopy(base)
    r["mesherOutput"]["mesher_matrices"]["air"] = [[[False] * 3 for _ in range(20)]
                                                   for _ in range(20)]
    with pytest.raises(ValueError, match="one 3-D shape"):
        mesher.parse_request(r)

    r = copy.deepcopy(base)
    r["solverInput"]["materials"][0]["name"] = "gold"
    with pytest.raises(ValueError, match="lacks"):
        mesher.parse_request(r)


def test_lanes_sweep_fp64_mode_runs_the_reference_gmres():
    """mode="fp64": every port solve is the FP64 GMRES (peec_gmres) with the given maxit,
    warm started along the sequence like the mixed sweep; record gets its iterations."""
    log, recs = [], []
    lanes = FakeLanes(2, log)
    pn = np.array([[0, 1], [10, 11], [20, 21]])
    V = np.zeros((1, 3), dtype=np.complex128)
    ok = lanes.sweep([0, 1], lambda k, pos: State(float(k + 1)), lambda k: None, pn, 1.0, V,
                     lambda k: 1e-8, {"maxit": 37},
                     lambda pos, k, c, V_, flag, relres, outer, inner: recs.append((pos, c, inner)),
                     mode="fp64")
    lanes.close()
    assert ok
    assert sorted(recs) == [(0, 0, 7), (0, 1, 7), (0, 2, 7), (1, 0, 7), (1, 1, 7), (1, 2, 7)]
    assert all(e[1] in ("set", "gmres") for e in log)
    assert all(e[4] == 37 for e in log if e[1] == "gmres")
    # warm starts: port c's final value is the sum of its two solves' increments
    assert np.allclose(V[0], [(1 + 0) + (2 + 0), (1 + 10) + (2 + 10), (1 + 20) + (2 + 20)])
    with pytest.raises(ValueError):
        lanes.sweep([0], lambda k, pos: State(1.0), lambda k: None, pn, 1.0, V, lambda k: 1e-8,
                    {}, lambda *a: None, mode="fp32")


def test_install_state_routes_device_formed_states():
    """A DeviceFrequencyState goes through set_frequency_device; the context's edge data is
    uploaded once per source (the diagonals and Zs objects it came from) and again when
    the source changes; host states with device_lu keep the refactorisation path."""
    import scipy.sparse as sp
    from solver_gb300.frequency import DeviceFrequencyState

    calls = []

    class Op:
        def set_edge_state(self, diag, zs, esc):
            calls.append(("edge", id(diag)))
            self._edge_state = True

        def set_frequency_device(self, w, Yle):
            calls.append(("device", w))

        def set_frequency_refactor(self, w, DZ, Yle):
            calls.append(("refactor", w))

    esc = {"freq": 1.0, "Yle": 1.0}
    ports = {"port_nodes": np.array([[0, 1]])}
    d1, z1, d2 = {"R": 1}, {"Zs": 1}, {"R": 2}
    op = Op()
    for w, edge in ((1.0, (d1, z1)), (2.0, (d1, z1)), (3.0, (d2, z1))):
        api.install_state(op, DeviceFrequencyState(w, esc, 4, {}, ports, 50.0, edge), True)
    assert calls == [("edge", id(d1)), ("device", 1.0), ("device", 2.0), ("edge", id(d2)),
                     ("device", 3.0)]
    st = State(4.0)
    st.Yle = sp.csr_matrix((4, 4))
    api.install_state(op, st, True)
    assert calls[-1] == ("refactor", 4.0)
    # a device-formed state without edge data on a context that has none is refused
    with pytest.raises(ValueError):
        api.install_state(Op(), DeviceFrequencyState(5.0, esc, 4, {}, ports, 50.0), True)
