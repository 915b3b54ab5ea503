"""GPU: the device-resident GMRES loop (peec_set_device_loop).

The Arnoldi iterations of peec_gmres and of the mixed solve's inner solves run in a CUDA
graph whose WHILE node repeats one iteration (operator application, orthogonalisation,
the FP64 scalar step with the Givens rotations) until the residual estimate reaches the
tolerance or the cycle is full. With the loop switched off the same kernels run one
iteration per host round trip. Both must give the same solution bit for bit, the same
flag, iteration counts and residual history, and the loop must really run on the device
(its graph launches and the iterations they ran are counted by the library)."""
import copy

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from solver_gb300 import configs, mesher
from solver_gb300.operator import GpuOperator

pytestmark = pytest.mark.gpu

CASES = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_24x20x12": lambda: configs.random_mixed((24, 20, 12), s=5e-5, p=0.35, seed=7,
                                                    nports=2, freqs=[1e8, 3e9], tol=1e-8),
}


@pytest.fixture(scope="module", params=sorted(CASES))
def case(request):
    req = CASES[request.param]()
    out, freqs, _settings, z0, grid = OM.parse_request(copy.deepcopy(req))
    esc, inc, cc, diag, exp, ports, le, _li, Zs = out
    pe = mesher.parse_request(copy.deepcopy(req))[0]
    op = GpuOperator(pe[1], pe[4], pe[3]["P"])
    op.set_rows(O.fill_rows(cc, esc, *grid))
    w = 2 * np.pi * freqs[-1] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    op.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
    tn = op.port_rhs(*ports["port_nodes"][0], esc["Is"])
    yield dict(op=op, tn=tn)
    op.close()


def _both(op, run):
    """run() with the device loop on, then off; the stats of the 'on' run."""
    op.set_device_loop(True)
    run()  # warm: the first iteration on fresh buffers runs eagerly
    s0 = op.device_loop_stats()
    a = run()
    s1 = op.device_loop_stats()
    op.set_device_loop(False)
    try:
        b = run()
        s2 = op.device_loop_stats()
    finally:
        op.set_device_loop(True)
    assert s2 == s1, "iterations ran in the graph with the device loop off"
    return a, b, (s1[0] - s0[0], s1[1] - s0[1])


def test_gmres_device_loop_matches_round_trips(case):
    op, tn = case["op"], case["tn"]
    a, b, (launches, iters) = _both(op, lambda: op.gmres(tn, None, 1e-8, 100))
    xa, fa, ra, ita, rva = a
    xb, fb, rb, itb, rvb = b
    assert (fa, list(ita)) == (fb, list(itb))
    assert np.array_equal(xa, xb)
    assert ra == rb and np.array_equal(rva, rvb)
    assert fa == 0
    # one graph launch runs every iteration up to the first convergence check
    assert launches >= 1 and iters >= 1
    assert iters >= ita[1] - launches


def test_restarted_gmres_device_loop_matches_round_trips(case):
    op, tn = case["op"], case["tn"]
    a, b, (launches, iters) = _both(op, lambda: op.gmres(tn, None, 1e-10, 4, restarted=True,
                                                         restart=5))
    assert (a[1], list(a[3])) == (b[1], list(b[3]))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[4], b[4])
    assert launches >= 1 and iters >= 1


def test_mixed_solve_device_loop_matches_round_trips(case):
    op, tn = case["op"], case["tn"]
    a, b, (launches, iters) = _both(op, lambda: op.solve_mixed(tn, None, 1e-8))
    assert a[1:] == b[1:]
    assert np.array_equal(a[0], b[0])
    assert a[1] == 0
    assert launches >= 1 and iters >= a[4] - launches


def test_device_loop_rejects_bad_switch(case):
    from solver_gb300 import _lib
    op = case["op"]
    with pytest.raises(_lib.PeecError):
        _lib.check(op.h, op.L.peec_set_device_loop(op.h, 2))
