"""GPU: failure detection without a GPU fault.

* A dependency wait of the triangular-solve kernel that nothing will satisfy gives up
  after its poll limit, the host reads the error word (PEEC_ERR_TIMEOUT), and the
  context keeps working (peec_check_wait_limit).
* A stop flag set on the host cancels a solve between Krylov steps (flag 99, the C ABI
  returning PEEC_ERR_CANCELLED), as the reference's is_stop_requested polling does
  (gmres_custom.jl:96-99); the frequency sweep then returns None.
* A NaN planted in the right-hand side ends the solve at its iteration limit with a
  non-converged flag; the next solve on the same context converges."""
import ctypes

import numpy as np
import pytest

from oracle import peec_oracle as O
from solver_gb300 import _lib, api, configs, mesher
from solver_gb300.operator import GpuOperator

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def crossbar():
    out, freqs, settings, z0, grid = mesher.parse_request(configs.crossbar_20x20x4())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    op = GpuOperator(inc, exp, diag["P"])
    op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"])
    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    op.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
    n1, n2 = np.asarray(ports["port_nodes"]).reshape(-1, 2)[0]
    tn = op.port_rhs(n1, n2, esc["Is"])
    yield dict(op=op, tn=tn, esc=esc, inc=inc, diag=diag, exp=exp, ports=ports, le=le, Zs=Zs,
               z0=z0, freqs=freqs, settings=settings)
    op.close()


def _converges(c):
    V, flag, relres, it, rv = c["op"].gmres(c["tn"], None, 1e-8, 100)
    return flag == 0 and relres <= 1e-8


def test_wait_limit_returns_timeout_and_context_stays_usable(crossbar):
    with pytest.raises(_lib.PeecError) as e:
        _lib.check(crossbar["op"].h, crossbar["op"].L.peec_check_wait_limit(crossbar["op"].h))
    assert e.value.code == -4  # PEEC_ERR_TIMEOUT
    assert _converges(crossbar)


def test_stop_flag_cancels_between_krylov_steps(crossbar):
    c = crossbar
    stop = ctypes.c_int(1)
    c["op"].set_stop_flag(stop)
    try:
        assert c["op"].gmres(c["tn"], None, 1e-8, 100)[1] == 99
        assert c["op"].solve_mixed(c["tn"], None, 1e-8)[1] == 99
        c["exp"]["gpu_ctx"] = c["op"]
        h = api.CirculantSpectra(c["op"])
        res = api.FFT_solver_QS_S_type(c["freqs"], c["esc"], c["inc"], h, h, c["diag"],
                                       c["ports"], c["z0"], c["le"], c["exp"],
                                       {"Inner_Iter": 100, "tol": np.full(len(c["freqs"]), 1e-6)},
                                       c["Zs"], stop_flag=stop)
        assert res is None
    finally:
        stop.value = 0
        c["op"].set_stop_flag(None)
        c["exp"].pop("gpu_ctx", None)
    assert _converges(c)


def test_nan_rhs_ends_without_converging(crossbar):
    c = crossbar
    b = np.array(c["tn"])
    b[len(b) // 2] = np.nan
    V, flag, relres, it, rv = c["op"].gmres(b, None, 1e-8, 30)
    assert flag != 0 or not np.isfinite(relres)
    x, fl, rel, outer, inner = c["op"].solve_mixed(b, None, 1e-8, inner_maxit=30, max_outer=2)
    assert fl != 0 or not np.isfinite(rel)
    assert _converges(c)
