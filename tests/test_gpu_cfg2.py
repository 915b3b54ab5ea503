"""GPU parity at the benchmark geometry: 128x128x64 voxels of 5e-5 m, Bernoulli(0.3)
occupancy (seed 2), copper / dielectric 50/50, 4 ports, first frequency 10 MHz.

Shared fill (the oracle's rows uploaded to the GPU context) and shared LU factors, as in
test_gpu_parity.py; the oracle side takes its topology from the oracle's mesher
restatement, the GPU side from the product mesher. Checks:
* one FP64 operator application against the oracle's (reference 2N extents, three LU
  solves), within max(1e-10, 20x the problem's own rounding noise: the distance between
  two algebraically identical oracle forms);
* one port's FP64 GMRES from a zero initial guess at relative residual 1e-8 against the
  oracle's gmres_custom: the same flag and iteration count, the port's impedance entry
  within 1e-10, the whole solution within max(1e-10, 20x the oracle's own distance
  between two algebraically identical preconditioner forms: 30 iterations at 750K
  unknowns put that floor near 1e-11);
* the port impedances of the mixed-precision solve (FP32 convolutions, float-float
  residuals, 1e-8) against FP64 GMRES toward 1e-12 on the GPU at the same frequency (it
  stagnates between 3e-10 and 1.2e-9, the FP64 operator's rounding floor at this size and
  frequency): <= 1e-7.
The oracle runs its FFTs on all host cores; the whole file takes about three minutes."""
import copy
import os

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from solver_gb300 import configs, mesher
from solver_gb300.operator import GpuOperator

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.fixture(scope="module")
def big():
    O.FFT_WORKERS = os.cpu_count() or 1
    req = configs.random_128x128x64()
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = \
        OM.parse_request(copy.deepcopy(req))
    prod = mesher.parse_request(copy.deepcopy(req))[0]
    assert grid == (128, 128, 64)
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    w = 2 * np.pi * freqs[0] * esc["freq"]
    fs = O.frequency_setup(w, esc, inc, diag, Zs, le, ports, z0)
    op = GpuOperator(prod[1], prod[4], prod[3]["P"])
    op.set_rows(rows)
    op.set_frequency(w, fs["DZ"], fs["Yle"], fs["lu"])
    mv = lambda x: O.ComputeMatrixVectorFTT(x, w, inc, FFTCP, FFTCLp, fs["DZ"], fs["Yle"], exp,
                                            fs["invZ"], fs["invP"], fs["F"])
    yield dict(op=op, mv=mv, w=w, fs=fs, inc=inc, esc=esc, ports=ports, z0=z0,
               FFTCP=FFTCP, FFTCLp=FFTCLp, exp=exp)
    op.close()
    O.FFT_WORKERS = None


def test_cfg2_matvec_fp64(big):
    c = big
    rng = np.random.default_rng(21)
    x = rng.standard_normal(c["op"].N) + 1j * rng.standard_normal(c["op"].N)
    y_ref = c["mv"](x)
    # noise floor: the single-solve form of the preconditioner (exact algebra) against the
    # reference's three-solve form, both in the oracle
    noise = _rel(_single_solve_mv(c)(x), y_ref)
    err = _rel(c["op"].matvec(x, 0), y_ref)
    assert err < max(1e-10, 20 * noise), (err, noise)


def _single_solve_mv(c):
    """The oracle operator with the single-solve form of the preconditioner (exact algebra,
    other rounding)."""
    saved = O.precond_3_3_vector

    def single(F, invZ, invP, A_, G_, w_, X1, X2, X3):
        Mv = F(A_.T @ (invZ @ X1) - 1j * w_ * (G_ @ (invP @ X2)) + X3)
        return np.concatenate([invZ @ (X1 - A_ @ Mv), invP @ (X2 + G_.T @ Mv), Mv])

    def mv(x):
        O.precond_3_3_vector = single
        try:
            return c["mv"](x)
        finally:
            O.precond_3_3_vector = saved
    return mv


def test_cfg2_port_gmres_fp64(big):
    """Same flag and iteration count; the port's impedance entry (its voltage across the
    port nodes) within 1e-10; the whole solution within max(1e-10, 20x the distance between
    the oracle's solutions with two algebraically identical preconditioner forms)."""
    c = big
    pn = np.asarray(c["ports"]["port_nodes"], dtype=np.int64)
    op = c["op"]
    tn = op.port_rhs(pn[0, 0], pn[0, 1], c["esc"]["Is"])
    xg, flag, relres, it, rv = op.gmres(tn, None, 1e-8, 100)
    xo, fo, ro, ito, rvo = O.gmres_custom(np.asarray(tn), False, 1e-8, 100, None, c["mv"])
    assert flag == fo == 0
    assert list(it) == list(ito), (it, ito)
    k = op.m + op.ns
    vg = xg[k + pn[0, 0]] - xg[k + pn[0, 1]]
    vo = xo[k + pn[0, 0]] - xo[k + pn[0, 1]]
    assert abs(vg - vo) / abs(vo) < 1e-10
    xa, fa, ra, ita, rva = O.gmres_custom(np.asarray(tn), False, 1e-8, 100, None,
                                          _single_solve_mv(c))
    noise = _rel(xa, xo)
    err = _rel(xg, xo)
    assert err < max(1e-10, 20 * noise), (err, noise)


def test_cfg2_mixed_impedance_vs_fp64_1e12(big):
    c = big
    op = c["op"]
    pn = np.asarray(c["ports"]["port_nodes"], dtype=np.int64)
    m, ns = op.m, op.ns
    npt = pn.shape[0]

    def zmat(solve):
        S = np.zeros((npt, npt), dtype=np.complex128)
        for c1 in range(npt):
            tn = op.port_rhs(pn[c1, 0], pn[c1, 1], c["esc"]["Is"])
            V = solve(tn)
            for c2 in range(npt):
                val = 2 * (V[m + ns + pn[c2, 0]] - V[m + ns + pn[c2, 1]])
                S[c1, c2] = (val - c["z0"]) / c["z0"] if c1 == c2 else val / c["z0"]
        I = np.eye(npt)
        return c["z0"] * np.linalg.solve(I - S, I + S)

    def fp64(tn):
        # at 750K unknowns 1e-12 is below the FP64 operator's rounding floor at 10 MHz: a
        # solve may end in stagnation (flag 3) at its smallest residual (3.4e-10 to 1.2e-9
        # measured over the four ports), which must still be a quarter of the tolerance of
        # the solve it checks
        V, flag, relres, it, rv = op.gmres(tn, None, 1e-12, 400)
        assert flag in (0, 3) and relres <= 2.5e-9, (flag, relres)
        return V

    def mixed(tn):
        V, flag, relres, outer, inner = op.solve_mixed(tn, None, 1e-8)
        assert flag == 0 and relres <= 1e-8
        return V
    Zref = zmat(fp64)
    Zmx = zmat(mixed)
    assert _rel(Zmx, Zref) <= 1e-7
