"""CPU: the oracle's restatement of the retarded (Rcc, QS_Rcc_FW == 2) operator set-up
(oracle/rcc_ref.py, the Rcc dispatch in oracle/fill_ref.c) held to what the formulas fix:

* on cells whose bodies never collapse to lines (cubic voxels, distances under 200 edges)
  the Rcc path's Lp rows (compute_Lp_Voxels_QS) equal the QS fill's (compute_Lp_Voxels)
  entry for entry; on elongated cells they differ exactly at the collinear line-line
  entries, where compute_Lp_Voxels_QS.jl:501-520 keeps its own integ_line_line_sp, and
  there they equal that formula evaluated directly;
* the Rcc P rows are filled with the block indices as face types
  (compute_rows_Rcc_P.jl:47-52): its (1,1) block is the QS P11 row, and its (2,2) block,
  on the x-face lattice, is the y-face row of the QS fill at the same displacements;
* the centre distances are the lattice distances; at zero frequency the Rcc spectra are
  those of the quasi-static parts;
* the Rcc sweep tends to the QS sweep over the same rows as the frequency falls, the
  difference in proportion to beta R (its first-order term)."""
import copy
import math

import numpy as np
import pytest

from oracle import mesher_ref as OM
from oracle import peec_oracle as O
from oracle import rcc_ref as RR
from solver_gb300 import configs


def _lattice(n, s, axis_steps=None):
    """centres of an (nx, ny, nz) lattice of cell size s, x fastest"""
    nx, ny, nz = n
    i, j, k = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    c = np.stack([i.ravel(order="F") * s[0], j.ravel(order="F") * s[1],
                  k.ravel(order="F") * s[2]], axis=1) + np.array(s) / 2
    return c


@pytest.mark.parametrize("dc", [1, 2, 3])
def test_rcc_lp_rows_equal_qs_rows_on_cubic_cells(dc):
    s = (1e-4, 1e-4, 1e-4)
    c = _lattice((9, 7, 5), s)
    qs = RR.lp_row_qs(dc, c, *s)
    ref = O.lp_row(dc, c, *s)
    assert np.array_equal(qs, ref)


def _ll_sp_qs(x1v, x2v):
    """integ_line_line_sp of compute_Lp_Voxels_QS.jl:501-520, evaluated directly"""
    def lgc(v):
        return math.log(abs(v)) if v != 0 else -math.inf
    sol = 0.0
    for c1 in range(2):
        for c2 in range(2):
            x1, x2 = x1v[c1], x2v[c2]
            R = math.sqrt((x1 - x2) ** 2)
            try:
                t = (x1 - x2) / R * (x1 - x2 * lgc(x2 - x1) + x1 * lgc(x1 - x2))
            except ZeroDivisionError:
                t = math.nan
            if not math.isfinite(t):
                t = 0.0
            sol += (-1) ** (c1 + c2 + 1) * t
    return sol


def test_rcc_lp_rows_differ_only_at_collinear_lines():
    # cells 100x longer in x than across: far along the x axis the two voxels collapse to
    # collinear lines (y and z suppressed, x kept), the only Lp case in which the two
    # dispatches apply different formulas (equal-size boxes collapse alike, so the
    # surface-line, surface-volume and orthogonal cases never arise in an Lp row)
    s = (1e-3, 1e-5, 1.3e-5)
    n = (40, 3, 3)
    c = _lattice(n, s)
    qs = RR.lp_row_qs(1, c, *s)
    ref = O.lp_row(1, c, *s)
    diff = np.nonzero(qs != ref)[0]
    assert diff.size > 0
    i = diff % n[0]
    j = (diff // n[0]) % n[1]
    k = diff // (n[0] * n[1])
    assert np.all(j == 0) and np.all(k == 0)  # on the source's own line
    r14 = lambda v: round(v * 1e14) / 1e14
    S = s[1] * s[2] * s[1] * s[2]
    x0 = c[0, 0]
    for p in diff:
        xv1 = [r14(x0 - s[0] / 2), r14(x0 + s[0] / 2)]
        xv2 = [r14(c[p, 0] - s[0] / 2), r14(c[p, 0] + s[0] / 2)]
        # line-line weight b1 c1 b2 c2 (compute_Lp_Voxels_QS.jl:218-219)
        w = (r14(c[0, 1] + s[1] / 2) - r14(c[0, 1] - s[1] / 2)) ** 2 * \
            (r14(c[0, 2] + s[2] / 2) - r14(c[0, 2] - s[2] / 2)) ** 2
        want = 1e-7 / S * (w * _ll_sp_qs(xv1, xv2))
        assert qs[p] == pytest.approx(want, rel=1e-12, abs=1e-30)


def test_rcc_lp_rows_raise_where_the_reference_does():
    # equal cross-section edges: the rounded box extents of two cells can order them
    # differently, so one box collapses y and the other z, and the entry lands in the
    # orthogonal surface-surface call that Julia cannot apply
    s = (1e-3, 1e-5, 1e-5)
    with pytest.raises(RR.ReferenceRaises):
        RR.lp_row_qs(1, _lattice((40, 3, 3), s), *s)


def test_rcc_p_rows_take_the_block_indices_as_face_types():
    req = configs.crossbar_20x20x4()
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = \
        OM.parse_request(copy.deepcopy(req))
    Nx, Ny, Nz = grid
    rows = RR.compute_rows_Rcc_P(cc)
    qs_fill = O.fill_rows(cc, {"Lp": 1.0, "P": 1.0}, Nx, Ny, Nz)
    assert np.array_equal(rows["p12_se"][0], qs_fill["p12_se"])
    # (2,2) on the x-face lattice p34_se (Nx+1, Ny, Nz) = y faces at the same displacement
    # as the QS (1,1) row on p12_se (Nx, Ny+1, Nz)
    a = rows["p34_se"][0].reshape((Nx + 1, Ny, Nz), order="F")[:Nx, :Ny, :]
    b = qs_fill["p12_se"].reshape((Nx, Ny + 1, Nz), order="F")[:Nx, :Ny, :]
    # the same integrals at other absolute coordinates: the closed forms cancel ~R^5 terms
    # down to ~s^6/R, so far entries agree to rounding of that cancellation (5e-10 seen)
    assert np.allclose(a, b, rtol=1e-8, atol=0)
    # and it is not the QS fill's x-face row (the two couple differently oriented faces)
    assert not np.allclose(rows["p34_se"][0], qs_fill["p34_se"], rtol=1e-3)


def test_rcc_distances():
    s = (1e-4, 2e-4, 5e-5)
    c = _lattice((4, 3, 2), s)
    R = RR.compute_Voxels_Rcc(c[0], c)
    want = np.sqrt(((c - c[0]) ** 2).sum(axis=1))
    assert np.allclose(R, want, rtol=1e-15, atol=1e-20)
    # face distances: y- face of the source to y+ faces is the centre distance shifted by sy
    Rf = RR.compute_P_vox_Rcc(c[0], c, *s, 1, 2)
    d = c - c[0]
    d[:, 1] += s[1]
    assert np.allclose(Rf, np.sqrt((d ** 2).sum(axis=1)), rtol=1e-14)


def test_rcc_spectra_at_zero_frequency_are_the_qs_spectra():
    req = configs.crossbar_20x20x4()
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = \
        OM.parse_request(copy.deepcopy(req))
    rL, rP = RR.compute_rows_Rcc_Lp(cc), RR.compute_rows_Rcc_P(cc)
    FL = RR.compute_Circulant_Lp_Rcc(rL, esc, 0.0, *grid)
    FP = RR.compute_Circulant_P_sup_Rcc(rP, esc, 0.0, *grid)
    QP, QL = O.spectra_from_rows(RR.rcc_rows_escaled(rL, rP, esc), *grid)
    for c in range(3):
        assert np.array_equal(FL[c], QL[c])
    for (i, j), _, _, _ in RR.RCC_P_ROWS:
        assert np.array_equal(FP[i][j], QP[i][j])


def test_reference_rcc_does_not_converge_on_mixed_grids():
    """On a copper / dielectric grid the reference's Rcc P rows (the block indices as face
    types) leave GMRES far from convergence, where the same retarded operator with the QS
    fill's face types converges: a property of the reference, kept by the restatement."""
    req = configs.random_mixed((24, 20, 12), s=5e-5, p=0.35, seed=7, nports=2, freqs=[1e8],
                               tol=1e-8)
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = \
        OM.parse_request(copy.deepcopy(req))
    rL, rP = RR.compute_rows_Rcc_Lp(cc), RR.compute_rows_Rcc_P(cc)
    st = {"Inner_Iter": 100, "tol": np.full(1, 1e-8)}
    as_ref = RR.FFT_solver_Rcc(freqs, esc, inc, rP, rL, diag, ports, z0, le, exp, st, Zs, grid)
    assert all(r["flag"] == 1 and r["relres"] > 1e-3 for r in as_ref["info"])
    qs_rows = O.fill_rows(cc, esc, *grid)
    rP_qs = {k: (qs_rows[k] / esc["P"], rP[k][1]) for k in rP}
    fixed = RR.FFT_solver_Rcc(freqs, esc, inc, rP_qs, rL, diag, ports, z0, le, exp, st, Zs, grid)
    assert all(r["flag"] == 0 and len(r["resvec"]) - 1 < 50 for r in fixed["info"])


def test_rcc_sweep_tends_to_the_qs_sweep_at_low_frequency():
    req = configs.crossbar_20x20x4()
    (esc, inc, cc, diag, exp, ports, le, li, Zs), freqs, settings, z0, grid = \
        OM.parse_request(copy.deepcopy(req))
    rL, rP = RR.compute_rows_Rcc_Lp(cc), RR.compute_rows_Rcc_P(cc)
    QP, QL = O.spectra_from_rows(RR.rcc_rows_escaled(rL, rP, esc), *grid)
    st = {"Inner_Iter": 100, "tol": np.full(2, 1e-10)}
    f = np.array([1e6, 1e9])
    rcc = RR.FFT_solver_Rcc(f, esc, inc, rP, rL, diag, ports, z0, le, exp, st, Zs, grid)
    qs = O.FFT_solver_QS_S_type(f, esc, inc, QP, QL, diag, ports, z0, le, exp, st, Zs)
    rel = [np.max(np.abs(rcc["Z"][..., k] - qs["Z"][..., k])) / np.max(np.abs(qs["Z"][..., k]))
           for k in range(2)]
    # exp(-i beta R) = 1 - i beta R + ...: the first-order term survives in the operator
    # (Lp R and P R are nearly constant, the radiation part), so the impedances differ in
    # proportion to the frequency: beta R ~ 6e-5 at 1 MHz over the 2 mm grid
    assert rel[0] < 1e-6, rel
    assert 300 < rel[1] / rel[0] < 3000, rel
