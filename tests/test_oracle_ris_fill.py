"""CPU: the oracle's dense RIS fill (oracle/fill_ref.c: calcola_Lp / calcola_P with the
Song_*_Ivana_strategy case trees), pinned by independent closed forms and quadrature.

* Compute_Lp_Self (the FastHenry bar formula) equals the six-fold volume integral of the
  same bar (the 64-term closed form) in long double.
* The P self term of a rectangle equals a numerical quadrature of its area integral.
* Far apart, every entry tends to the point-point value; every suppressed (collapsed-
  dimension) form of both trees lies within 0.5 (size / R)^2 of it.
* The double restatement agrees with the long double one within 64 eps of each entry's
  sum of |terms| on seeded bodies that take every branch.
* On a voxel geometry written as RIS bodies the dense fill gives the voxel path's dense
  blocks (an independent fill through the circulant rows)."""
import ctypes

import numpy as np
import pytest

from solver_gb300 import configs
from tests import ris_cases

EPS = np.finfo(np.float64).eps


def _lib():
    from oracle import build
    L = ctypes.CDLL(str(build.build()))
    dp = ctypes.POINTER(ctypes.c_double)
    for sfx in ("_d", "_ld"):
        f = getattr(L, "oracle_ris_lp_self" + sfx)
        f.restype = ctypes.c_double
        f.argtypes = [dp, ctypes.c_int, dp]
    return L, dp


@pytest.mark.parametrize("lwt", [(1e-3, 1e-3, 1e-3), (2e-3, 5e-4, 1e-4), (1e-4, 3e-3, 2e-4),
                                 (5e-3, 5e-5, 5e-5)])
def test_self_term_is_the_volume_integral(lwt):
    l, W, T = lwt
    for d in (1, 2, 3):
        ext = [W, W, W]
        ext[d - 1] = l
        t = [q for q in range(3) if q != d - 1]
        ext[t[0]], ext[t[1]] = (T, W) if d == 1 else ((T, W) if d == 2 else (W, T))
        lo, hi = np.zeros(3), np.array(ext)
        vol = {"coordinate": np.array([ris_cases._brick24(lo, hi)] * 2),
               "S": np.array([W * T] * 2)}
        counts = [0, 0, 0]
        counts[d - 1] = 2
        Lp, _, _, _, bad = ris_cases.oracle_dense_fill(
            vol, {"estremi_celle": np.zeros((0, 12)), "S": np.zeros(0)}, *counts, ld=True)
        M = Lp[("Lp_x", "Lp_y", "Lp_z")[d - 1]]
        assert bad == 0
        # the off-diagonal entry of two coincident bars is the full closed form
        assert abs(M[0, 1] - M[0, 0]) <= 1e-12 * M[0, 0]


def _rect_self(a, b):
    """4 int_0^a int_0^b (a-u)(b-v) / sqrt(u^2+v^2) dv du (the area integral of 1/R over
    an a x b rectangle), by quadrature."""
    from scipy import integrate
    f = lambda v, u: (a - u) * (b - v) / np.hypot(u, v)
    val, err = integrate.dblquad(f, 0, a, 0, b, epsabs=0, epsrel=1e-12)
    return 4 * val


@pytest.mark.parametrize("ab", [(1e-3, 1e-3), (2e-3, 5e-4), (1e-4, 7e-4)])
def test_p_self_term_is_the_area_integral(ab):
    a, b = ab
    for nrm in range(3):
        lo = np.zeros(3)
        hi = np.zeros(3)
        t = [q for q in range(3) if q != nrm]
        hi[t[0]], hi[t[1]] = a, b
        surf = {"estremi_celle": np.array([ris_cases._rect12(lo.tolist(), hi.tolist())]),
                "S": np.array([a * b])}
        _, P, _, _, bad = ris_cases.oracle_dense_fill(
            {"coordinate": np.zeros((0, 24)), "S": np.zeros(0)}, surf, 0, 0, 0, ld=True)
        ref = _rect_self(a, b) / (4 * np.pi * 8.854187816997944e-12 * (a * b) ** 2)
        assert bad == 0
        assert abs(P["P"][0, 0] - ref) <= 1e-9 * ref


def test_far_entries_tend_to_the_point_value():
    lo1, hi1 = np.zeros(3), np.array([1e-3, 2e-4, 1e-4])
    off = np.array([0.31, 0.17, 0.05])
    vol = {"coordinate": np.array([ris_cases._brick24(lo1, hi1),
                                   ris_cases._brick24(lo1 + off, hi1 + off)]),
           "S": np.array([2e-8, 2e-8])}
    Lp, _, _, _, _ = ris_cases.oracle_dense_fill(
        vol, {"estremi_celle": np.zeros((0, 12)), "S": np.zeros(0)}, 2, 0, 0)
    V = 1e-3 * 2e-4 * 1e-4
    assert Lp["Lp_x"][0, 1] == pytest.approx(1e-7 * V * V / (2e-8 * 2e-8) / np.linalg.norm(off),
                                            rel=1e-6)
    r1 = ris_cases._rect12([0, 0, 0], [1e-3, 1e-3, 0])
    r2 = ris_cases._rect12((off).tolist(), (off + [1e-3, 0, 1e-3]).tolist())
    surf = {"estremi_celle": np.array([r1, r2]), "S": np.array([1e-6, 1e-6])}
    _, P, _, _, _ = ris_cases.oracle_dense_fill(
        {"coordinate": np.zeros((0, 24)), "S": np.zeros(0)}, surf, 0, 0, 0)
    c1 = np.array([5e-4, 5e-4, 0])
    c2 = off + [5e-4, 0, 5e-4]
    ref = 1 / (4 * np.pi * 8.854187816997944e-12 * np.linalg.norm(c1 - c2))
    assert P["P"][0, 1] == pytest.approx(ref, rel=1e-6)


def test_double_matches_long_double_on_every_branch():
    vol, surf = ris_cases.random_bodies(7, 40, 30, 25, 60)
    Ld, Pd, sLd, sPd, bad_d = ris_cases.oracle_dense_fill(vol, surf, 40, 30, 25)
    Ll, Pl, _, _, bad_l = ris_cases.oracle_dense_fill(vol, surf, 40, 30, 25, ld=True)
    for k in ("Lp_x", "Lp_y", "Lp_z"):
        fin = np.isfinite(Ll[k])
        assert np.array_equal(np.isfinite(Ld[k]), fin)
        assert np.all(np.abs(Ld[k] - Ll[k])[fin] <= 64 * EPS * sLd[k][fin] + 1e-300)
        assert np.array_equal(Ld[k], Ld[k].T)
    fin = np.isfinite(Pl["P"])
    assert np.all(np.abs(Pd["P"] - Pl["P"])[fin] <= 64 * EPS * sPd[fin] + 1e-300)
    assert np.array_equal(Pd["P"], Pd["P"].T)
    assert bad_d == bad_l


def test_random_bodies_take_every_branch():
    """The seeded bodies (clustered and far apart, some thin) take every case of both trees:
    Lp pairs from volume-volume (no dimension collapsed) to point-point (six), P pairs from
    surface-surface (the two normals) to point-point."""
    vol, surf = ris_cases.random_bodies(7, 40, 30, 25, 60)
    forms = {}
    ris_cases.oracle_dense_fill(vol, surf, 40, 30, 25, forms=forms)
    lp = np.concatenate([forms[k][np.triu_indices(forms[k].shape[0], 1)]
                         for k in ("Lp_x", "Lp_y", "Lp_z")])
    assert set(np.unique(lp)) == set(range(7))
    assert set(np.unique(forms["P"])) == set(range(2, 7))


def test_voxel_bodies_give_the_voxel_dense_blocks():
    c = ris_cases.voxel_case(configs.crossbar_20x20x4())
    Lp_v, P_v = ris_cases.dense_blocks(c)
    vol, surf = ris_cases.ris_geometry(c)
    inc = c["inc"]
    Lp_r, P_r, _, _, bad = ris_cases.oracle_dense_fill(vol, surf, inc["mx"], inc["my"],
                                                       inc["mz"], c["esc"]["Lp"], c["esc"]["P"])
    assert bad == 0
    for k in ("Lp_x", "Lp_y", "Lp_z"):
        A, B = Lp_r[k], Lp_v[k]
        if not B.size:
            continue
        off = ~np.eye(A.shape[0], dtype=bool)
        assert np.max(np.abs(A - B)[off]) <= 1e-9 * np.max(np.abs(B)), k
        # the voxel path lengthens the self terms of edges at a conductor's border to 1.5
        # and 2 voxels (compute_diagonals.jl:109-126); its interior edges carry the bar
        # formula of one voxel, the RIS fill's self term of the same brick
        assert np.allclose(np.diag(A), np.min(np.diag(B)), rtol=1e-13, atol=0), k
    assert np.max(np.abs(P_r["P"] - P_v["P"])) <= 1e-9 * np.max(np.abs(P_v["P"]))


def _nan_case():
    """Two x-directed bodies: a small cube far from a thin plate, its centre in the plate's
    mid-plane and on the line of one of the plate's edges. The suppression tests make them
    a point and a surface, and the point-surface form's arctangent of the quotient
    (integ_point_sup_sharedRis, Song_improved_Ivana_strategy.jl:449-478) meets 0/0 there.
    Every coordinate is a short dyadic fraction, exact in binary and under 14 decimals."""
    h = 2.0 ** -12
    mid = 2.0 ** -14
    cube_lo, cube_hi = np.array([-h, 0.5 - h, mid - h]), np.array([h, 0.5 + h, mid + h])
    plate_lo, plate_hi = np.array([0.0, 0.0, 0.0]), np.array([2.0 ** -5, 2.0 ** -5, 2 * mid])
    vol = {"coordinate": np.array([ris_cases._brick24(cube_lo, cube_hi),
                                   ris_cases._brick24(plate_lo, plate_hi)]),
           "S": np.array([4 * h * h, 2 * mid * 2.0 ** -5])}
    return vol


def test_point_in_a_surface_plane_gives_the_reference_nan():
    vol = _nan_case()
    forms = {}
    Lp, _, _, _, bad = ris_cases.oracle_dense_fill(
        vol, {"estremi_celle": np.zeros((0, 12)), "S": np.zeros(0)}, 2, 0, 0, forms=forms)
    assert forms["Lp_x"][0, 1] == 4  # point (3 collapsed) against surface (1)
    assert np.isnan(Lp["Lp_x"][0, 1]) and np.isnan(Lp["Lp_x"][1, 0])
    assert bad == 1


def test_suppressed_forms_tend_to_the_point_value():
    """Every collapsed-dimension form of both trees (a body replaced by a surface, a line or
    a point once its dimension passes the suppression test) is a far-field approximation of
    the same integral: against the point-point value V1 V2 / R it errs by at most a small
    multiple of (size / R)^2. A mistyped form would miss by O(1)."""
    mx, my, mz, ns = 40, 30, 25, 60
    vol, surf = ris_cases.random_bodies(7, mx, my, mz, ns)
    forms = {}
    Lp, P, _, _, _ = ris_cases.oracle_dense_fill(vol, surf, mx, my, mz, ld=True, forms=forms)
    C = np.asarray(vol["coordinate"]).reshape(-1, 8, 3)
    lo, hi = C.min(1), C.max(1)
    ctr, ext = 0.5 * (lo + hi), hi - lo
    V, S, size = ext.prod(1), np.asarray(vol["S"]), ext.max(1)

    def check(M, f, pp, r, first):
        iu = np.triu_indices(M.shape[0], 1)
        sel = f[iu] >= first
        assert sel.sum() > 50
        rel = np.abs(M[iu][sel] - pp[iu][sel]) / pp[iu][sel]
        assert np.all(rel <= 0.5 * r[iu][sel] ** 2), float(np.max(rel / r[iu][sel] ** 2))

    off = 0
    for k, n in (("Lp_x", mx), ("Lp_y", my), ("Lp_z", mz)):
        sl = slice(off, off + n)
        off += n
        R = np.linalg.norm(ctr[sl][:, None] - ctr[sl][None], axis=-1)
        R = np.where(R > 0, R, 1.0)
        pp = 1e-7 * np.outer(V[sl], V[sl]) / np.outer(S[sl], S[sl]) / R
        r = np.maximum.outer(size[sl], size[sl]) / R
        check(Lp[k], forms[k], pp, r, 1)
    E = np.asarray(surf["estremi_celle"])
    slo, shi = np.minimum(E[:, :3], E[:, 9:]), np.maximum(E[:, :3], E[:, 9:])
    R = np.linalg.norm(0.5 * (slo + shi)[:, None] - 0.5 * (slo + shi)[None], axis=-1)
    R = np.where(R > 0, R, 1.0)
    pp = 1 / (4 * np.pi * 8.854187816997944e-12 * R)
    r = np.maximum.outer((shi - slo).max(1), (shi - slo).max(1)) / R
    check(P["P"], forms["P"], pp, r, 3)
