"""CPU: the reciprocity gradient of a port's |Z| in per-voxel conductivity
(solver_gb300/gradient.py) against central finite differences of dense oracle solves
(one LU solve per perturbed conductivity, so the difference carries no iterative
noise), on a copper bar joining the port terminals."""
import numpy as np
import pytest

from gradient_dense import DensePort, bar_request


@pytest.fixture(scope="module")
def bar():
    return DensePort(bar_request([1e6, 1e8], shape=(8, 4, 4)))


@pytest.mark.parametrize("k", [0, 1])
def test_reciprocity_gradient_matches_dense_differences(bar, k):
    absZ, g, Z = bar.solve(k)
    assert abs(Z.real) > 0 and absZ > 0
    vox = np.concatenate([np.argsort(-np.abs(g))[:2],
                          np.random.default_rng(3).choice(bar.nvox, 2, replace=False)])
    fd = bar.finite_difference(k, vox, h_rel=1e-4)
    scale = np.max(np.abs(g))
    assert np.max(np.abs(fd - g[vox])) <= 1e-5 * scale, (fd, g[vox])



def test_edge_impedance_derivatives_match_differences():
    """gradient.dz_edges: the derivative of every edge impedance DZ_e with respect to the
    conductivity of each of its two voxels (half resistances, their RC parallels, and the
    surface impedance with its keep-the-larger-real-part switch) against central
    differences of DZ itself, away from the switch."""
    from solver_gb300 import configs, gradient as G
    from gradient_dense import DensePort
    P = DensePort(configs.random_copper((10, 8, 6), p=0.5, seed=9, freqs=(2e9,)))
    w = 2 * np.pi * P.freqs[0] * P.esc["freq"]
    DZ, d1, d2 = G.dz_edges(w, P.esc, P.diag, P.Zs, P.sigma_ref, P.v1, P.v2, P.sigma_edge)
    se = np.asarray(P.Zs["surface_edges"], dtype=np.int64)
    assert se.size > 0  # the surface-impedance branch is exercised
    rng = np.random.default_rng(9)
    checked = 0
    for v in rng.choice(np.flatnonzero(P.sigma_ref > 0), size=12, replace=False):
        h = 1e-6 * P.sigma_ref[v]
        plus, minus = P.sigma_ref.copy(), P.sigma_ref.copy()
        plus[v] += h
        minus[v] -= h
        Dp = G.dz_edges(w, P.esc, P.diag, P.Zs, plus, P.v1, P.v2, P.sigma_edge)[0]
        Dm = G.dz_edges(w, P.esc, P.diag, P.Zs, minus, P.v1, P.v2, P.sigma_edge)[0]
        fd = (Dp - Dm) / (2 * h)
        want = np.where(P.v1 == v, d1, 0) + np.where(P.v2 == v, d2, 0)
        # skip edges whose switch flips inside the difference step
        smooth = (np.sign(Dp.real - DZ.real) == np.sign(DZ.real - Dm.real)) | (want == 0)
        touch = ((P.v1 == v) | (P.v2 == v)) & smooth
        scale = np.max(np.abs(want[touch]))
        assert np.max(np.abs(fd[touch] - want[touch])) <= 1e-6 * scale
        assert np.all(np.abs(fd[~((P.v1 == v) | (P.v2 == v))]) == 0)
        checked += int(touch.sum())
    assert checked > 24
