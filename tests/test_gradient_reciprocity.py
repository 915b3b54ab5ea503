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

