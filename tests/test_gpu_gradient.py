"""GPU: gradient of a port's |Z| with respect to per-voxel conductivity (adjoint by
reciprocity, solver_gb300/gradient.py) from the GPU's port solves.

On a copper bar joining the port terminals the port impedance is R + jwL and one bar
voxel moves |Z| enough for a central difference of FP64 GMRES solves to resolve the
gradient. On a random copper grid whose terminals are not joined, |Z| is capacitive and
moves by less than the solves' rounding floor when one voxel (or all of them, by 1e-3)
changes; there the gradient is checked against the one from a dense oracle solve, and
the mixed-precision solution's gradient against the FP64 one."""
import numpy as np
import pytest

from gradient_dense import DensePort, bar_request
from solver_gb300 import configs, gradient as G, mesher

pytestmark = pytest.mark.gpu

RANDOM = dict(shape=(12, 12, 6), p=0.35, seed=5, nports=1, freqs=[1e8, 5e9], tol=1e-10)


@pytest.fixture(scope="module")
def bar():
    P = G.PortImpedanceProblem(mesher.parse_request(bar_request([1e6, 1e8])))
    yield P
    P.close()


@pytest.fixture(scope="module")
def problem():
    P = G.PortImpedanceProblem(mesher.parse_request(configs.random_copper(**RANDOM)))
    yield P
    P.close()


@pytest.mark.parametrize("k", [0, 1])
def test_gradient_matches_finite_differences_on_bar(bar, k):
    _, g, _ = bar.solve(k, mode="fp64", tol=1e-12, warm=False, maxit=600)
    rng = np.random.default_rng(5)
    vox = np.concatenate([np.argsort(-np.abs(g))[:3],
                          rng.choice(bar.conductor_voxels, size=3, replace=False)])
    fd = bar.finite_difference(k, vox, h_rel=1e-3, tol=1e-12)
    scale = np.max(np.abs(g[bar.conductor_voxels]))
    assert np.max(np.abs(fd - g[vox])) <= 1e-3 * scale, (fd, g[vox])


@pytest.mark.parametrize("k", [0, 1])
def test_gradient_matches_dense_oracle(problem, k):
    _, g, Z = problem.solve(k, mode="fp64", tol=1e-12, warm=False, maxit=600)
    _, g_ref, Z_ref = DensePort(configs.random_copper(**RANDOM)).solve(k)
    assert abs(Z - Z_ref) <= 1e-8 * abs(Z_ref)
    scale = np.max(np.abs(g_ref))
    assert np.max(np.abs(g - g_ref)) <= 1e-5 * scale


def test_mixed_gradient_matches_fp64(problem):
    _, g64, _ = problem.solve(1, mode="fp64", tol=1e-10, warm=False, maxit=600)
    _, gmx, _ = problem.solve(1, mode="mixed", tol=1e-10, warm=False)
    scale = np.max(np.abs(g64))
    assert np.max(np.abs(gmx - g64)) <= 1e-6 * scale


def test_autograd_function(bar):
    torch = pytest.importorskip("torch")
    f = G.impedance_magnitude_function()
    sigma = torch.tensor(bar.sigma_ref_voxel, dtype=torch.float64, requires_grad=True)
    z = f.apply(sigma, bar, 0, "fp64")
    z.backward()
    _, g, _ = bar.solve(0, mode="fp64")
    assert np.allclose(sigma.grad.numpy(), g, rtol=1e-6, atol=1e-6 * np.max(np.abs(g)))


def test_device_scatter_matches_host(problem):
    """peec_adjoint (the per-voxel scatter on the GPU, double atomics) against the
    host scatter of the same solution and derivative tables."""
    k = 0
    w = 2 * np.pi * problem.freqs[k] * problem.esc["freq"]
    _fs, d1, d2 = problem._state(w, problem.sigma_ref_voxel)
    absZ, g_dev, _ = problem.solve(k, mode="fp64", tol=1e-10, warm=False, maxit=600)
    V = problem._x["fp64"]
    n1, n2 = np.asarray(problem.ports["port_nodes"]).reshape(-1, 2)[0]
    a_host, g_host, _ = G.port_impedance_and_gradient(
        V, problem.m, problem.ns, (n1, n2), problem.z0, problem.esc["Is"], d1, d2, problem.v1,
        problem.v2, problem.nvox)
    assert a_host == absZ
    assert np.max(np.abs(g_dev - g_host)) <= 1e-12 * np.max(np.abs(g_host))
