"""GPU fill against the oracle on grids whose rows take the reference's far-field
(suppressed) integral branches: a long cubic-voxel grid (point-point beyond ~200
edges), thin voxels (surface-surface from a few cells on), long needle voxels
(parallel and collinear line-line) and anisotropic voxels (line-surface and
point-surface between P faces of different orientation). Both fills restate the same
branch formulas with the same scalar rounding (no FMA contraction on the GPU), so the
rows agree to within the rounding of the terms each entry sums."""
import numpy as np
import pytest

from oracle import peec_oracle as O
from solver_gb300 import configs, mesher

pytestmark = pytest.mark.gpu

GRIDS = {
    "cubic_232x3x2": ((232, 3, 2), (5e-5, 5e-5, 5e-5)),
    "thin_40x40x3": ((40, 40, 3), (1e-4, 1e-4, 1e-6)),
    "needle_60x4x4": ((60, 4, 4), (1e-3, 1e-5, 1e-5)),
    "aniso_120x48x4": ((120, 48, 4), (1e-4, 2e-4, 5e-5)),
}


def far_request(shape, cell):
    cu = np.zeros(shape, dtype=bool)
    cu[0:3, 0, 0] = True
    return configs.make_request({"copper": cu}, [dict(configs.COPPER)], cell,
                                [((0, 0, 0), (2, 0, 0))], [1e9], 1e-8)


@pytest.mark.parametrize("name", sorted(GRIDS))
def test_far_field_fill_matches_oracle(name):
    from solver_gb300.operator import GpuOperator
    shape, cell = GRIDS[name]
    out, _freqs, _settings, _z0, grid = mesher.parse_request(far_request(shape, cell))
    esc, inc, cc, diag, exp = out[0], out[1], out[2], out[3], out[4]
    far = {}
    ref = O.fill_rows(cc, esc, *grid, with_scale=True, far_counts=far)
    assert sum(far.values()) > 0, "the grid does not reach the far-field branches"
    op = GpuOperator(inc, exp, diag["P"])
    try:
        got = op.fill(cc["origin"], cc["sx"], cc["sy"], cc["sz"], esc["Lp"], esc["P"],
                      return_rows=True)
    finally:
        op.close()
    eps = np.finfo(float).eps
    for key, (row, scale) in ref.items():
        err = np.abs(got[key] - row)
        bound = 64 * eps * scale + 1e-300
        assert np.all(np.isfinite(got[key])), key
        assert np.all(err <= bound), (key, far[key], float(np.max(err / bound)))
