"""CPU: the oracle's restatement of the reference mesher (oracle/mesher_ref.py, written from
mesher_FFT.jl and its helpers) against the product mesher (solver_gb300/csrc/mesher.cpp via
solver_gb300.mesher), index for index: incidence A, Gamma, the Lp lattice maps, the nine
P lattice maps, family sizes, edge grids and border classes, the diagonals, the surface
impedance and its edge classes, port and lumped-element nodes, and the lattice centres.
Inputs: the reference's three request fixtures, the 20x20x4 crossbar, and seeded random
multi-material grids (copper and dielectric, two conductors, a conductor-free grid)."""
import gzip
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import mesher_ref as OM
from solver_gb300 import configs, mesher

GOLD = Path(__file__).resolve().parent / "golden"


def _load(name):
    p = GOLD / name
    if name.endswith(".gz"):
        return json.loads(gzip.decompress(p.read_bytes()))
    return json.loads(p.read_text())


def _same_sparse(a, b, what):
    a = a.tocsr().astype(np.float64)
    b = b.tocsr().astype(np.float64)
    assert a.shape == b.shape, (what, a.shape, b.shape)
    a.sum_duplicates()
    b.sum_duplicates()
    a.sort_indices()
    b.sort_indices()
    a.eliminate_zeros()
    b.eliminate_zeros()
    assert np.array_equal(a.indptr, b.indptr), what
    assert np.array_equal(a.indices, b.indices), what
    assert np.array_equal(a.data, b.data), what


def _random_request(shape, seed, kinds):
    """Seeded Bernoulli grids; kinds: the materials, each voxel drawn from one of them."""
    rng = np.random.default_rng(seed)
    occ = configs.drop_isolated(rng.random(shape) < 0.45)
    which = rng.integers(0, len(kinds), size=shape)
    grids = {m["name"]: occ & (which == i) for i, m in enumerate(kinds)}
    cond = [g for m, g in zip(kinds, grids.values()) if m["conductivity"] > 0]
    pool = np.argwhere(cond[0] if cond else occ)
    pick = rng.choice(len(pool), size=4, replace=False)
    v = [tuple(int(t) for t in pool[i]) for i in pick]
    return configs.make_request(grids, [dict(m) for m in kinds], (1e-4, 2e-4, 5e-5),
                                [(v[0], v[1]), (v[2], v[3])], [1e9], 1e-6)


BRASS = {"name": "brass", "color": "#aa8800", "permeability": 1, "permittivity": 1,
         "conductivity": 1.5e7}
TEFLON = {"name": "teflon", "color": "#ffffff", "permeability": 1, "permittivity": 2.1,
          "conductivity": 0}

CASES = {
    "first_run_data": lambda: _load("first_run_data.json"),
    "first_run_data_2_materials": lambda: _load("first_run_data_2_materials.json"),
    "crossbar_fixture": lambda: _load("crossbar.json.gz"),
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "random_cu_diel": lambda: _random_request((9, 7, 5), 11, [configs.COPPER, configs.DIELECTRIC]),
    "random_two_conductors": lambda: _random_request((8, 8, 6), 12,
                                                     [configs.COPPER, BRASS, configs.DIELECTRIC]),
    "random_diel_first": lambda: _random_request((7, 9, 4), 13,
                                                 [configs.DIELECTRIC, configs.COPPER, TEFLON]),
    "random_mixed_small": lambda: configs.random_mixed((12, 10, 6), s=5e-5, seed=3, nports=2,
                                                       freqs=[1e8]),
    "random_three_24x20x12": lambda: _random_request((24, 20, 12), 14,
                                                     [configs.COPPER, configs.DIELECTRIC, BRASS]),
    # the benchmark geometry itself
    "random_128x128x64": configs.random_128x128x64,
}


@pytest.mark.parametrize("case", list(CASES))
def test_oracle_mesher_equals_product_mesher(case):
    req = CASES[case]()
    (out_o, f_o, set_o, z0_o, grid_o) = OM.parse_request(json.loads(json.dumps(req)))
    (out_p, f_p, set_p, z0_p, grid_p) = mesher.parse_request(json.loads(json.dumps(req)))
    assert tuple(grid_o) == tuple(grid_p)
    assert np.array_equal(f_o, f_p) and z0_o == z0_p and set_o == set_p
    esc_o, inc_o, cc_o, dg_o, ex_o, po_o, le_o, li_o, zs_o = out_o
    esc_p, inc_p, cc_p, dg_p, ex_p, po_p, le_p, li_p, zs_p = out_p
    assert esc_o == esc_p
    # topology
    for k in ("mx", "my", "mz"):
        assert inc_o[k] == inc_p[k], k
    _same_sparse(inc_o["A"], inc_p["A"], "A")
    _same_sparse(inc_o["Gamma"], inc_p["Gamma"], "Gamma")
    for k in ("N1", "N2", "N3"):
        assert ex_o[k] == ex_p[k], k
    for c in range(3):
        _same_sparse(ex_o["mat_map_Lp"][c][0], ex_p["mat_map_Lp"][c][0], f"mat_map_Lp[{c}]")
    for i in range(3):
        for j in range(3):
            _same_sparse(ex_o["exp_P"][i][j], ex_p["exp_P"][i][j], f"exp_P[{i}][{j}]")
    # edge grids and border classes
    mats_o = np.concatenate([li_o["lix_mat"], li_o["liy_mat"], li_o["liz_mat"]])
    mats_p = np.concatenate([li_p["lix_mat"], li_p["liy_mat"], li_p["liz_mat"]])
    assert np.array_equal(mats_o, mats_p)
    b_o = np.concatenate([li_o["lix_border"], li_o["liy_border"], li_o["liz_border"]])
    assert np.array_equal(b_o[:, 0], li_p["border1"]) and np.array_equal(b_o[:, 1], li_p["border2"])
    # diagonals: the same expressions in the same order
    assert np.array_equal(dg_o["R"], dg_p["R"])
    assert np.array_equal(dg_o["Cd"], dg_p["Cd"])
    np.testing.assert_allclose(dg_o["Lp"], dg_p["Lp"], rtol=4e-16, atol=0)
    np.testing.assert_allclose(dg_o["fc_Lp"], dg_p["fc_Lp"], rtol=0,
                               atol=4e-16 * np.max(np.abs(dg_p["Lp"])))
    # P self terms: the oracle's C fill of a face with itself against the product's
    # closed form of the same integral
    np.testing.assert_allclose(dg_o["P"], dg_p["P"], rtol=1e-13, atol=0)
    # surface impedance and its edge classes
    np.testing.assert_array_equal(zs_o["internal_edges"], zs_p["internal_edges"])
    np.testing.assert_array_equal(zs_o["surface_edges"], zs_p["surface_edges"])
    np.testing.assert_allclose(zs_o["Zs"], zs_p["Zs"], rtol=4e-16, atol=0)
    # terminals
    assert np.array_equal(np.asarray(po_o["port_nodes"]), np.asarray(po_p["port_nodes"]))
    assert np.array_equal(np.asarray(po_o["port_voxels"]), np.asarray(po_p["port_voxels"]))
    assert np.array_equal(np.asarray(le_o["le_nodes"]).reshape(-1, 2),
                          np.asarray(le_p["le_nodes"]).reshape(-1, 2))
    # lattice centres the rows are filled on
    for key in ("p12_se", "p34_se", "p56_se", "p1234", "p1256", "p3456", "Lpx", "Lpy", "Lpz"):
        assert np.array_equal(cc_o[key], cc_p[key]), key


def test_oracle_mesher_counts_of_a_solid_bar():
    """Known answer: a solid 3 x 2 x 2 copper bar. Every voxel is on the boundary, so
    every voxel keeps its own node (n = 12); edges join face neighbours (x: 2*2*2 = 8,
    y: 3*1*2 = 6, z: 3*2*1 = 6); the surfaces are the bar's two end faces along each axis,
    one per cell of the end (y: 2 x 3*2, x: 2 x 2*2, z: 2 x 3*2)."""
    cu = np.ones((3, 2, 2), dtype=bool)
    req = configs.make_request({"copper": cu}, [dict(configs.COPPER)], (1e-4, 1e-4, 1e-4),
                               [((0, 0, 0), (2, 1, 1))], [1e9], 1e-6)
    (out, *_rest) = OM.parse_request(req)
    inc, ex = out[1], out[4]
    assert inc["A"].shape == (8 + 6 + 6, 12)
    assert (inc["mx"], inc["my"], inc["mz"]) == (8, 6, 6)
    # surfaces: two per voxel column along each axis (the two end faces)
    assert (ex["N1"], ex["N2"], ex["N3"]) == (2 * 3 * 2, 2 * 2 * 2, 2 * 3 * 2)
    # every edge joins two distinct nodes with -1 / +1
    A = inc["A"].tocsr()
    assert np.all(np.diff(A.indptr) == 2)
    assert np.array_equal(np.asarray(A.sum(axis=1)).ravel(), np.zeros(20))
