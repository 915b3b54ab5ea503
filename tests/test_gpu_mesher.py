"""GPU: the voxel mesher on the GPU (csrc/mesher_gpu.cu) produces the host mesher's
topology (csrc/mesher.cpp, itself held index for index to the oracle's restatement of
mesher_FFT.jl in tests/test_oracle_mesher.py) array for array: voxel and node numbering,
edges with their incidence, materials, borders and surface-impedance counters, surfaces
with their families, lattice cells and nodes. Cases: the reference's request fixtures,
the crossbar, random multi-material grids with dominant and non-dominant grids (some
single-layer, some with one-voxel-thin axes) and the 128x128x64 benchmark geometry; and a
whole request parsed with the GPU mesher equals the host parse."""
import copy
import gzip
import json

import numpy as np
import pytest

from solver_gb300 import configs, mesher

pytestmark = pytest.mark.gpu

GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"


def _random_grids(shape, G, p, seed):
    rng = np.random.default_rng(seed)
    occ = rng.random(shape) < p
    which = rng.integers(0, G, size=shape)
    return np.stack([occ & (which == k) for k in range(G)])


def _cases():
    out = {}
    for name in ("first_run_data.json", "first_run_data_2_materials.json"):
        out[name] = mesher.load_request(GOLDEN / name)
    out["crossbar57"] = json.load(gzip.open(GOLDEN / "crossbar.json.gz"))
    out["crossbar20"] = configs.crossbar_20x20x4()
    return out


RANDOM = [((9, 7, 5), 3, 0.5, 1, [0, 2]), ((12, 10, 1), 2, 0.6, 2, [1]),
          ((1, 8, 6), 3, 0.55, 3, [0]), ((16, 1, 9), 2, 0.5, 4, [0, 1]),
          ((24, 20, 12), 3, 0.35, 5, [2]), ((7, 7, 7), 4, 0.7, 6, [])]


def _compare(grids, dominant, sigma):
    host = mesher._raw_mesh(grids, dominant, sigma)
    gpu = mesher._raw_mesh(grids, dominant, sigma, device=0)
    for k in mesher.MESH_ARRAYS:
        assert host[k].dtype == gpu[k].dtype and np.array_equal(host[k], gpu[k]), k


@pytest.mark.parametrize("i", range(len(RANDOM)))
def test_gpu_mesher_random_grids(i):
    shape, G, p, seed, dom = RANDOM[i]
    grids = _random_grids(shape, G, p, seed)
    dominant = np.zeros(G, dtype=np.uint8)
    dominant[dom] = 1
    sigma = np.where(dominant == 1, 5.8e7, 0.0)
    if G > 2:
        sigma[-1] = 1e3  # a lossy non-dominant grid: surface-impedance counters
    _compare(grids, dominant, sigma)


@pytest.mark.parametrize("name", sorted(_cases()))
def test_gpu_mesher_requests(name):
    req = _cases()[name]
    host = mesher.parse_request(copy.deepcopy(req))
    gpu = mesher.parse_request(copy.deepcopy(req), device=0)
    (esc, inc, cc, diag, exp, ports, le, li, Zs), *_ = host
    (esc2, inc2, cc2, diag2, exp2, ports2, le2, li2, Zs2), *_ = gpu
    assert (inc["A"] != inc2["A"]).nnz == 0 and (inc["Gamma"] != inc2["Gamma"]).nnz == 0
    for k in ("edge_cell", "surf_cell", "surf_fam", "vox_map"):
        assert np.array_equal(exp[k], exp2[k]), k
    for k in ("R", "Cd", "Lp", "P"):
        assert np.array_equal(diag[k], diag2[k]), k
    assert np.array_equal(Zs["Zs"], Zs2["Zs"])
    assert np.array_equal(ports["port_nodes"], ports2["port_nodes"])


def test_gpu_mesher_benchmark_geometry():
    req = configs.random_128x128x64()
    out, freqs, settings, z0, grid = mesher.parse_request(copy.deepcopy(req), device=0)
    ref = mesher.parse_request(copy.deepcopy(req))[0]
    assert (out[1]["A"] != ref[1]["A"]).nnz == 0
    assert (out[1]["Gamma"] != ref[1]["Gamma"]).nnz == 0
    assert np.array_equal(out[4]["edge_cell"], ref[4]["edge_cell"])
    assert np.array_equal(out[5]["port_nodes"], ref[5]["port_nodes"])
