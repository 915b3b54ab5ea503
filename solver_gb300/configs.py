"""Synthetic voxel geometries of the benchmark configurations.

Every geometry is produced as a solve request in the reference's JSON schema
(mesherOutput / solverInput / solverAlgoParams, do_solving_fft.jl:1-62) so that it
goes through the same parsing and mesher as a real request. Inputs are seeded
synthetic stand-ins with the stated shapes, sizes and distributions.

* crossbar_20x20x4  -- two copper bars (4 voxels wide, 1 thick) crossing at right
  angles on layers 1 and 3 of a 20x20x4 grid of 1e-4 m voxels, one port between the
  bar ends, 1 GHz, tol 1e-6.
* random_128x128x64 -- 128x128x64 grid of 5e-5 m voxels, occupancy Bernoulli(0.3)
  (seed 2), copper / FR4-like dielectric (eps_r 4.4) 50/50, 4 ports between random
  occupied copper voxels on the outer faces, 10 frequencies log-spaced
  10 MHz - 10 GHz, tol 1e-8. Voxels without any occupied face neighbour are removed
  (drop_isolated), since the reference algorithm cannot solve a geometry that has them.
* random_copper(a, b, c, p, seed) -- copper-only Bernoulli(p) grids.
* batched_sweep -- 12 uneven copper grids a x a x a/2 (a = 32..96 from seed 4),
  Bernoulli(0.25), one port each, 64 frequencies 1 MHz - 10 GHz, tol 1e-8.
"""
from __future__ import annotations

import numpy as np

COPPER = {"name": "copper", "color": "#b87333", "permeability": 1, "permittivity": 1,
          "conductivity": 5.8e7}
DIELECTRIC = {"name": "dielectric", "color": "#00aa00", "permeability": 1, "permittivity": 4.4,
              "conductivity": 0}


def _centre(idx, s, origin=(0.0, 0.0, 0.0)):
    return [origin[d] + s[d] * idx[d] + s[d] / 2 for d in range(3)]


def make_request(grids: dict, materials: list, cell, ports, freqs, tol, inner=100):
    """grids: name -> bool array (Nx,Ny,Nz); ports: list of (voxel_a, voxel_b) 0-based."""
    names = list(grids.keys())
    shape = grids[names[0]].shape
    mm = {k: np.asarray(v, dtype=bool).tolist() for k, v in grids.items()}
    return {
        "mesherOutput": {
            "cell_size": {"cell_size_x": cell[0], "cell_size_y": cell[1], "cell_size_z": cell[2]},
            "origin": {"origin_x": 0.0, "origin_y": 0.0, "origin_z": 0.0},
            "n_cells": {"n_cells_x": shape[0], "n_cells_y": shape[1], "n_cells_z": shape[2]},
            "n_materials": len(names),
            "mesher_matrices": mm,
        },
        "solverInput": {
            "unit": "m",
            "materials": materials,
            "ports": [{"name": f"Port{i + 1}", "type": 1,
                       "inputElement": _centre(a, cell), "outputElement": _centre(b, cell),
                       "rlcParams": {"resistance": 50}} for i, (a, b) in enumerate(ports)],
            "lumped_elements": [],
            "frequencies": [float(f) for f in freqs],
            "ports_scattering_value": 50.0,
        },
        "solverAlgoParams": {"innerIteration": inner, "outerIteration": 1,
                             "convergenceThreshold": tol},
        "solverType": 1,
    }


def crossbar_20x20x4():
    N = (20, 20, 4)
    cu = np.zeros(N, dtype=bool)
    cu[0:20, 8:12, 0] = True   # bar A: x = 1..20, y = 9..12, z = 1 (1-based)
    cu[8:12, 0:20, 2] = True   # bar B: x = 9..12, y = 1..20, z = 3
    return make_request({"copper": cu}, [dict(COPPER)], (1e-4, 1e-4, 1e-4),
                        [((19, 9, 0), (9, 19, 2))], [1e9], 1e-6, inner=100)


def _draw(shape, p, rng):
    n = int(np.prod(shape))
    return (rng.random(n) < p).reshape(shape, order="F")


def drop_isolated(occ):
    """Removes voxels with no occupied face neighbour. Such a voxel gets neither an
    inductive edge nor a charge surface in the reference mesher (every face test of
    create_mapping_Gamma_no_rep.jl:32,59,86,113 and the x/z analogues needs a
    neighbour), so its node would leave the Schur complement SS exactly singular."""
    nb = np.zeros(occ.shape, dtype=np.int32)
    for ax in range(3):
        for sh in (1, -1):
            r = np.roll(occ, sh, axis=ax)
            sl = [slice(None)] * 3
            sl[ax] = 0 if sh == 1 else -1
            r[tuple(sl)] = False
            nb += r
    return occ & (nb > 0)


def _boundary_ports(mask, nports, rng):
    Nx, Ny, Nz = mask.shape
    face = np.zeros_like(mask)
    face[[0, -1], :, :] = True
    face[:, [0, -1], :] = True
    face[:, :, [0, -1]] = True
    cand = np.argwhere(mask & face)
    pick = rng.choice(len(cand), size=2 * nports, replace=False)
    v = [tuple(int(t) for t in cand[i]) for i in pick]
    return [(v[2 * k], v[2 * k + 1]) for k in range(nports)]


def random_mixed(shape=(128, 128, 64), s=5e-5, p=0.3, seed=2, nports=4,
                 freqs=None, tol=1e-8, inner=100):
    """Bernoulli(p) occupancy, copper/dielectric 50/50 drawn from the seed."""
    rng = np.random.default_rng(seed)
    occ = _draw(shape, p, rng)
    is_cu = _draw(shape, 0.5, rng)
    occ = drop_isolated(occ)
    cu = occ & is_cu
    di = occ & ~is_cu
    ports = _boundary_ports(cu, nports, rng)
    if freqs is None:
        freqs = np.logspace(7, 10, 10)
    return make_request({"copper": cu, "dielectric": di}, [dict(COPPER), dict(DIELECTRIC)],
                        (s, s, s), ports, freqs, tol, inner=inner)


def random_128x128x64():
    return random_mixed()


def random_copper(shape, s=5e-5, p=0.3, seed=5, nports=1, freqs=(1e9,), tol=1e-8, inner=100):
    rng = np.random.default_rng(seed)
    cu = drop_isolated(_draw(shape, p, rng))
    ports = _boundary_ports(cu, nports, rng)
    return make_request({"copper": cu}, [dict(COPPER)], (s, s, s), ports, freqs, tol, inner=inner)


def batched_sweep(count=12, seed=4, side_range=(4, 13), nfreq=64, fmin=1e6, fmax=1e10, s=5e-5,
                  p=0.25, tol=1e-8, inner=100):
    """Uneven copper grids for a batched frequency sweep: side a = 8*integers(side_range)
    drawn from the seed, grid a x a x a/2, Bernoulli(p) copper occupancy and one port per
    geometry drawn from a per-geometry seed (1000*seed + index), nfreq log-spaced
    frequencies from fmin to fmax on every geometry."""
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_range[0], side_range[1], size=count) * 8
    freqs = list(np.logspace(np.log10(fmin), np.log10(fmax), nfreq))
    return [random_copper((int(a), int(a), int(a) // 2), s=s, p=p, seed=1000 * seed + i,
                          nports=1, freqs=freqs, tol=tol, inner=inner)
            for i, a in enumerate(sides)]
