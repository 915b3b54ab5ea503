"""Host-side setup of the FFT-PEEC operator: request parsing and the voxel mesher.

The GPU path consumes the same data structures the reference solver builds before
its frequency loop, so this module produces them with the reference's layout:

* ``incidence_selection`` -- ``A`` (m x n, -1/+1 per edge), ``Gamma`` (n x ns) and the
  per-direction edge counts ``mx, my, mz`` (src/lib/solverFFT/mesher_FFT.jl:36-54);
* ``expansions`` -- lattice maps ``mat_map_Lp`` / ``exp_P`` and family sizes
  ``N1..N3`` (mesher_FFT.jl:58-84, create_mapping_Gamma_no_rep.jl:382-419);
* ``diagonals`` -- per-edge R/Cd halves, Lp and P self terms
  (compute_diagonals.jl:1-134, mesher_FFT.jl:114-138);
* ``Zs_info`` -- surface impedance per edge (compute_Zs_with_indices.jl);
* ``circulant_centers`` -- the lattice centres the Lp/P rows are filled on
  (build_center_P_Voxels.jl, build_centers_Lp_with_air.jl), built lazily because
  the cross lattices hold ~4M points each at 128x128x64.

Indices are 0-based throughout (the reference is 1-based).
"""
from __future__ import annotations

import ctypes
import json
import math
from pathlib import Path

import numpy as np
import scipy.sparse as sp

from . import build as _build

EPS0 = 8.854187816997944e-12  # compute_diagonals.jl:5, compute_row_P_sup.jl:2

ESCALINGS = {"Lp": 1e6, "P": 1e-12, "R": 1e-3, "Cd": 1e12, "Is": 1e3, "Yle": 1e3,
             "freq": 1e-9, "time": 1e9}  # mesher_FFT.jl:5-15


_mesh_lib = None


def _lib():
    global _mesh_lib
    if _mesh_lib is None:
        path = _build.LIBDIR / "libpeec_mesh.so"
        if not path.exists():
            _build.build_mesh()
        L = ctypes.CDLL(str(path))
        L.peec_mesh_build.restype = ctypes.c_void_p
        L.peec_mesh_build.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        L.peec_mesh_len.restype = ctypes.c_int64
        L.peec_mesh_len.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int)]
        L.peec_mesh_copy.restype = ctypes.c_int
        L.peec_mesh_copy.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p]
        L.peec_mesh_free.argtypes = [ctypes.c_void_p]
        _mesh_lib = L
    return _mesh_lib


MESH_ARRAYS = ("vox_map", "vox_node", "counts", "edge_n1", "edge_n2", "edge_cell", "edge_mat",
               "edge_border1", "edge_border2", "edge_zs", "surf_node", "surf_fam", "surf_cell",
               "nodes", "nodes_red")


def _raw_mesh(grids: np.ndarray, dominant, sigma, device=None) -> dict:
    """Runs the native mesher; grids is (G, Nx, Ny, Nz) bool, dominant a length-G mask of
    the conductor grids and sigma the G conductivities (the library reads G of each).
    device None: the host mesher (C++, OpenMP); an int: the GPU mesher on that device
    (the same arrays, index for index)."""
    G, Nx, Ny, Nz = grids.shape
    g = np.ascontiguousarray(np.transpose(grids.astype(np.uint8), (0, 3, 2, 1)))  # x fastest
    dom = np.ascontiguousarray(np.asarray(dominant, dtype=np.uint8))
    sig = np.ascontiguousarray(np.asarray(sigma, dtype=np.float64))
    if dom.shape != (G,) or sig.shape != (G,):
        raise ValueError(f"dominant and sigma need one entry per grid ({G}); "
                         f"got {dom.shape} and {sig.shape}")
    if device is None:
        L = _lib()
        h = L.peec_mesh_build(g.ctypes.data, G, Nx, Ny, Nz, dom.ctypes.data, sig.ctypes.data)
        length, copy, free = L.peec_mesh_len, L.peec_mesh_copy, L.peec_mesh_free
        if not h:
            raise ValueError("mesher rejected the grid")
    else:
        from . import _lib as _glib
        L = _glib.load()
        err = ctypes.c_char_p()
        h = L.peec_mesh_gpu_build(g.ctypes.data, G, Nx, Ny, Nz, dom.ctypes.data,
                                  sig.ctypes.data, int(device), ctypes.byref(err))
        length, copy, free = L.peec_mesh_gpu_len, L.peec_mesh_gpu_copy, L.peec_mesh_gpu_free
        if not h:
            raise RuntimeError((err.value or b"GPU mesher failed").decode())
    out = {}
    try:
        for name in MESH_ARRAYS:
            isd = ctypes.c_int(0)
            n = length(h, name.encode(), ctypes.byref(isd))
            arr = np.empty(n, dtype=np.float64 if isd.value else np.int64)
            if n > 0:
                copy(h, name.encode(), arr.ctypes.data)
            out[name] = arr
    finally:
        free(h)
    return out


# ----------------------------------------------------------------------------------------
# materials / request parsing (src/lib/format_input_output_solver_functions.jl:34-210,
# src/lib/solverFFT/do_solving_fft.jl:1-98)
# ----------------------------------------------------------------------------------------

def get_escal_from(unit: str) -> float:
    return {"m": 1.0, "dm": 1e-1, "cm": 1e-2, "mm": 1e-3, "microm": 1e-6,
            "nanom": 1e-9}.get(unit, 1.0)


def material(d: dict) -> dict:
    tan_d = d.get("tangent_delta_conductivity", 0)
    return {"name": d["name"], "sigmar": float(d["conductivity"]), "tan_D": float(tan_d),
            "eps_re": float(d["permittivity"]), "mur": d.get("permeability", 1), "epsr": 1.0}


def _lp_self(l, W, T):
    """Closed-form partial self inductance of a bar (compute_diagonals.jl:136-155)."""
    w = W / l
    t = T / l
    r = math.sqrt(w * w + t * t)
    aw = math.sqrt(w * w + 1)
    at = math.sqrt(t * t + 1)
    ar = math.sqrt(w * w + t * t + 1)
    mu0 = 4 * math.pi * 1e-7
    ash = math.asinh
    a = 0.25 * (1 / w * ash(w / at) + 1 / t * ash(t / aw) + ash(1 / r))
    b = (1 / 24) * (t * t / w * ash(w / (t * at * (r + ar))) + w * w / t * ash(t / (w * aw * (r + ar)))
                    + t * t / (w * w) * ash(w * w / (t * r * (at + ar)))
                    + w * w / (t * t) * ash(t * t / (w * r * (aw + ar)))
                    + 1 / (w * t * t) * ash(w * t * t / (at * (aw + ar)))
                    + 1 / (t * w * w) * ash(t * w * w / (aw * (at + ar))))
    c = (1 / 6) * (1 / (w * t) * math.atan(w * t / ar) + t / w * math.atan(w / (t * ar))
                   + w / t * math.atan(t / (w * ar)))
    d = (1 / 60) * ((ar + r + t + at) * t * t / ((ar + r) * (r + t) * (t + at) * (at + ar))
                    + (ar + r + w + aw) * w * w / ((ar + r) * (r + w) * (w + aw) * (aw + ar))
                    + (ar + aw + 1 + at) / ((ar + aw) * (aw + 1) * (1 + at) * (at + ar)))
    e = (1 / 20) * (1 / (r + ar) + 1 / (aw + ar) + 1 / (at + ar))
    return 2 * mu0 * l / math.pi * (a + b - c - d - e)


def _log0(v: float) -> float:
    return math.log(v) if v > 0 else (-math.inf if v == 0 else math.nan)


def _surf_surf_para(x1v, y1v, z1, x2v, y2v, z2):
    """Parallel-face Newton integral (compute_Lp_Voxels_QS.jl:695-730), used here
    only for the three P self terms of the mesher (mesher_FFT.jl:114-138)."""
    sol = 0.0
    for c1 in range(2):
        x1 = x1v[c1]
        for c2 in range(2):
            y1 = y1v[c2]
            for c3 in range(2):
                y2 = y2v[c3]
                for c4 in range(2):
                    x2 = x2v[c4]
                    dx, dy, dz = x1 - x2, y1 - y2, z1 - z2
                    R = math.sqrt(dx * dx + dy * dy + dz * dz)
                    t1 = -1 / 6 * (dx * dx + dy * dy - 2 * dz * dz) * R
                    t2 = -dx * dy * abs(dz) * math.atan2(dx * dy, abs(dz) * R)
                    with np.errstate(all="ignore"):
                        t3 = float(np.float64(0.5 * (dx * dx - dz * dz) * dy) * np.float64(_log0(dy + R)))
                        t4 = float(np.float64(0.5 * (dy * dy - dz * dz) * dx) * np.float64(_log0(dx + R)))
                    if not math.isfinite(t3):
                        t3 = 0.0
                    if not math.isfinite(t4):
                        t4 = 0.0
                    sgn = 1.0 if (c1 + c2 + c3 + c4) % 2 == 0 else -1.0
                    sol += sgn * (t1 + t2 + t3 + t4)
    return sol


def p_self_terms(sx, sy, sz):
    """P self terms of the three face families, escaled (mesher_FFT.jl:114-138):
    the face-face integral of a face with itself over 4*pi*eps0*A^2."""
    out = []
    # family 12: faces normal to y, extent sx x sz ; integral in the (x, z) plane
    A = sx * sz
    out.append(ESCALINGS["P"] / (4 * math.pi * EPS0 * A * A) *
               _surf_surf_para([-sx / 2, sx / 2], [-sz / 2, sz / 2], 0.0,
                               [-sx / 2, sx / 2], [-sz / 2, sz / 2], 0.0))
    A = sy * sz
    out.append(ESCALINGS["P"] / (4 * math.pi * EPS0 * A * A) *
               _surf_surf_para([-sy / 2, sy / 2], [-sz / 2, sz / 2], 0.0,
                               [-sy / 2, sy / 2], [-sz / 2, sz / 2], 0.0))
    A = sx * sy
    out.append(ESCALINGS["P"] / (4 * math.pi * EPS0 * A * A) *
               _surf_surf_para([-sx / 2, sx / 2], [-sy / 2, sy / 2], 0.0,
                               [-sx / 2, sx / 2], [-sy / 2, sy / 2], 0.0))
    return out


class LazyCenters(dict):
    """``circulant_centers`` of build_center_P_Voxels.jl:1-111 and
    build_centers_Lp_with_air.jl:1-60; arrays are built on first access.
    Coordinates follow the reference expression order
    ``origin + s*(i-1) + s/2`` (and ``0.5*(A+B)`` for the Lp lattices)."""

    _LAZY = ("p12_se", "p34_se", "p56_se", "p1234", "p1256", "p3456", "Lpx", "Lpy", "Lpz")

    def __init__(self, origin, Nx, Ny, Nz, sx, sy, sz):
        super().__init__(sx=sx, sy=sy, sz=sz, Nx=Nx, Ny=Ny, Nz=Nz, origin=tuple(origin))

    def __contains__(self, k):
        return k in self._LAZY or super().__contains__(k)

    def __missing__(self, key):
        if key not in self._LAZY:
            raise KeyError(key)
        val = lattice_centers(key, self["origin"], self["Nx"], self["Ny"], self["Nz"],
                              self["sx"], self["sy"], self["sz"])
        self[key] = val
        return val


def _axis(o, s, n, half=False):
    i = np.arange(1, n + 1, dtype=np.float64)
    if half:
        i = np.ceil(i / 2)
    return o + s * (i - 1) + s / 2


def lattice_centers(key, origin, Nx, Ny, Nz, sx, sy, sz):
    ox, oy, oz = origin
    if key == "p12_se":
        ax = (_axis(ox, sx, Nx), _axis(oy, sy, Ny + 1), _axis(oz, sz, Nz))
    elif key == "p34_se":
        ax = (_axis(ox, sx, Nx + 1), _axis(oy, sy, Ny), _axis(oz, sz, Nz))
    elif key == "p56_se":
        ax = (_axis(ox, sx, Nx), _axis(oy, sy, Ny), _axis(oz, sz, Nz + 1))
    elif key == "p1234":
        ax = (_axis(ox, sx, 2 * Nx + 1, True), _axis(oy, sy, 2 * Ny + 1, True), _axis(oz, sz, Nz))
    elif key == "p1256":
        ax = (_axis(ox, sx, Nx), _axis(oy, sy, 2 * Ny + 1, True), _axis(oz, sz, 2 * Nz + 1, True))
    elif key == "p3456":
        ax = (_axis(ox, sx, 2 * Nx + 1, True), _axis(oy, sy, Ny), _axis(oz, sz, 2 * Nz + 1, True))
    elif key in ("Lpx", "Lpy", "Lpz"):
        cx, cy, cz = _axis(ox, sx, Nx), _axis(oy, sy, Ny), _axis(oz, sz, Nz)
        if key == "Lpx":
            ax = (0.5 * (cx[:-1] + cx[1:]), 0.5 * (cy + cy), 0.5 * (cz + cz))
        elif key == "Lpy":
            ax = (0.5 * (cx + cx), 0.5 * (cy[:-1] + cy[1:]), 0.5 * (cz + cz))
        else:
            ax = (0.5 * (cx + cx), 0.5 * (cy + cy), 0.5 * (cz[:-1] + cz[1:]))
    else:
        raise KeyError(key)
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return np.stack([X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")], axis=1)


def lattice_dims(Nx, Ny, Nz):
    """Lattice extents of the Lp edge families and P face families / cross lattices."""
    return {
        "Lpx": (Nx - 1, Ny, Nz), "Lpy": (Nx, Ny - 1, Nz), "Lpz": (Nx, Ny, Nz - 1),
        "p12_se": (Nx, Ny + 1, Nz), "p34_se": (Nx + 1, Ny, Nz), "p56_se": (Nx, Ny, Nz + 1),
        "p1234": (2 * Nx + 1, 2 * Ny + 1, Nz), "p1256": (Nx, 2 * Ny + 1, 2 * Nz + 1),
        "p3456": (2 * Nx + 1, Ny, 2 * Nz + 1),
    }


def _f1d(i, j, k, M, N):
    """from_3D_to_1D with 0-based inputs and output."""
    return (k * M * N) + (j * M) + i


def mesher_FFT(materials, sx, sy, sz, grids, ports, lumped_elements, origin, dominant_list,
               build_full_expansions=True, device=None):
    """Host mesher producing the structures of mesher_FFT.jl:1-112.

    grids: (G, Nx, Ny, Nz) bool, in the same order as ``materials`` (the reference
    indexes materials by grid index). ``ports`` / ``lumped_elements``: dicts with
    ``port_start``/``port_end`` (or ``le_*``) as (np, 3) coordinate arrays.
    """
    grids = np.asarray(grids, dtype=bool)
    G, Nx, Ny, Nz = grids.shape
    for mt in materials:
        mt["epsr"] = mt["eps_re"] - 1j * mt["eps_re"] * mt["tan_D"]  # mesher_FFT.jl:20-22
    dominant = np.zeros(G, dtype=np.uint8)
    dominant[list(dominant_list)] = 1
    sigma = [materials[k]["sigmar"] for k in range(G)]
    raw = _raw_mesh(grids, dominant, sigma, device)
    num_vox, n, mx, my, mz, N1, N2, N3 = (int(v) for v in raw["counts"])
    m = mx + my + mz
    ns = N1 + N2 + N3

    # incidence A (create_A_mats_and_find_borders_with_map_Zs.jl:227)
    rows = np.repeat(np.arange(m), 2)
    cols = np.stack([raw["edge_n1"], raw["edge_n2"]], axis=1).ravel()
    vals = np.tile([-1.0, 1.0], m)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    # Gamma (create_mapping_Gamma_no_rep.jl:381)
    Gamma = sp.csc_matrix((np.ones(ns), (raw["surf_node"], np.arange(ns))), shape=(n, ns))
    incidence_selection = {"A": A, "Gamma": Gamma, "mx": mx, "my": my, "mz": mz}

    dims = lattice_dims(Nx, Ny, Nz)
    edge_cell = raw["edge_cell"]
    offs = [0, mx, mx + my, m]
    mat_map = [[None] * 3 for _ in range(3)]
    N_ind = [int(np.prod(dims[k])) for k in ("Lpx", "Lpy", "Lpz")]
    for c in range(3):
        mc = offs[c + 1] - offs[c]
        mat_map[c][0] = sp.csc_matrix((np.ones(mc), (edge_cell[offs[c]:offs[c + 1]], np.arange(mc))),
                                      shape=(N_ind[c], mc))
    surf_cell = raw["surf_cell"]
    fam = raw["surf_fam"]
    exp_P = [[None] * 3 for _ in range(3)]
    sidx = np.arange(ns)
    fam_keys = ("p12_se", "p34_se", "p56_se")
    fam_sel = [fam == f for f in range(3)]
    for f in range(3):
        rows_f = surf_cell[fam_sel[f]]
        exp_P[f][f] = sp.csr_matrix((np.ones(rows_f.size), (rows_f, sidx[fam_sel[f]])),
                                    shape=(int(np.prod(dims[fam_keys[f]])), ns))
    if build_full_expansions:
        # cross lattices (create_mapping_Gamma_no_rep.jl:36-37,63-64,... placements)
        def fam_coords(f):
            d = dims[fam_keys[f]]
            c = surf_cell[fam_sel[f]]
            return c % d[0], (c // d[0]) % d[1], c // (d[0] * d[1]), sidx[fam_sel[f]]

        def place(lat, coords, sx_, sy_, sz_):
            d = dims[lat]
            x, y, z, s = coords
            r = _f1d(sx_(x), sy_(y), sz_(z), d[0], d[1])
            return sp.csr_matrix((np.ones(s.size), (r, s)), shape=(int(np.prod(d)), ns))

        c12, c34, c56 = fam_coords(0), fam_coords(1), fam_coords(2)
        ev = lambda a: 2 * a + 1   # 1-based 2c   -> 0-based 2c-1
        od = lambda a: 2 * a       # 1-based 2c-1 -> 0-based 2c-2
        idn = lambda a: a
        exp_P[1][0] = place("p1234", c12, ev, od, idn)
        exp_P[0][1] = place("p1234", c34, od, ev, idn)
        exp_P[2][0] = place("p1256", c12, idn, od, ev)
        exp_P[0][2] = place("p1256", c56, idn, ev, od)
        exp_P[2][1] = place("p3456", c34, od, idn, ev)
        exp_P[1][2] = place("p3456", c56, ev, idn, od)
    expansions = {"mat_map_Lp": mat_map, "N_ind": N_ind, "exp_P": exp_P,
                  "N1": N1, "N2": N2, "N3": N3,
                  # compact lattice placement used by the GPU operator
                  "edge_cell": edge_cell, "surf_cell": surf_cell, "surf_fam": fam,
                  "grid": (Nx, Ny, Nz),
                  # voxel number (1-based, 0 empty) per lattice cell, x fastest
                  "vox_map": np.asarray(raw["vox_map"])}

    # diagonals (compute_diagonals.jl:1-134)
    mats = raw["edge_mat"]
    b1, b2 = raw["edge_border1"], raw["edge_border2"]
    R = np.zeros((m, 4))
    Cd = np.zeros((m, 4), dtype=np.complex128)
    s_of = [(sx, sy, sz), (sy, sx, sz), (sz, sy, sx)]
    for c in range(3):
        sl = slice(offs[c], offs[c + 1])
        for kk, mt in enumerate(materials):
            k1 = kk + 1
            sig, epsr = mt["sigmar"], mt["epsr"]
            l_, a_, b_ = s_of[c]
            Rv = 0.5 * l_ / (sig * a_ * b_) if sig != 0 else 0.0
            if sig != 0 and epsr == 1:
                Cv = 0.0
            else:
                Cv = EPS0 * (epsr - 1) * a_ * b_ / (0.5 * l_)
            for col, arr in ((0, mats), (1, mats), (2, b1), (3, b2)):
                sel = np.nonzero(arr[sl] == k1)[0] + offs[c]
                if Rv != 0:
                    R[sel, col] = Rv
                if Cv != 0:
                    Cd[sel, col] = Cv
    aux = (b1 != 0).astype(int) + (b2 != 0).astype(int)
    selfs = []
    for c in range(3):
        l_, a_, b_ = s_of[c]
        selfs.append((_lp_self(l_, a_, b_), _lp_self(l_ + l_ / 2, a_, b_), _lp_self(2 * l_, a_, b_)))
    dLp = np.empty(m)
    for c in range(3):
        sl = slice(offs[c], offs[c + 1])
        dLp[sl] = np.choose(aux[sl], selfs[c])
    base = np.concatenate([np.full(offs[c + 1] - offs[c], selfs[c][0]) for c in range(3)])
    Pself = p_self_terms(sx, sy, sz)
    diagonals = {"R": ESCALINGS["R"] * R, "Cd": ESCALINGS["Cd"] * Cd,
                 "Lp": ESCALINGS["Lp"] * dLp, "fc_Lp": ESCALINGS["Lp"] * (dLp - base),
                 "P": np.concatenate([np.full(N1, Pself[0]), np.full(N2, Pself[1]),
                                      np.full(N3, Pself[2])])}

    # surface impedance (compute_Zs_with_indices.jl)
    Zs_info = _compute_zs(materials, mats, b1, b2, raw["edge_zs"].reshape(m, 4), offs, sx, sy, sz)

    # ports / lumped elements (find_voxels_port_pp.jl)
    vox_cells = np.nonzero(raw["vox_map"])[0]  # ordered by voxel number
    vx, vy, vz = vox_cells % Nx, (vox_cells // Nx) % Ny, vox_cells // (Nx * Ny)
    centri_vox = np.stack([origin[0] + sx * vx + sx / 2, origin[1] + sy * vy + sy / 2,
                           origin[2] + sz * vz + sz / 2], axis=1)
    vox_node = raw["vox_node"]

    def nearest(pt, skip):
        # the first voxel (in voxel order) nearest to pt, skipping `skip`: the first entry of
        # a stable sort by distance that is not `skip` (find_voxels_port_pp.jl:6-7)
        d = np.sqrt(np.sum((centri_vox - np.asarray(pt, dtype=np.float64)[None, :]) ** 2, axis=1))
        if skip >= 0:
            d[skip] = np.inf
        return int(np.argmin(d))

    ports = dict(ports)
    P0 = np.asarray(ports["port_start"], dtype=np.float64).reshape(-1, 3)
    P1 = np.asarray(ports["port_end"], dtype=np.float64).reshape(-1, 3)
    pv = np.zeros((P0.shape[0], 2), dtype=np.int64)
    for c in range(P0.shape[0]):
        pv[c, 0] = nearest(P0[c], -1)
        pv[c, 1] = nearest(P1[c], pv[c, 0])
    ports["port_voxels"] = pv
    ports["port_nodes"] = vox_node[pv]
    le = dict(lumped_elements)
    L0 = np.asarray(le.get("le_start", np.zeros((0, 3))), dtype=np.float64).reshape(-1, 3)
    L1 = np.asarray(le.get("le_end", np.zeros((0, 3))), dtype=np.float64).reshape(-1, 3)
    lv = np.zeros((L0.shape[0], 2), dtype=np.int64)
    for c in range(L0.shape[0]):
        lv[c, 0] = nearest(L0[c], -1)
        lv[c, 1] = nearest(L1[c], lv[c, 0])
    le["le_voxels"] = lv
    le["le_nodes"] = vox_node[lv] if lv.size else np.zeros((0, 2), dtype=np.int64)

    circulant_centers = LazyCenters(origin, Nx, Ny, Nz, sx, sy, sz)
    li_mats = {"lix_mat": mats[:mx], "liy_mat": mats[mx:mx + my], "liz_mat": mats[mx + my:],
               "border1": b1, "border2": b2, "sx": sx, "sy": sy, "sz": sz}
    return (dict(ESCALINGS), incidence_selection, circulant_centers, diagonals, expansions,
            ports, le, li_mats, Zs_info)


def _compute_zs(materials, mats, b1, b2, zs, offs, sx, sy, sz):
    m = mats.size
    Zsw = np.zeros((m, 4), dtype=np.complex128)
    cont_fac = [(sx / sy, sx / sz), (sy / sx, sy / sz), (sz / sx, sz / sy)]
    for kk, mt in enumerate(materials):
        sig = mt["sigmar"]
        if sig == 0:
            continue
        k1 = kk + 1
        base = (1 + 1j) * math.sqrt(2 * math.pi * 1e-7 / sig)
        for c in range(3):
            sl = np.arange(offs[c], offs[c + 1])
            ca, cb = 0.5 * cont_fac[c][0] * base, 0.5 * cont_fac[c][1] * base
            inm = mats[sl] == k1
            # columns: 1 <- kind a side 1, 3 <- kind a side 2, 2 <- kind b side 1, 4 <- kind b side 2
            for col, cnt, val, brd in ((0, zs[sl, 0], ca, b1), (2, zs[sl, 1], ca, b2),
                                       (1, zs[sl, 2], cb, b1), (3, zs[sl, 3], cb, b2)):
                sel = inm & (cnt > 0)
                e = sl[sel]
                Zsw[e, col] = val
                dbl = e[brd[e] == k1]
                Zsw[dbl, col] = 2 * Zsw[dbl, col]

    def par(a, b):
        out = a + b
        both = (np.abs(a) != 0) & (np.abs(b) != 0)
        out[both] = a[both] * b[both] / (a[both] + b[both])
        return out

    Zs = par(Zsw[:, 0], Zsw[:, 1]) + par(Zsw[:, 2], Zsw[:, 3])
    internal = np.nonzero(np.abs(Zs) == 0)[0]
    surface = np.nonzero(np.abs(Zs) != 0)[0]
    # Zsw: the four contributions per edge (columns 0, 1 lie in the edge's first voxel,
    # 2, 3 in its second), kept for conductivity derivatives
    return {"Zs": Zs, "internal_edges": internal, "surface_edges": surface,
            "materials": mats.copy(), "Zsw": Zsw}


# ----------------------------------------------------------------------------------------
# request parsing
# ----------------------------------------------------------------------------------------

def parse_request(req: dict, device=None):
    """Reads a solve request body (mesherOutput / solverInput / solverAlgoParams) the way
    doSolvingFFT does (do_solving_fft.jl:1-98) and runs the mesher.

    Grid order is the JSON key order of ``mesher_matrices`` (the reference iterates a
    Julia Dict there); ``materials`` is indexed by that grid order, as in the reference.
    device: None meshes on the host (C++); an int meshes on that GPU (the same arrays).
    """
    mo, si = req["mesherOutput"], req["solverInput"]
    escal = get_escal_from(si.get("unit", "m"))
    cs = mo["cell_size"]
    sx, sy, sz = cs["cell_size_x"] * escal, cs["cell_size_y"] * escal, cs["cell_size_z"] * escal
    o = mo["origin"]
    origin = (o["origin_x"], o["origin_y"], o["origin_z"])
    MATERIALS = [material(el) for el in si["materials"]]
    names = list(mo["mesher_matrices"].keys())
    if not names:
        raise ValueError("mesher_matrices holds no material grid")
    arrs = [np.asarray(mo["mesher_matrices"][k], dtype=bool) for k in names]
    shapes = {a.shape for a in arrs}
    if len(shapes) != 1 or len(arrs[0].shape) != 3:
        raise ValueError(f"material grids must share one 3-D shape, got {sorted(shapes)}")
    grids = np.stack(arrs)
    nc = mo.get("n_cells")
    if nc is not None:
        want = (int(nc["n_cells_x"]), int(nc["n_cells_y"]), int(nc["n_cells_z"]))
        if grids.shape[1:] != want:
            raise ValueError(f"material grids are {grids.shape[1:]}, n_cells says {want}")
    if not grids.any():
        raise ValueError("the material grids hold no occupied voxel")
    by_name = {mt["name"]: mt for mt in MATERIALS}
    missing = [nm for nm in names if nm not in by_name]
    if missing:
        raise ValueError(f"mesher_matrices names {missing} that solverInput.materials lacks")
    dominant = [i for i, nm in enumerate(names) if by_name[nm]["sigmar"] > 0]
    ports = {"port_start": np.array([[v * escal for v in p["inputElement"]] for p in si["ports"]]).reshape(-1, 3),
             "port_end": np.array([[v * escal for v in p["outputElement"]] for p in si["ports"]]).reshape(-1, 3)}
    les = si.get("lumped_elements", [])
    lumped = {"le_start": np.array([[v * escal for v in p["inputElement"]] for p in les]).reshape(-1, 3),
              "le_end": np.array([[v * escal for v in p["outputElement"]] for p in les]).reshape(-1, 3),
              "type": np.array([int(p["type"]) for p in les], dtype=np.int64),
              "R_value": np.array([float(p["rlcParams"].get("resistance", 0.0)) for p in les]),
              "L_value": np.array([float(p["rlcParams"].get("inductance", 0.0)) for p in les]),
              "C_value": np.array([float(p["rlcParams"].get("capacitance", 0.0)) for p in les])}
    out = mesher_FFT(MATERIALS, sx, sy, sz, grids, ports, lumped, origin, dominant,
                     device=device)
    ap = req.get("solverAlgoParams", {})
    settings = {"Inner_Iter": int(ap.get("innerIteration", 100)),
                "Outer_Iter": int(ap.get("outerIteration", 1)),
                "tol": float(ap.get("convergenceThreshold", 1e-4))}
    freqs = np.asarray(si["frequencies"], dtype=np.float64)
    z0 = float(si.get("ports_scattering_value", 50.0))
    return out, freqs, settings, z0, (grids.shape[1], grids.shape[2], grids.shape[3])


def load_request(path) -> dict:
    return json.loads(Path(path).read_text())
