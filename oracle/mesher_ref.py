"""ORACLE -- test infrastructure only.

CPU restatement of the reference voxel mesher and request reader of the FFT-PEEC path
(src/lib/solverFFT/do_solving_fft.jl:1-98, mesher_FFT.jl:1-138 and the helpers it
calls), written from the reference sources and independent of the product's mesher
(solver_gb300/csrc/mesher.cpp). tests/test_oracle_mesher.py holds the two equal, index
for index; the oracle's solves, the fixture generator and bench.py's CPU arms build
their topology from here.

The reference walks voxels in nested loops; here each loop nest becomes array
operations over the same positions, enumerated in the same loop order where the order
fixes a numbering (nodes, surfaces, edges). Every function cites the reference lines it
follows. Reference indices are 1-based; arrays here are 0-based, and the 1-based
formulas are kept where they define a number (node ids, lattice positions).

Parity status: parity unpinned (the reference cannot run here, and it ships no outputs
for this path). Two things are left out because nothing on the path reads them: the
"rug" index lists of compute_Zs_with_indices.jl (which need maps_Zs columns 3-4) and
the surface-port fields set to empty at mesher_FFT.jl:95-99.
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp

EPS0 = 8.854187816997944e-12  # compute_diagonals.jl:5


# ----------------------------------------------------------------------------------------
# small helpers (From_3D_to_1D.jl, bin_search.jl)
# ----------------------------------------------------------------------------------------

def from_3D_to_1D(i, j, k, M, N):
    """From_3D_to_1D.jl:1-3, 1-based in and out."""
    return (k - 1) * M * N + (j - 1) * M + i


def bin_search(vals, sorted_arr):
    """bin_search.jl:1-6 over arrays: the 1-based position of each value in sorted_arr,
    0 where it is absent."""
    vals = np.asarray(vals)
    pos = np.searchsorted(sorted_arr, vals, side="left")
    inside = pos < sorted_arr.size
    hit = np.zeros(vals.shape, dtype=bool)
    hit[inside] = sorted_arr[pos[inside]] == vals[inside]
    return np.where(hit, pos + 1, 0).astype(np.int64)


def _sh(a, axis, d):
    """b[i] = a[i + d] along axis, False outside the grid."""
    out = np.zeros_like(a)
    n = a.shape[axis]
    src = [slice(None)] * a.ndim
    dst = [slice(None)] * a.ndim
    if d > 0:
        src[axis], dst[axis] = slice(d, n), slice(0, n - d)
    else:
        src[axis], dst[axis] = slice(0, n + d), slice(-d, n)
    out[tuple(dst)] = a[tuple(src)]
    return out


def _coord(shape, axis):
    """0-based coordinate along axis, broadcast to shape."""
    s = [1] * len(shape)
    s[axis] = shape[axis]
    return np.arange(shape[axis]).reshape(s) * np.ones(shape, dtype=np.int64)


def _others(g, k):
    """OR of the grids other than k."""
    G = g.shape[0]
    out = np.zeros(g.shape[1:], dtype=bool)
    for k2 in range(G):
        if k2 != k:
            out |= g[k2]
    return out


def _first_k(conds):
    """Per position, the first k whose condition holds (the reference's `for k ... break`),
    and whether any does."""
    c = np.stack(conds)
    return c.any(0), np.argmax(c, axis=0)


# ----------------------------------------------------------------------------------------
# volumes, centres and exposed faces (create_volumes_mapping.jl, create_volume_centers.jl,
# create_Grids_externals.jl)
# ----------------------------------------------------------------------------------------

def create_volumes_mapping(g):
    """create_volumes_mapping.jl:1-23: voxel numbers in x-fastest order, 0 for empty."""
    occ = g.any(0).ravel(order="F")
    mapping = np.where(occ, np.cumsum(occ), 0).astype(np.int64)
    return mapping, int(occ.sum())


def create_volume_centers(g, mapping, num_centri, sx, sy, sz, min_v):
    """create_volume_centers.jl:1-25: centre of each voxel, by voxel number."""
    G, Nx, Ny, Nz = g.shape
    occ = g.any(0)
    x, y, z = np.nonzero(occ)
    lin = x + Nx * y + Nx * Ny * z
    pos = mapping[lin] - 1
    c = np.zeros((num_centri, 3))
    c[pos, 0] = min_v[0] + sx * x + sx / 2
    c[pos, 1] = min_v[1] + sy * y + sy / 2
    c[pos, 2] = min_v[2] + sz * z + sz / 2
    return c


def create_Grids_externals(g):
    """create_Grids_externals.jl:1-181: per grid the six exposed-face flags
    (faces 1/2: -y/+y, 3/4: -x/+x, 5/6: -z/+z); a face is exposed at the grid boundary
    or where the neighbour is not of the same grid."""
    G, Nx, Ny, Nz = g.shape
    ext = np.zeros((G, 6, Nx, Ny, Nz), dtype=bool)
    for k in range(G):
        a = g[k]
        ext[k, 0] = a & ~_sh(a, 1, -1)   # y = 0: the shifted array is False there
        ext[k, 1] = a & ~_sh(a, 1, +1)
        ext[k, 2] = a & ~_sh(a, 0, -1)
        ext[k, 3] = a & ~_sh(a, 0, +1)
        ext[k, 4] = a & ~_sh(a, 2, -1)
        ext[k, 5] = a & ~_sh(a, 2, +1)
    return ext


# ----------------------------------------------------------------------------------------
# nodes (create_nodes_ref.jl:1-489)
# ----------------------------------------------------------------------------------------

# build_nodes (create_nodes_ref.jl:433-489): the 26 neighbour offsets in the order tried
_NEIGH26 = [(-1, -1, -1), (-1, -1, 0), (-1, -1, 1), (0, -1, -1), (0, -1, 0), (0, -1, 1),
            (1, -1, -1), (1, -1, 0), (1, -1, 1), (-1, 0, -1), (-1, 0, 0), (-1, 0, 1),
            (0, 0, -1), (0, 0, 1), (1, 0, -1), (1, 0, 0), (1, 0, 1), (-1, 1, -1),
            (-1, 1, 0), (-1, 1, 1), (0, 1, -1), (0, 1, 0), (0, 1, 1), (1, 1, -1),
            (1, 1, 0), (1, 1, 1)]


def _face_flags(g, ext, k):
    """is_f1..is_f6 of grid k (create_nodes_ref.jl:14-116): the exposed faces, with an
    exposed pair on one axis resolved by which side touches another grid's exposed face.
    The neighbour tests use `cont - 1 > 1` (not >= 1) on the low side, as written."""
    G, Nx, Ny, Nz = g.shape
    shape = (Nx, Ny, Nz)
    xs, ys, zs = _coord(shape, 0), _coord(shape, 1), _coord(shape, 2)
    oth = [k2 for k2 in range(G) if k2 != k]

    def any_other(face, axis, d, ok):
        out = np.zeros(shape, dtype=bool)
        for k2 in oth:
            out |= _sh(ext[k2, face], axis, d)
        return out & ok

    f = [ext[k, i] for i in range(6)]
    fc = [any_other(1, 1, -1, ys - 1 > 0),        # f1_c: cont2 - 1 > 1 (1-based)
          any_other(0, 1, +1, ys + 2 <= Ny),      # f2_c: cont2 + 1 <= Ny
          any_other(3, 0, -1, xs - 1 > 0),        # f3_c
          any_other(2, 0, +1, xs + 2 <= Nx),      # f4_c
          any_other(5, 2, -1, zs - 1 > 0),        # f5_c
          any_other(4, 2, +1, zs + 2 <= Nz)]      # f6_c
    isf = list(f)
    for a, b in ((0, 1), (2, 3), (4, 5)):
        both = f[a] & f[b]
        isf[a] = np.where(both, fc[a] & ~fc[b], f[a])
        isf[b] = np.where(both, ~fc[a] & fc[b], f[b])
    return isf


def _offset_node(isf, c1, c2, c3, M3, N3):
    """The node on the exposed corner / edge / face of the voxel
    (create_nodes_ref.jl:118-221): -1 / +1 along each axis with an exposed face."""
    dx = np.where(isf[2], -1, np.where(isf[3], 1, 0))
    dy = np.where(isf[0], -1, np.where(isf[1], 1, 0))
    dz = np.where(isf[4], -1, np.where(isf[5], 1, 0))
    return from_3D_to_1D(c1 + dx, c2 + dy, c3 + dz, M3, N3)


def create_nodes_ref(g, num_full_vox, ext, mapping, dominant_list):
    """create_nodes_ref.jl:1-418. Conductor grids (dominant) place each voxel's node on
    its exposed corner, edge or face; the other grids reuse a neighbouring conductor
    boundary node when one of the 26 neighbours holds one (in build_nodes order), and
    otherwise place theirs the same way. Interior voxels keep the centre node. Node ids
    are positions in a 3Nx x 3Ny x ... lattice; later grids overwrite earlier ones."""
    G, Nx, Ny, Nz = g.shape
    nodes = np.zeros(num_full_vox, dtype=np.int64)
    M3, N3 = 3 * Nx, 3 * Ny
    lista = []
    order = list(dominant_list)
    for k in order:
        x, y, z = np.nonzero(g[k])
        if x.size == 0:
            continue
        isf = [a[x, y, z] for a in _face_flags(g, ext, k)]
        c1, c2, c3 = 2 * x + 2, 2 * y + 2, 2 * z + 2   # 1 + 2(cont-1) + 1 with cont = i+1
        anyf = isf[0] | isf[1] | isf[2] | isf[3] | isf[4] | isf[5]
        val = np.where(anyf, _offset_node(isf, c1, c2, c3, M3, N3),
                       from_3D_to_1D(c1, c2, c3, M3, N3))
        vox = mapping[x + Nx * y + Nx * Ny * z] - 1
        nodes[vox] = val
        lista.append(val[anyf])
    nodes_red_dom = np.unique(np.concatenate(lista)) if lista else np.zeros(0, dtype=np.int64)
    non_dom = [k for k in range(G) if k not in set(order)]
    reused = []
    for k in non_dom:
        x, y, z = np.nonzero(g[k])
        if x.size == 0:
            continue
        isf = [a[x, y, z] for a in _face_flags(g, ext, k)]
        c1, c2, c3 = 2 * x + 2, 2 * y + 2, 2 * z + 2
        anyf = isf[0] | isf[1] | isf[2] | isf[3] | isf[4] | isf[5]
        # bin_search_mod (create_nodes_ref.jl:420-431): the first of the 26 neighbours
        # that is a conductor boundary node
        found = np.zeros(x.size, dtype=bool)
        shared = np.zeros(x.size, dtype=np.int64)
        for (ox, oy, oz) in _NEIGH26:
            cand = from_3D_to_1D(c1 + ox, c2 + oy, c3 + oz, M3, N3)
            hit = (bin_search(cand, nodes_red_dom) != 0) & ~found
            shared[hit] = cand[hit]
            found |= hit
        own = _offset_node(isf, c1, c2, c3, M3, N3)
        val = np.where(anyf, np.where(found, shared, own), from_3D_to_1D(c1, c2, c3, M3, N3))
        vox = mapping[x + Nx * y + Nx * Ny * z] - 1
        nodes[vox] = val
        reused.append(shared[anyf & found])
    nodes_red = np.unique(nodes)
    nodes_reused_clean = np.unique(np.concatenate(reused)) if reused else np.zeros(0, np.int64)
    return nodes, nodes_red, nodes_reused_clean


# ----------------------------------------------------------------------------------------
# surfaces and Gamma (create_mapping_Gamma_no_rep.jl:1-414)
# ----------------------------------------------------------------------------------------

def create_mapping_Gamma_no_rep(g, mapping, nodes, nodes_red, ext):
    """create_mapping_Gamma_no_rep.jl:1-414: numbers the P surfaces family by family
    (12: faces normal to y, 34: x, 56: z), four position blocks per family in the
    reference's loop order, and places each in its own face lattice and in the two
    interleaved cross lattices. Returns (expansions with exp_P and N1..N3, Gamma) and
    the per-family surface records used by the tests."""
    G, Nx, Ny, Nz = g.shape
    shape = (Nx, Ny, Nz)
    xs, ys, zs = _coord(shape, 0), _coord(shape, 1), _coord(shape, 2)
    nidx = np.zeros(Nx * Ny * Nz, dtype=np.int64)
    occ = mapping > 0
    nidx[occ] = bin_search(nodes[mapping[occ] - 1], nodes_red)
    d12, d34, d56 = (Nx, Ny + 1, Nz), (Nx + 1, Ny, Nz), (Nx, Ny, Nz + 1)
    L1234 = (2 * (Nx + 1) - 1, 2 * (Ny + 1) - 1, Nz)
    L1256 = (Nx, 2 * (Ny + 1) - 1, 2 * (Nz + 1) - 1)
    L3456 = (2 * (Nx + 1) - 1, Ny, 2 * (Nz + 1) - 1)
    maps = {key: np.zeros(int(np.prod(d)), dtype=np.int64) for key, d in
            (("12", d12), ("34", d34), ("56", d56), ("1234", L1234), ("1256", L1256),
             ("3456", L3456))}
    dims = {"12": d12, "34": d34, "56": d56, "1234": L1234, "1256": L1256, "3456": L3456}
    ind_r, ind_c = [], []
    counter = [0]

    def emit(sel, fam, own, crossA, crossB, base):
        """sel: positions (x, y, z arrays, 0-based, in loop order) that get a surface;
        own / crossA / crossB: functions of (x, y, z) giving 1-based lattice coordinates."""
        x, y, z = sel
        num = counter[0] + np.arange(1, x.size + 1)
        counter[0] += x.size
        for key, fn in ((fam, own), crossA, crossB):
            i, j, k = fn(x, y, z)
            d = dims[key]
            maps[key][from_3D_to_1D(i, j, k, d[0], d[1]) - 1] = base + num
        ind_r.append(nidx[x + Nx * y + Nx * Ny * z])
        ind_c.append(base + num)

    def block(mask, conds, extra=None):
        """The positions of `mask` (in C order over x, y, z: x outermost) at which the
        first grid k with conds[k] true exists; extra(k) an extra test on that k
        (the `controllo_altri` of the fourth blocks)."""
        hit, kf = _first_k(conds)
        take = mask & hit
        if extra is not None:
            ok = np.zeros(shape, dtype=bool)
            for k in range(G):
                ok |= (kf == k) & extra(k)
            take &= ok
        x, y, z = np.nonzero(take)  # C order: x outer, z inner
        return x, y, z

    oth = [_others(g, k) for k in range(G)]
    # -- family 12 (faces normal to y), lines 19-136 ------------------------------------
    c1234_12 = lambda x, y, z: (2 * (x + 1), 2 * (y + 1) - 1, z + 1)
    c1256_12 = lambda x, y, z: (x + 1, 2 * (y + 1) - 1, 2 * (z + 1))
    c1234_12u = lambda x, y, z: (2 * (x + 1), 2 * (y + 2) - 1, z + 1)
    c1256_12u = lambda x, y, z: (x + 1, 2 * (y + 2) - 1, 2 * (z + 1))
    own12 = lambda x, y, z: (x + 1, y + 1, z + 1)
    own12u = lambda x, y, z: (x + 1, y + 2, z + 1)
    up = [_sh(o, 1, +1) for o in oth]
    dn = [_sh(o, 1, -1) for o in oth]
    m = ys == 0
    s = block(m, [g[k] & (~ext[k, 1] | (up[k] & (ys + 1 <= Ny - 1))) for k in range(G)])
    emit(s, "12", own12, ("1234", c1234_12), ("1256", c1256_12), 0)
    m = ys >= 1
    s = block(m, [g[k] & ~_sh(g[k], 1, -1) & (~ext[k, 1] | (up[k] & (ys + 1 <= Ny - 1)))
                  for k in range(G)])
    emit(s, "12", own12, ("1234", c1234_12), ("1256", c1256_12), 0)
    m = ys == Ny - 1
    s = block(m, [g[k] & (~ext[k, 0] | (dn[k] & (ys >= 1))) for k in range(G)])
    emit(s, "12", own12u, ("1234", c1234_12u), ("1256", c1256_12u), 0)
    m = ys <= Ny - 2
    s = block(m, [g[k] & ~_sh(g[k], 1, +1) & (~ext[k, 0] | (dn[k] & (ys >= 1)))
                  for k in range(G)], extra=lambda k: ~up[k])
    emit(s, "12", own12u, ("1234", c1234_12u), ("1256", c1256_12u), 0)
    n12 = counter[0]
    # -- family 34 (faces normal to x), lines 137-254 ----------------------------------
    counter[0] = 0
    c1234_34 = lambda x, y, z: (2 * (x + 1) - 1, 2 * (y + 1), z + 1)
    c3456_34 = lambda x, y, z: (2 * (x + 1) - 1, y + 1, 2 * (z + 1))
    c1234_34u = lambda x, y, z: (2 * (x + 2) - 1, 2 * (y + 1), z + 1)
    c3456_34u = lambda x, y, z: (2 * (x + 2) - 1, y + 1, 2 * (z + 1))
    own34 = lambda x, y, z: (x + 1, y + 1, z + 1)
    own34u = lambda x, y, z: (x + 2, y + 1, z + 1)
    up = [_sh(o, 0, +1) for o in oth]
    dn = [_sh(o, 0, -1) for o in oth]
    m = xs == 0
    s = block(m, [g[k] & (~ext[k, 3] | (up[k] & (xs + 1 <= Nx - 1))) for k in range(G)])
    emit(s, "34", own34, ("1234", c1234_34), ("3456", c3456_34), n12)
    m = xs >= 1
    s = block(m, [g[k] & ~_sh(g[k], 0, -1) & (~ext[k, 3] | (up[k] & (xs + 1 <= Nx - 1)))
                  for k in range(G)])
    emit(s, "34", own34, ("1234", c1234_34), ("3456", c3456_34), n12)
    m = xs == Nx - 1
    s = block(m, [g[k] & (~ext[k, 2] | (dn[k] & (xs >= 1))) for k in range(G)])
    emit(s, "34", own34u, ("1234", c1234_34u), ("3456", c3456_34u), n12)
    m = xs <= Nx - 2
    s = block(m, [g[k] & ~_sh(g[k], 0, +1) & (~ext[k, 2] | (dn[k] & (xs >= 1)))
                  for k in range(G)], extra=lambda k: ~up[k])
    emit(s, "34", own34u, ("1234", c1234_34u), ("3456", c3456_34u), n12)
    n34 = counter[0]
    # -- family 56 (faces normal to z), lines 255-372 ----------------------------------
    counter[0] = 0
    c1256_56 = lambda x, y, z: (x + 1, 2 * (y + 1), 2 * (z + 1) - 1)
    c3456_56 = lambda x, y, z: (2 * (x + 1), y + 1, 2 * (z + 1) - 1)
    c1256_56u = lambda x, y, z: (x + 1, 2 * (y + 1), 2 * (z + 2) - 1)
    c3456_56u = lambda x, y, z: (2 * (x + 1), y + 1, 2 * (z + 2) - 1)
    own56 = lambda x, y, z: (x + 1, y + 1, z + 1)
    own56u = lambda x, y, z: (x + 1, y + 1, z + 2)
    up = [_sh(o, 2, +1) for o in oth]
    dn = [_sh(o, 2, -1) for o in oth]
    m = zs == 0
    s = block(m, [g[k] & (~ext[k, 5] | (up[k] & (zs + 1 <= Nz - 1))) for k in range(G)])
    emit(s, "56", own56, ("1256", c1256_56), ("3456", c3456_56), n12 + n34)
    m = zs >= 1
    s = block(m, [g[k] & ~_sh(g[k], 2, -1) & (~ext[k, 5] | (up[k] & (zs + 1 <= Nz - 1)))
                  for k in range(G)])
    emit(s, "56", own56, ("1256", c1256_56), ("3456", c3456_56), n12 + n34)
    m = zs == Nz - 1
    s = block(m, [g[k] & (~ext[k, 4] | (dn[k] & (zs >= 1))) for k in range(G)])
    emit(s, "56", own56u, ("1256", c1256_56u), ("3456", c3456_56u), n12 + n34)
    m = zs <= Nz - 2
    s = block(m, [g[k] & ~_sh(g[k], 2, +1) & (~ext[k, 4] | (dn[k] & (zs >= 1)))
                  for k in range(G)], extra=lambda k: ~up[k])
    emit(s, "56", own56u, ("1256", c1256_56u), ("3456", c3456_56u), n12 + n34)
    n56 = counter[0]

    ns = n12 + n34 + n56
    r = np.concatenate(ind_r) - 1
    c = np.concatenate(ind_c) - 1
    Gamma = sp.csc_matrix((np.ones(r.size), (r, c)), shape=(nodes_red.size, ns))

    def expand(key, sel):
        mp = maps[key]
        inn = np.nonzero(sel(mp))[0]
        return sp.csr_matrix((np.ones(inn.size), (inn, mp[inn] - 1)), shape=(mp.size, ns))

    E = [[None] * 3 for _ in range(3)]
    E[0][0] = expand("12", lambda v: v != 0)
    E[1][1] = expand("34", lambda v: v != 0)
    E[2][2] = expand("56", lambda v: v != 0)
    E[1][0] = expand("1234", lambda v: (v <= n12) & (v != 0))
    E[0][1] = expand("1234", lambda v: v > n12)
    E[2][0] = expand("1256", lambda v: (v <= n12) & (v != 0))
    E[0][2] = expand("1256", lambda v: v > n12 + n34)
    E[2][1] = expand("3456", lambda v: (v <= n12 + n34) & (v != 0))
    E[1][2] = expand("3456", lambda v: v > n12 + n34)
    exp_mat = {"exp_P": E, "N1": int(np.count_nonzero(maps["12"])),
               "N2": int(np.count_nonzero(maps["34"])), "N3": int(np.count_nonzero(maps["56"]))}
    return exp_mat, Gamma, maps


# ----------------------------------------------------------------------------------------
# edges, incidence A, borders and surface-impedance counts
# (create_mapping_A{x,y,z}_v2.jl, create_A_mats_and_find_borders_with_map_Zs.jl:1-425,
# create_expansion_ind_Lp_{x,y,z}_grids_v2.jl)
# ----------------------------------------------------------------------------------------

def _edges(g, mapping, nodes, nodes_red, axis, number_order, materials):
    """Edges along `axis` between two voxels of one grid whose nodes differ. Numbered in
    the loop order of create_mapping_A{x,y,z}_v2.jl (number_order: the axes from outer to
    inner). Returns per edge (in number order): lattice position (0-based, lattice of
    extent N-1 along axis, x fastest), the two node indices (1-based), the first grid k
    joining the two voxels, the border grids and the surface-impedance face counts."""
    G, Nx, Ny, Nz = g.shape
    shape = [Nx, Ny, Nz]
    lat = list(shape)
    lat[axis] -= 1
    sl0 = [slice(None)] * 3
    sl1 = [slice(None)] * 3
    sl0[axis] = slice(0, shape[axis] - 1)
    sl1[axis] = slice(1, shape[axis])
    sl0, sl1 = tuple(sl0), tuple(sl1)
    occ = g.any(0)
    nid = np.zeros(Nx * Ny * Nz, dtype=np.int64)
    lin_occ = mapping > 0
    nid[lin_occ] = nodes[mapping[lin_occ] - 1]
    node3 = nid.reshape((Nx, Ny, Nz), order="F")
    n1, n2 = node3[sl0], node3[sl1]
    both = [g[k][sl0] & g[k][sl1] for k in range(G)]
    hit, kf = _first_k(both)
    exists = hit & (n1 != n2)
    # numbering order: transpose to (outer, middle, inner) and take C order
    perm = list(number_order)
    ex_t = np.transpose(exists, perm)
    idx = np.nonzero(ex_t)
    coords = [None] * 3
    for p, a in enumerate(perm):
        coords[a] = idx[p]
    x, y, z = coords
    lpos = x + lat[0] * y + lat[0] * lat[1] * z
    k_e = kf[x, y, z]
    nn1 = bin_search(n1[x, y, z], nodes_red)
    nn2 = bin_search(n2[x, y, z], nodes_red)
    # borders (create_A_mats...:125-138, 264-276, 403-415)
    c = coords[axis]
    N = shape[axis]

    def occ_k(dx, dy, dz):
        """g[k_e] at the edge's first voxel + offset, False outside the grid."""
        xx, yy, zz = x + dx, y + dy, z + dz
        inside = (xx >= 0) & (xx < Nx) & (yy >= 0) & (yy < Ny) & (zz >= 0) & (zz < Nz)
        out = np.zeros(x.size, dtype=bool)
        out[inside] = g[k_e[inside], xx[inside], yy[inside], zz[inside]]
        return out

    o = [0, 0, 0]
    o[axis] = -1
    b1 = np.where((c == 0) | ((c > 0) & ~occ_k(*o)), k_e + 1, 0)
    o = [0, 0, 0]
    o[axis] = 2
    b2 = np.where(c + 1 == N - 1, k_e + 1,
                  np.where((c + 2 <= N - 1) & ~occ_k(*o), k_e + 1, 0))
    # surface-impedance face counts (maps_Zs columns 1-2): for each of the two transverse
    # axes, faces of the edge's two voxels not covered by the same grid; a voxel on the
    # grid boundary of that axis counts one face, its neighbours unchecked
    sig = np.array([materials[k]["sigmar"] for k in range(G)])
    cond = sig[k_e] != 0
    counts = {}
    pos = [x, y, z]
    for t in range(3):
        if t == axis:
            continue
        ct = pos[t]
        Nt = shape[t]
        bnd = (ct == 0) | (ct == Nt - 1)
        c1 = np.zeros(x.size, dtype=np.int64)
        c2 = np.zeros(x.size, dtype=np.int64)
        c1[bnd] += 1
        c2[bnd] += 1
        inner = ~bnd
        for d in (-1, 1):
            od = [0, 0, 0]
            od[t] = d
            c1 += inner & ~occ_k(*od)
            od2 = list(od)
            # second voxel of the edge, shifted along t; z edges test the first voxel's
            # +t neighbour instead for d = +1 (create_A_mats...:346,391, as written)
            if not (axis == 2 and d == 1):
                od2[axis] += 1
            c2 += inner & ~occ_k(*od2)
        counts[t] = (np.where(cond, c1, 0), np.where(cond, c2, 0))
    return {"lpos": lpos, "nn1": nn1, "nn2": nn2, "k": k_e + 1, "b1": b1, "b2": b2,
            "counts": counts, "lat": tuple(lat)}


# ----------------------------------------------------------------------------------------
# diagonals and surface impedance (compute_diagonals.jl:1-155, compute_Zs_with_indices.jl)
# ----------------------------------------------------------------------------------------

def Lp_self(l, W, T):
    """compute_diagonals.jl:136-155, the closed-form partial self inductance of a bar
    of length l and cross-section W x T, in the reference's expression order."""
    w = W / l
    t = T / l
    r = math.sqrt(w ** 2 + t ** 2)
    aw = math.sqrt(w ** 2 + 1)
    at = math.sqrt(t ** 2 + 1)
    ar = math.sqrt(w ** 2 + t ** 2 + 1)
    mu0 = 4 * math.pi * 1e-7
    Lp = 2 * mu0 * l / math.pi * (
        1 / 4 * (1 / w * math.asinh(w / at) + 1 / t * math.asinh(t / aw) + math.asinh(1 / r))
        + 1 / 24 * (t ** 2 / w * math.asinh(w / (t * at * (r + ar)))
                    + w ** 2 / t * math.asinh(t / (w * aw * (r + ar)))
                    + t ** 2 / w ** 2 * math.asinh(w ** 2 / (t * r * (at + ar)))
                    + w ** 2 / t ** 2 * math.asinh(t ** 2 / (w * r * (aw + ar)))
                    + 1 / (w * t ** 2) * math.asinh(w * t ** 2 / (at * (aw + ar)))
                    + 1 / (t * w ** 2) * math.asinh(t * w ** 2 / (aw * (at + ar))))
        - 1 / 6 * (1 / (w * t) * math.atan(w * t / ar) + t / w * math.atan(w / (t * ar))
                   + w / t * math.atan(t / (w * ar)))
        - 1 / 60 * ((ar + r + t + at) * t ** 2 / ((ar + r) * (r + t) * (t + at) * (at + ar))
                    + (ar + r + w + aw) * w ** 2 / ((ar + r) * (r + w) * (w + aw) * (aw + ar))
                    + (ar + aw + 1 + at) / ((ar + aw) * (aw + 1) * (1 + at) * (at + ar)))
        - 1 / 20 * (1 / (r + ar) + 1 / (aw + ar) + 1 / (at + ar)))
    return Lp


def compute_diagonals(escalings, materials, sx, sy, sz, li_mat, li_border):
    """compute_diagonals.jl:1-134. li_mat / li_border: per direction (x, y, z) the edge
    grid numbers (1-based) and border grids."""
    lens = [(sx, sy, sz), (sy, sx, sz), (sz, sy, sx)]
    Rd, Cd, Lpd, base = [], [], [], []
    for c in range(3):
        me = li_mat[c]
        b1, b2 = li_border[c]
        R = np.zeros((me.size, 4))
        C = np.zeros((me.size, 4), dtype=np.complex128)
        for kk, mt in enumerate(materials):
            sig, epsr = mt["sigmar"], mt["epsr"]
            l_, a_, b_ = lens[c]
            if sig != 0:
                Rv = 0.5 * l_ / (sig * a_ * b_)
                # compute_diagonals.jl:10-12: Rx = 0.5*sx/(sigmar*sy*sz),
                # Ry = 0.5*sy/(sigmar*sx*sz), Rz = 0.5*sz/(sigmar*sy*sx)
                Cv = 0 if epsr == 1 else EPS0 * (epsr - 1) * a_ * b_ / (0.5 * l_)
            else:
                Rv = 0
                Cv = EPS0 * (epsr - 1) * a_ * b_ / (0.5 * l_)
            k1 = kk + 1
            for col, arr in ((0, me), (1, me), (2, b1), (3, b2)):
                sel = arr == k1
                if Rv != 0:
                    R[sel, col] = Rv
                if Cv != 0:
                    C[sel, col] = Cv
        Rd.append(R)
        Cd.append(C)
        aux = np.ceil(b1 / 100).astype(int) + np.ceil(b2 / 100).astype(int)
        l_, a_, b_ = lens[c]
        s0, s1, s2 = Lp_self(l_, a_, b_), Lp_self(l_ + l_ / 2, a_, b_), Lp_self(2 * l_, a_, b_)
        d = np.full(me.size, s0)
        d[aux == 1] = s1
        d[aux == 2] = s2
        Lpd.append(d)
        base.append(np.full(me.size, s0))
    Lp = np.concatenate(Lpd)
    return {"R": escalings["R"] * np.concatenate(Rd), "Cd": escalings["Cd"] * np.concatenate(Cd),
            "Lp": escalings["Lp"] * Lp,
            "fc_Lp": escalings["Lp"] * (Lp - np.concatenate(base))}


def compute_Zs(materials, li_mat, li_border, counts, sx, sy, sz):
    """compute_Zs_with_indices.jl:1-411 (Zs, internal and surface edges): per conductor
    grid a surface impedance per exposed transverse face, doubled on the border sides,
    the two faces of each voxel side in parallel, the two sides summed."""
    # contenitore (lines 23-34): per direction the two cell-side ratios, in the order
    # 0.5 * s_edge / s_other * (1 + 1im) * sqrt(2*pi*1e-7/sigmar)
    sides = [(sx, sy, sz), (sy, sx, sz), (sz, sx, sy)]
    # per direction: which transverse axis feeds columns (1, 3) and which (2, 4)
    tr = {0: (2, 1), 1: (2, 0), 2: (0, 1)}
    out = []
    for c in range(3):
        me = li_mat[c]
        b1, b2 = li_border[c]
        Zsw = np.zeros((me.size, 4), dtype=np.complex128)
        ta, tb = tr[c]
        a1, a2 = counts[c][ta]
        bb1, bb2 = counts[c][tb]
        se, sa, sb = sides[c]
        for kk, mt in enumerate(materials):
            sig = mt["sigmar"]
            if sig == 0:
                continue
            k1 = kk + 1
            va = 0.5 * se / sa * (1 + 1j) * math.sqrt(2 * math.pi * 1e-7 / sig)
            vb = 0.5 * se / sb * (1 + 1j) * math.sqrt(2 * math.pi * 1e-7 / sig)
            inm = me == k1
            i1 = inm & (a1 > 0)
            i3 = inm & (a2 > 0)
            i2 = inm & (bb1 > 0)
            i4 = inm & (bb2 > 0)
            Zsw[i1, 0] = va
            Zsw[i3, 2] = va
            Zsw[i2, 1] = vb
            Zsw[i4, 3] = vb
            d1 = b1 == k1
            d2 = b2 == k1
            Zsw[i1 & d1, 0] = 2 * Zsw[i1 & d1, 0]
            Zsw[i2 & d1, 1] = 2 * Zsw[i2 & d1, 1]
            Zsw[i3 & d2, 2] = 2 * Zsw[i3 & d2, 2]
            Zsw[i4 & d2, 3] = 2 * Zsw[i4 & d2, 3]

        def par(p, q):
            s = p + q
            both = (np.abs(p) != 0) & (np.abs(q) != 0)
            s[both] = p[both] * q[both] / (p[both] + q[both])
            return s

        out.append(par(Zsw[:, 0], Zsw[:, 1]) + par(Zsw[:, 2], Zsw[:, 3]))
    Zs = np.concatenate(out)
    internal = np.nonzero(np.abs(Zs) == 0)[0]
    surface = np.setdiff1d(np.arange(Zs.size), internal)
    return {"Zs": Zs, "internal_edges": internal, "surface_edges": surface,
            "materials": np.concatenate(li_mat)}


# ----------------------------------------------------------------------------------------
# ports and lattice centres (find_voxels_port_pp.jl, build_center_P_Voxels.jl,
# build_centers_Lp_with_air.jl, build_center_air_Voxels.jl)
# ----------------------------------------------------------------------------------------

def nodes_find_rev(pt, centri, skip):
    """find_voxels_port_pp.jl:87-110: the nearest voxel centre (1-based voxel number),
    the second nearest when the nearest is `skip`; ties keep the lower number (stable)."""
    d = np.sqrt(np.sum((centri - np.asarray(pt, dtype=np.float64).reshape(1, 3)) ** 2, axis=1))
    order = np.argsort(d, kind="stable") + 1
    return int(order[0] if order[0] != skip else order[1])


def find_voxels_pp(starts, ends, centri, nodes, nodes_red):
    """find_voxels_port_pp.jl:1-85: voxels and 0-based node indices of two-point terminals."""
    starts = np.asarray(starts, dtype=np.float64).reshape(-1, 3)
    ends = np.asarray(ends, dtype=np.float64).reshape(-1, 3)
    vox = np.zeros((starts.shape[0], 2), dtype=np.int64)
    nd = np.zeros((starts.shape[0], 2), dtype=np.int64)
    for c in range(starts.shape[0]):
        vox[c, 0] = nodes_find_rev(starts[c], centri, -1)
        vox[c, 1] = nodes_find_rev(ends[c], centri, vox[c, 0])
        nd[c, 0] = bin_search(nodes[vox[c, 0] - 1], nodes_red) - 1
        nd[c, 1] = bin_search(nodes[vox[c, 1] - 1], nodes_red) - 1
    return vox - 1, nd


def build_center_P_Voxels(min_v, Nx, Ny, Nz, sx, sy, sz):
    """build_center_P_Voxels.jl:1-111 (lattice order x fastest)."""
    def grid(ix, iy, iz):
        X, Y, Z = np.meshgrid(ix, iy, iz, indexing="ij")
        return np.stack([X.ravel(order="F"), Y.ravel(order="F"), Z.ravel(order="F")], axis=1)

    ax = lambda o, s, n: o + s * (np.arange(1, n + 1) - 1) + s / 2
    hx = lambda o, s, n: o + s * (np.ceil(np.arange(1, n + 1) / 2) - 1) + s / 2
    ox, oy, oz = min_v
    c = {}
    c["p12_se"] = grid(ax(ox, sx, Nx), ax(oy, sy, Ny + 1), ax(oz, sz, Nz))
    c["p34_se"] = grid(ax(ox, sx, Nx + 1), ax(oy, sy, Ny), ax(oz, sz, Nz))
    c["p56_se"] = grid(ax(ox, sx, Nx), ax(oy, sy, Ny), ax(oz, sz, Nz + 1))
    c["p1234"] = grid(hx(ox, sx, 2 * (Nx + 1) - 1), hx(oy, sy, 2 * (Ny + 1) - 1), ax(oz, sz, Nz))
    c["p3456"] = grid(hx(ox, sx, 2 * (Nx + 1) - 1), ax(oy, sy, Ny), hx(oz, sz, 2 * (Nz + 1) - 1))
    c["p1256"] = grid(ax(ox, sx, Nx), hx(oy, sy, 2 * (Ny + 1) - 1), hx(oz, sz, 2 * (Nz + 1) - 1))
    return c


def build_centers_Lp_with_air(Nx, Ny, Nz, sx, sy, sz, min_v):
    """build_centers_Lp_with_air.jl:1-60 over build_center_air_Voxels.jl:1-26."""
    ax = lambda o, s, n: o + s * (np.arange(1, n + 1) - 1) + s / 2
    cx, cy, cz = ax(min_v[0], sx, Nx), ax(min_v[1], sy, Ny), ax(min_v[2], sz, Nz)
    X, Y, Z = np.meshgrid(cx, cy, cz, indexing="ij")
    air = np.stack([X, Y, Z], axis=-1)  # [x, y, z, 3]

    def mid(a, b):
        v = 0.5 * (a + b)
        return v.transpose(2, 1, 0, 3).reshape(-1, 3)  # x fastest

    return (mid(air[:-1], air[1:]), mid(air[:, :-1], air[:, 1:]), mid(air[:, :, :-1], air[:, :, 1:]))


# ----------------------------------------------------------------------------------------
# the mesher and the request reader
# ----------------------------------------------------------------------------------------

ESCALINGS = {"Lp": 1e6, "P": 1e-12, "R": 1e-3, "Cd": 1e12, "Is": 1e3, "Yle": 1e3,
             "freq": 1e-9, "time": 1e9}  # mesher_FFT.jl:5-15 with use_escalings = 1


def mesher_FFT(materials, sx, sy, sz, g, ports, lumped_elements, origin, dominant_list):
    """mesher_FFT.jl:1-112. g: (G, Nx, Ny, Nz) bool in grid order; materials indexed by
    grid number, as the reference does. Returns the reference's nine outputs (0-based
    indices) plus a dict of intermediate arrays for the tests."""
    g = np.asarray(g, dtype=bool)
    G, Nx, Ny, Nz = g.shape
    for mt in materials:
        mt["epsr"] = mt["eps_re"] - 1j * mt["eps_re"] * mt["tan_D"]
    mapping, num_centri = create_volumes_mapping(g)
    centri = create_volume_centers(g, mapping, num_centri, sx, sy, sz, origin)
    ext = create_Grids_externals(g)
    num_full_vox = int(sum(np.count_nonzero(g[k]) for k in range(G)))
    nodes, nodes_red, nodes_reused = create_nodes_ref(g, num_full_vox, ext, mapping, dominant_list)
    exp_mat, Gamma, surf_maps = create_mapping_Gamma_no_rep(g, mapping, nodes, nodes_red, ext)
    # edges: numbering loop orders of create_mapping_A{x,y,z}_v2.jl (outer to inner)
    orders = {0: (1, 2, 0), 1: (2, 0, 1), 2: (0, 1, 2)}
    ed = [_edges(g, mapping, nodes, nodes_red, a, orders[a], materials) for a in range(3)]
    mx, my, mz = (e["lpos"].size for e in ed)
    m = mx + my + mz
    n = nodes_red.size
    offs = [0, mx, mx + my]
    rows = np.concatenate([np.repeat(np.arange(e["lpos"].size) + offs[a], 2)
                           for a, e in enumerate(ed)])
    cols = np.concatenate([np.stack([e["nn1"], e["nn2"]], axis=1).ravel() for e in ed]) - 1
    vals = np.concatenate([np.tile([-1.0, 1.0], e["lpos"].size) for e in ed])
    A = sp.csr_matrix((vals, (rows, cols)), shape=(m, n))
    li_mat = [e["k"] for e in ed]
    li_border = [(e["b1"], e["b2"]) for e in ed]
    counts = [e["counts"] for e in ed]
    Zs_info = compute_Zs(materials, li_mat, li_border, counts, sx, sy, sz)
    N_ind = [(Nx - 1) * Ny * Nz, (Ny - 1) * Nx * Nz, (Nz - 1) * Nx * Ny]
    mat_map = [[None] * 3 for _ in range(3)]
    # create_expansion_ind_Lp_{x,y,z}_grids_v2.jl: (lattice position, edge number) rows in
    # their own loop order (outer to inner); mesher_FFT.jl:61-84 then masks those rows with
    # the border flags, which are indexed by edge number (as written: the two orders
    # differ for y and z edges; these two maps are not read on the operator path)
    exp_orders = {0: (2, 1, 0), 1: (2, 0, 1), 2: (0, 1, 2)}
    for a, e in enumerate(ed):
        mc = e["lpos"].size
        M = sp.csc_matrix((np.ones(mc), (e["lpos"], np.arange(mc))), shape=(N_ind[a], mc))
        mat_map[a][0] = M
        lat = e["lat"]
        lx = e["lpos"] % lat[0]
        ly = (e["lpos"] // lat[0]) % lat[1]
        lz = e["lpos"] // (lat[0] * lat[1])
        lc = (lx, ly, lz)
        o = exp_orders[a]
        rows_exp = np.lexsort((lc[o[2]], lc[o[1]], lc[o[0]]))  # edge numbers in loop order
        for j, b in ((1, e["b1"]), (2, e["b2"])):
            keep = rows_exp[b != 0]
            mat_map[a][j] = sp.csc_matrix((np.ones(keep.size), (e["lpos"][keep], keep)),
                                          shape=(N_ind[a], mc))
    expansions = dict(exp_mat)
    expansions["mat_map_Lp"] = mat_map
    expansions["N_ind"] = N_ind
    diagonals = compute_diagonals(ESCALINGS, materials, sx, sy, sz, li_mat, li_border)
    # compute_diagonal_P_v2 (mesher_FFT.jl:114-138): the face self terms from the P row
    # integral of a face with itself
    from . import peec_oracle as O
    z = np.zeros((1, 3))
    selfP = [float(O.p_row(c, c, z, sx, sy, sz, ESCALINGS["P"])[0]) for c in (1, 3, 5)]
    diagonals["P"] = np.concatenate([np.full(exp_mat["N1"], selfP[0]),
                                     np.full(exp_mat["N2"], selfP[1]),
                                     np.full(exp_mat["N3"], selfP[2])])
    ports = dict(ports)
    ports["port_voxels"], ports["port_nodes"] = find_voxels_pp(
        ports["port_start"], ports["port_end"], centri, nodes, nodes_red)
    le = dict(lumped_elements)
    le["le_voxels"], le["le_nodes"] = find_voxels_pp(
        le.get("le_start", np.zeros((0, 3))), le.get("le_end", np.zeros((0, 3))), centri,
        nodes, nodes_red)
    cc = build_center_P_Voxels(origin, Nx, Ny, Nz, sx, sy, sz)
    cc["Lpx"], cc["Lpy"], cc["Lpz"] = build_centers_Lp_with_air(Nx, Ny, Nz, sx, sy, sz, origin)
    cc.update(sx=sx, sy=sy, sz=sz, Nx=Nx, Ny=Ny, Nz=Nz, origin=tuple(origin))
    incidence_selection = {"A": A, "Gamma": Gamma, "mx": mx, "my": my, "mz": mz}
    li_mats = {"lix_mat": li_mat[0], "liy_mat": li_mat[1], "liz_mat": li_mat[2],
               "lix_border": np.stack(li_border[0], 1), "liy_border": np.stack(li_border[1], 1),
               "liz_border": np.stack(li_border[2], 1), "sx": sx, "sy": sy, "sz": sz}
    inter = {"mapping_vols": mapping, "nodes": nodes, "nodes_red": nodes_red,
             "nodes_reused_clean": nodes_reused, "externals": ext, "surface_maps": surf_maps,
             "edge_lattice_pos": [e["lpos"] for e in ed], "centri_vox": centri}
    return (dict(ESCALINGS), incidence_selection, cc, diagonals, expansions, ports, le,
            li_mats, Zs_info), inter


def material(d):
    """format_input_output_solver_functions.jl:34-58 (the fields the path reads)."""
    return {"name": d["name"], "sigmar": d["conductivity"],
            "tan_D": d.get("tangent_delta_conductivity", 0), "eps_re": d["permittivity"],
            "mur": d.get("permeability", 1), "epsr": 1}


def get_escal_from(unit):
    """getEscalFrom, format_input_output_solver_functions.jl:190-210."""
    return {"m": 1.0, "dm": 1e-1, "cm": 1e-2, "mm": 1e-3, "microm": 1e-6,
            "nanom": 1e-9}.get(unit, 1.0)


def parse_request(req, return_intermediates=False):
    """doSolvingFFT's input handling (do_solving_fft.jl:1-98) and the mesher: grids in
    the key order of mesher_matrices, conductor grids (by material name) dominant,
    ports and lumped elements scaled by the unit. Returns (mesher outputs, freqs,
    GMRES settings, z0, grid shape)."""
    mo, si = req["mesherOutput"], req["solverInput"]
    escal = get_escal_from(si["unit"])
    cs = mo["cell_size"]
    sx, sy, sz = cs["cell_size_x"] * escal, cs["cell_size_y"] * escal, cs["cell_size_z"] * escal
    o = mo["origin"]
    origin = (o["origin_x"], o["origin_y"], o["origin_z"])
    MATERIALS = [material(el) for el in si["materials"]]
    names = list(mo["mesher_matrices"].keys())
    grids = np.stack([np.asarray(mo["mesher_matrices"][k], dtype=bool) for k in names])
    cond = {mt["name"]: mt["sigmar"] > 0 for mt in MATERIALS}  # isMaterialConductor
    dominant = [i for i, nm in enumerate(names) if cond[nm]]
    ports = {"port_start": np.array([[v * escal for v in p["inputElement"]] for p in si["ports"]]),
             "port_end": np.array([[v * escal for v in p["outputElement"]] for p in si["ports"]])}
    les = si.get("lumped_elements", [])
    lumped = {"le_start": np.array([[v * escal for v in p["inputElement"]] for p in les]).reshape(-1, 3),
              "le_end": np.array([[v * escal for v in p["outputElement"]] for p in les]).reshape(-1, 3),
              "type": np.array([int(p["type"]) for p in les], dtype=np.int64),
              "R_value": np.array([float(p["rlcParams"].get("resistance", 0.0)) for p in les]),
              "L_value": np.array([float(p["rlcParams"].get("inductance", 0.0)) for p in les]),
              "C_value": np.array([float(p["rlcParams"].get("capacitance", 0.0)) for p in les])}
    out, inter = mesher_FFT(MATERIALS, sx, sy, sz, grids, ports, lumped, origin, dominant)
    ap = req.get("solverAlgoParams", {})
    settings = {"Inner_Iter": int(ap.get("innerIteration", 100)),
                "Outer_Iter": int(ap.get("outerIteration", 1)),
                "tol": float(ap.get("convergenceThreshold", 1e-4))}
    freqs = np.asarray(si["frequencies"], dtype=np.float64)
    z0 = float(si.get("ports_scattering_value", 50.0))
    res = (out, freqs, settings, z0, grids.shape[1:])
    return (res, inter) if return_intermediates else res
