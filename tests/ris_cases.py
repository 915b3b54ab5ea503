"""Dense RIS test problems built from voxel requests (helpers for the RIS tests).

The voxel path's operator has the same block structure as the RIS solver's, with its Lp
and P products given by circulant convolutions. Written out as dense matrices (one
convolution per unit vector, with the oracle), those blocks make a dense RIS problem
whose operator must equal the voxel path's:
  Lp_ris = Lp_circ + diag(self terms)   (the voxel circulant leaves Lp's diagonal out and
                                         keeps the self terms in diagonals["Lp"])
  P_ris  = P_circ                       (the P circulant holds the self terms)
  Z_self_ris = DZ - jw diag(Lp)         (so that invZ = 1 / (Z_self + jw diag(Lp)) = 1/DZ)
"""
from __future__ import annotations

import copy

import numpy as np

from oracle import mesher_ref as OM
from oracle import peec_oracle as O


def voxel_case(req):
    out, freqs, settings, z0, grid = OM.parse_request(copy.deepcopy(req))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    rows = O.fill_rows(cc, esc, *grid)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, *grid)
    return dict(esc=esc, inc=inc, cc=cc, diag=diag, exp=exp, ports=ports, le=le, Zs=Zs,
                rows=rows, FFTCP=FFTCP, FFTCLp=FFTCLp, freqs=freqs, settings=settings, z0=z0,
                grid=grid)


def dense_blocks(c):
    """Lp_ris blocks and P_ris written out from the voxel case's circulants."""
    inc, exp = c["inc"], c["exp"]
    mx, my, mz = inc["mx"], inc["my"], inc["mz"]
    ns = inc["Gamma"].shape[1]
    dLp = np.asarray(c["diag"]["Lp"], dtype=np.float64).ravel()
    Lp = {}
    off = 0
    for k, (key, size) in enumerate((("Lp_x", mx), ("Lp_y", my), ("Lp_z", mz))):
        M = np.zeros((size, size))
        if size:
            Mk = exp["mat_map_Lp"][k][0]
            for j in range(size):
                e = np.zeros(size)
                e[j] = 1.0
                M[:, j] = (Mk.T @ O._conv(c["FFTCLp"][k], Mk @ e)).real
            M[np.arange(size), np.arange(size)] += dLp[off:off + size]
        Lp[key] = M
        off += size
    E = exp["exp_P"]
    P = np.zeros((ns, ns))
    for j in range(ns):
        e = np.zeros(ns)
        e[j] = 1.0
        col = np.zeros(ns, dtype=np.complex128)
        for c1 in range(3):
            for c2 in range(c1, 3):
                spec = c["FFTCP"][c1][c2]
                col += E[c2][c1].T @ O._conv(spec, E[c1][c2] @ e)
                if c1 != c2:
                    col += E[c1][c2].T @ O._conv(spec, E[c2][c1] @ e)
        P[:, j] = col.real
    return Lp, {"P": P}


def volumi_of(c, seed=0):
    """A RIS 'volumi' description for the case's edges: R the edge resistances, the
    dielectric edges (no resistance) with their capacitances, and a surface-impedance
    part on a seeded quarter of the conductor edges."""
    R = np.real(np.asarray(c["diag"]["R"])).astype(np.float64).sum(axis=1)
    Cd = np.real(np.asarray(c["diag"]["Cd"])).astype(np.float64)
    Cd_eff = np.zeros(R.size)
    nz = (Cd > 0).sum(axis=1) > 0
    with np.errstate(divide="ignore"):
        Cd_eff[nz] = 1.0 / np.sum(np.where(Cd[nz] > 0, 1.0 / np.where(Cd[nz] > 0, Cd[nz], 1.0),
                                           0.0), axis=1)
    diel = np.flatnonzero((R == 0) & (Cd_eff > 0))
    rng = np.random.default_rng(seed)
    Zs_part = np.zeros(R.size)
    cond = np.flatnonzero(R > 0)
    pick = rng.choice(cond, size=max(1, cond.size // 4), replace=False) if cond.size else []
    Zs_part[pick] = R[pick] * rng.uniform(0.2, 3.0, size=len(pick)) / np.sqrt(2 * np.pi * 1e9)
    return {"R": R, "Cd": Cd_eff, "indici_dielettrici": diel, "Zs_part": Zs_part}


def with_distances(c, Lp, P):
    """Lp_data / P_data with the centre distances of the retarded RIS operator: Rx, Ry, Rz
    between the edges of each direction and R_cc between the surfaces (metres, from the
    lattice cells of the case's mesh; zero on the diagonal)."""
    from solver_gb300.operator import _edge_cells, _surf_cells, row_dims
    inc, exp = c["inc"], c["exp"]
    mx, my, mz = inc["mx"], inc["my"], inc["mz"]
    ns = inc["Gamma"].shape[1]
    Nx, Ny, Nz = c["grid"][:3]
    cell = np.array([c["cc"]["sx"], c["cc"]["sy"], c["cc"]["sz"]], dtype=np.float64)
    dims = row_dims(Nx, Ny, Nz)

    def coords(ids, d, shift):
        ids = np.asarray(ids, dtype=np.int64)
        ix, iy, iz = ids % d[0], (ids // d[0]) % d[1], ids // (d[0] * d[1])
        return (np.stack([ix, iy, iz], axis=1) + np.asarray(shift)) * cell

    def dist(pos):
        return np.sqrt(((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1))

    ec = _edge_cells(exp, mx, my, mz)
    Lp = dict(Lp)
    Lp["Rx"] = dist(coords(ec[:mx], dims["Lpx"], (1.0, 0.5, 0.5)))
    Lp["Ry"] = dist(coords(ec[mx:mx + my], dims["Lpy"], (0.5, 1.0, 0.5)))
    Lp["Rz"] = dist(coords(ec[mx + my:], dims["Lpz"], (0.5, 0.5, 1.0)))
    fam, scell = _surf_cells(exp, ns)
    spos = np.zeros((ns, 3))
    for f, (key, sh) in enumerate((("p12_se", (0.5, 0.0, 0.5)), ("p34_se", (0.0, 0.5, 0.5)),
                                   ("p56_se", (0.5, 0.5, 0.0)))):
        sel = fam == f
        spos[sel] = coords(scell[sel], dims[key], sh)
    P = dict(P)
    P["R_cc"] = dist(spos)
    return Lp, P


def _brick24(lo, hi):
    """The 24 vertex coordinates of an axis-aligned brick in the reference's vertex order
    (x alternating fastest, then y, then z: the min/max index sets of calcola_Lp.jl:22-28
    and the end faces of mean_length_rev)."""
    v = []
    for z in (lo[2], hi[2]):
        for y in (lo[1], hi[1]):
            for x in (lo[0], hi[0]):
                v += [x, y, z]
    return v


def _rect12(lo, hi):
    """Four vertices of an axis-aligned rectangle; vertices 1 and 4 are the opposite
    corners process_surfaces! reads (calcola_P.jl:110-121)."""
    lo, hi = list(lo), list(hi)
    mid1 = [hi[0], lo[1], lo[2]] if hi[0] != lo[0] else [lo[0], hi[1], lo[2]]
    mid2 = [lo[0], hi[1], hi[2]] if hi[0] != lo[0] else [lo[0], lo[1], hi[2]]
    return lo + mid1 + mid2 + hi


def ris_geometry(c):
    """volumi / superfici of the voxel case's bodies as the RIS solver's mesher describes
    them: each edge's Lp cell (one voxel length along the edge, centred between the two
    voxel centres) and each surface's voxel face, with cross-sections, areas and centres."""
    from solver_gb300.operator import _edge_cells, _surf_cells, row_dims
    inc, exp = c["inc"], c["exp"]
    mx, my, mz = inc["mx"], inc["my"], inc["mz"]
    ns = inc["Gamma"].shape[1]
    Nx, Ny, Nz = c["grid"][:3]
    cell = np.array([c["cc"]["sx"], c["cc"]["sy"], c["cc"]["sz"]], dtype=np.float64)
    dims = row_dims(Nx, Ny, Nz)

    def idx3(ids, d):
        ids = np.asarray(ids, dtype=np.int64)
        return np.stack([ids % d[0], (ids // d[0]) % d[1], ids // (d[0] * d[1])], axis=1)

    ec = _edge_cells(exp, mx, my, mz)
    coords, S, ctr = [], [], []
    for d, (key, sl) in enumerate((("Lpx", slice(0, mx)), ("Lpy", slice(mx, mx + my)),
                                   ("Lpz", slice(mx + my, mx + my + mz)))):
        for ijk in idx3(ec[sl], dims[key]):
            lo = ijk.astype(np.float64)
            lo[d] += 0.5
            hi = lo + 1.0
            coords.append(_brick24(lo * cell, hi * cell))
            t = [q for q in range(3) if q != d]
            S.append(cell[t[0]] * cell[t[1]])
            ctr.append((0.5 * (lo + hi) * cell).tolist())
    volumi = {"coordinate": np.array(coords).reshape(-1, 24), "S": np.array(S),
              "centri": np.array(ctr).reshape(-1, 3)}
    fam, scell = _surf_cells(exp, ns)
    ends, A, sc = [], [], []
    for s_ in range(ns):
        f = int(fam[s_])
        key = ("p12_se", "p34_se", "p56_se")[f]
        nrm = (1, 0, 2)[f]
        lo = idx3([scell[s_]], dims[key])[0].astype(np.float64)
        hi = lo + 1.0
        hi[nrm] = lo[nrm]
        ends.append(_rect12((lo * cell).tolist(), (hi * cell).tolist()))
        t = [q for q in range(3) if q != nrm]
        A.append(cell[t[0]] * cell[t[1]])
        sc.append((0.5 * (lo + hi) * cell).tolist())
    superfici = {"estremi_celle": np.array(ends).reshape(-1, 12), "S": np.array(A),
                 "centri": np.array(sc).reshape(-1, 3)}
    return volumi, superfici


def random_bodies(seed, mx, my, mz, ns, span=0.2):
    """Seeded bricks (mx along x, my along y, mz along z) and rectangles (ns, random
    normals) of widely varying sizes and aspect ratios, some clustered and some far apart,
    so that every branch of the dense fill's case trees (the full closed forms and the
    surface, line and point forms of the suppressed dimensions) is taken."""
    rng = np.random.default_rng(seed)

    def sizes(k):
        base = 10.0 ** rng.uniform(-4.3, -3.0, size=(k, 3))
        thin = rng.random(k) < 0.3  # a thin dimension: surface-like bodies
        ax = rng.integers(0, 3, size=k)
        base[thin, ax[thin]] *= 10.0 ** rng.uniform(-3, -1.5, size=thin.sum())
        return base

    def places(k):
        near = rng.random(k) < 0.5
        p = rng.uniform(0, span, size=(k, 3))
        p[near] = rng.uniform(0, span * 0.01, size=(near.sum(), 3))
        return p

    coords, S, ctr = [], [], []
    for d, k in enumerate((mx, my, mz)):
        sz = sizes(k)
        sz[:, d] *= rng.uniform(1.0, 6.0, size=k)  # longer along the current
        lo = places(k)
        for i in range(k):
            hi = lo[i] + sz[i]
            coords.append(_brick24(lo[i], hi))
            t = [q for q in range(3) if q != d]
            S.append(sz[i, t[0]] * sz[i, t[1]])
            ctr.append((0.5 * (lo[i] + hi)).tolist())
    volumi = {"coordinate": np.array(coords, dtype=np.float64).reshape(-1, 24),
              "S": np.array(S), "centri": np.array(ctr).reshape(-1, 3)}
    sz = sizes(ns)
    nrm = rng.integers(0, 3, size=ns)
    lo = places(ns)
    ends, A, sc = [], [], []
    for i in range(ns):
        hi = lo[i] + sz[i]
        hi[nrm[i]] = lo[i][nrm[i]]
        ends.append(_rect12(lo[i].tolist(), hi.tolist()))
        t = [q for q in range(3) if q != nrm[i]]
        A.append(sz[i, t[0]] * sz[i, t[1]])
        sc.append((0.5 * (lo[i] + hi)).tolist())
    superfici = {"estremi_celle": np.array(ends).reshape(-1, 12), "S": np.array(A),
                 "centri": np.array(sc).reshape(-1, 3)}
    return volumi, superfici


def oracle_dense_fill(*args, **kw):
    """The oracle's dense Lp blocks and P (oracle/ris_fill.py)."""
    from oracle import ris_fill
    return ris_fill.dense_fill(*args, **kw)
