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
