"""ORACLE -- test infrastructure only. CPU restatement of the reference's retarded
("Rcc", QS_Rcc_FW == 2) operator set-up, used by tests/ as the checker; never imported by
the product.

Parity unpinned: the reference (Julia) cannot run here and ships no outputs for this
path. The restatement is held to what follows from the formulas themselves
(tests/test_oracle_rcc.py): at zero frequency the spectra are those of the quasi-static
rows; on cubic cells the Rcc Lp rows equal the QS fill's rows; the P rows the Rcc path
fills with the block indices as face types are the QS rows of those face types; the
centre distances are the distances of the lattice points.

Follows:
  src/lib/solverFFT/compute_rows_Rcc_Lp.jl:1-111     Lp rows (QS part) and distances
  src/lib/solverFFT/compute_Lp_Voxels_QS.jl:8-397    their integral dispatch (oracle C)
  src/lib/solverFFT/compute_rows_Rcc_P.jl:1-79       P rows (QS part) and distances
  src/lib/solverFFT/compute_Voxels_Rcc.jl:1-13       voxel centre distances
  src/lib/solverFFT/compute_P_vox_Rcc.jl:1-84        face centre distances
  src/lib/solverFFT/build_row_vox_Rcc.jl:1-11        row * exp(-i beta R)
  src/lib/solverFFT/compute_Circulant_Lp_Rcc.jl:1-70 Lp spectra per frequency
  src/lib/solverFFT/compute_Circulant_P_sup_Rcc.jl:1-70 P spectra per frequency
  src/lib/solverFFT/FFT_solver_QS_S_type.jl:61-93,179 the per-frequency rebuild and solve
"""
from __future__ import annotations

import math

import numpy as np

from . import peec_oracle as O


class ReferenceRaises(RuntimeError):
    """The reference raises at this input (its Julia code cannot evaluate it)."""


def lp_row_qs(dc, centers, sx, sy, sz, with_scale=False):
    """compute_Lp_Voxels_QS(centers[0], centers, ...) (compute_Lp_Voxels_QS.jl:8-42),
    unescaled. Entries that fall in the dispatch's orthogonal surface-surface case, whose
    call the reference cannot apply (compute_Lp_Voxels_QS.jl:330-352), raise.
    with_scale: also the per-entry sum of |terms| times the same prefactor."""
    centers = np.ascontiguousarray(centers, dtype=np.float64)
    N = centers.shape[0]
    out = np.empty(N)
    scale = np.empty(N) if with_scale else None
    src = np.ascontiguousarray(centers[0])
    O._fill_lib().oracle_lp_row_qs_d(dc, src.ctypes.data, centers.ctypes.data, N, sx, sy, sz,
                                     out.ctypes.data, scale.ctypes.data if with_scale else None)
    if np.isnan(out).any():
        raise ReferenceRaises(
            f"{int(np.isnan(out).sum())} Lp entries of direction {dc} fall in the orthogonal "
            "surface-surface case of compute_Lp_Voxels_QS's dispatch, where the reference "
            "passes an interval for a coordinate and Julia raises")
    return (out, scale) if with_scale else out


def rcc_row_scales(cc, escalings):
    """Per entry of every escaled Rcc row, the sum of |terms| of its closed form (the
    cancellation-aware scale of a rounding bound)."""
    sx, sy, sz = cc["sx"], cc["sy"], cc["sz"]
    out = {}
    for _, key, dc in O.LP_ROWS:
        ctr = np.asarray(cc[key], dtype=np.float64)
        if ctr.shape[0]:
            out[key] = escalings["Lp"] * lp_row_qs(dc, ctr, sx, sy, sz, with_scale=True)[1]
    for _, key, (q1, q2), _ in RCC_P_ROWS:
        ctr = np.asarray(cc[key], dtype=np.float64)
        out[key] = O.p_row(q1, q2, ctr, sx, sy, sz, escalings["P"], with_scale=True)[1]
    return out


def compute_Voxels_Rcc(centri_m, centri_n):
    """|centri_m - centri_n[k]| (compute_Voxels_Rcc.jl:1-13), components summed x, y, z."""
    d = np.asarray(centri_m, dtype=np.float64)[None, :] - np.asarray(centri_n, dtype=np.float64)
    return np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])


def _face_centres(c, caser, sx, sy, sz):
    c = np.array(c, dtype=np.float64, copy=True)
    axis = {1: 1, 2: 1, 3: 0, 4: 0, 5: 2, 6: 2}[caser]
    s = (sx, sy, sz)[axis]
    if caser in (1, 3, 5):
        c[..., axis] = c[..., axis] - s / 2
    else:
        c[..., axis] = c[..., axis] + s / 2
    return c


def compute_P_vox_Rcc(centers_o, centers, sx, sy, sz, caser, caser2):
    """Distances between face caser of the generating cell and face caser2 of every
    lattice cell (compute_P_vox_Rcc.jl:1-84)."""
    f1 = _face_centres(centers_o, caser, sx, sy, sz)
    f2 = _face_centres(centers, caser2, sx, sy, sz)
    return compute_Voxels_Rcc(f1, f2)


# (block, lattice key, face types of the QS parts, face types of the distances)
RCC_P_ROWS = (((0, 0), "p12_se", (1, 1), (1, 1)), ((1, 1), "p34_se", (2, 2), (3, 3)),
              ((2, 2), "p56_se", (3, 3), (5, 5)), ((0, 1), "p1234", (1, 2), (3, 2)),
              ((0, 2), "p1256", (1, 3), (5, 2)), ((1, 2), "p3456", (2, 3), (5, 4)))


def compute_rows_Rcc_Lp(cc):
    """rows_Lp of compute_rows_Rcc_Lp.jl:1-111: per direction the unescaled QS row (self
    entry zeroed) and the centre distances."""
    sx, sy, sz = cc["sx"], cc["sy"], cc["sz"]
    rows = {}
    for c, key, dc in O.LP_ROWS:
        ctr = np.asarray(cc[key], dtype=np.float64)
        if ctr.shape[0] == 0:
            rows[key] = (np.zeros(0), np.zeros(0))
            continue
        qs = lp_row_qs(dc, ctr, sx, sy, sz)
        qs[0] = 0.0
        rows[key] = (qs, compute_Voxels_Rcc(ctr[0], ctr))
    return rows


def compute_rows_Rcc_P(cc):
    """rows_P of compute_rows_Rcc_P.jl:1-79: per block the unescaled QS row, filled with
    the block indices as face types (:47-52), and the face centre distances (:55-60)."""
    sx, sy, sz = cc["sx"], cc["sy"], cc["sz"]
    rows = {}
    for blk, key, (q1, q2), (r1, r2) in RCC_P_ROWS:
        ctr = np.asarray(cc[key], dtype=np.float64)
        qs = O.p_row(q1, q2, ctr, sx, sy, sz, 1.0)
        rows[key] = (qs, compute_P_vox_Rcc(ctr[0], ctr, sx, sy, sz, r1, r2))
    return rows


def build_row_vox_Rcc(mat_QS, Rcc, freq):
    """mat_QS .* exp(-i beta Rcc), beta = 2 pi f sqrt(eps0 mu0) (build_row_vox_Rcc.jl:1-11)."""
    mu0 = 4 * math.pi * 1e-7
    eps0 = 8.854187816997944e-12
    beta = 2 * math.pi * freq * math.sqrt(eps0 * mu0)
    return np.asarray(mat_QS) * np.exp(-1j * beta * np.asarray(Rcc))


def compute_Circulant_Lp_Rcc(rows_Lp, escalings, freq, Nx, Ny, Nz):
    """FFTCLp at one frequency (compute_Circulant_Lp_Rcc.jl:1-26)."""
    d = O.ref_dims(Nx, Ny, Nz)
    out = [None, None, None]
    for c, key, _ in O.LP_ROWS:
        qs, R = rows_Lp[key]
        if qs.size == 0:
            ext = [2 * Nx, 2 * Ny, 2 * Nz]
            ext[c] = 0
            out[c] = np.zeros(ext, dtype=np.complex128)
            continue
        row = escalings["Lp"] * build_row_vox_Rcc(qs, R, freq)
        out[c] = O._fftn(O.store_circulant_fft(row, *d[key]))
    return out


def compute_Circulant_P_sup_Rcc(rows_P, escalings, freq, Nx, Ny, Nz):
    """FFTCP (upper triangle) at one frequency (compute_Circulant_P_sup_Rcc.jl:1-28)."""
    d = O.ref_dims(Nx, Ny, Nz)
    out = [[None] * 3 for _ in range(3)]
    for (i, j), key, _, _ in RCC_P_ROWS:
        qs, R = rows_P[key]
        row = escalings["P"] * build_row_vox_Rcc(qs, R, freq)
        out[i][j] = O._fftn(O.store_circulant_fft(row, *d[key]))
    return out


def rcc_rows_escaled(rows_Lp, rows_P, escalings):
    """The QS parts, escaled, keyed as the product's rows (for a shared-fill upload)."""
    out = {}
    for _, key, _ in O.LP_ROWS:
        out[key] = escalings["Lp"] * rows_Lp[key][0]
    for _, key, _, _ in RCC_P_ROWS:
        out[key] = escalings["P"] * rows_P[key][0]
    return out


def FFT_solver_Rcc(freq, escalings, incidence_selection, rows_P, rows_Lp, diagonals, ports,
                   ports_scatter_value, lumped_elements, expansions, GMRES_settings, Zs_info,
                   grid, callback=None):
    """The frequency x port loop with QS_Rcc_FW == 2 (FFT_solver_QS_S_type.jl:1-234): per
    frequency the spectra are rebuilt from the rows (:61-93) and the ports solved with
    them (:179), warm started as in the QS loop."""
    Nx, Ny, Nz = grid
    freq = np.asarray(freq, dtype=np.float64).ravel() * escalings["freq"]
    inner = GMRES_settings["Inner_Iter"]
    A = incidence_selection["A"]
    m, n = A.shape
    ns = incidence_selection["Gamma"].shape[1]
    w = 2 * np.pi * freq
    pn = np.asarray(ports["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    S = np.zeros((npt, npt, w.size), dtype=np.complex128)
    Vrest = np.zeros((m + n + ns, npt), dtype=np.complex128)
    info = []
    tol = GMRES_settings["tol"]
    for k in range(w.size):
        f_hz = freq[k] / escalings["freq"]
        FFTCLp = compute_Circulant_Lp_Rcc(rows_Lp, escalings, f_hz, Nx, Ny, Nz)
        FFTCP = compute_Circulant_P_sup_Rcc(rows_P, escalings, f_hz, Nx, Ny, Nz)
        fs = O.frequency_setup(w[k], escalings, incidence_selection, diagonals, Zs_info,
                               lumped_elements, ports, ports_scatter_value)

        def mv(x, fs=fs, wk=w[k], FFTCP=FFTCP, FFTCLp=FFTCLp):
            return O.ComputeMatrixVectorFTT(x, wk, incidence_selection, FFTCP, FFTCLp,
                                            fs["DZ"], fs["Yle"], expansions, fs["invZ"],
                                            fs["invP"], fs["F"])

        for c1 in range(npt):
            n1, n2 = pn[c1]
            is_ = np.zeros(n)
            is_[n1] = escalings["Is"]
            is_[n2] = -escalings["Is"]
            tn = O.precond_3_3_Kt_fft(fs["F"], fs["invZ"], fs["invP"], A,
                                      incidence_selection["Gamma"], m, ns, is_)
            tk = tol[k] if np.ndim(tol) else tol
            V, flag, relres, it, resvec = O.gmres_custom(tn, False, tk, inner, Vrest[:, c1], mv)
            info.append({"freq": k, "port": c1, "flag": flag, "relres": relres, "iter": it,
                         "resvec": resvec})
            if callback:
                callback(k, c1, V)
            Vrest[:, c1] = V
            for c2 in range(c1, npt):
                n3, n4 = pn[c2]
                val = 2 * (V[m + ns + n3] - V[m + ns + n4])
                if c1 == c2:
                    S[c1, c2, k] = (val - ports_scatter_value) / ports_scatter_value
                else:
                    S[c1, c2, k] = val / ports_scatter_value
                    S[c2, c1, k] = S[c1, c2, k]
    return {"S": S, "Z": O.s2z(S, ports_scatter_value), "Y": O.s2y(S, ports_scatter_value),
            "f": freq / escalings["freq"], "info": info, "Vrest": Vrest}
