"""ORACLE -- test infrastructure only.

CPU restatement of the reference FFT-PEEC hot path, used by tests/ (and the
cpu_baseline leg of bench.py) as the checker. It is never imported by the product
package. Every function follows the reference at the cited lines and keeps its
algorithm as written: 2N-extent circulant embeddings (store_circulant_fft), the
per-call zero-padded FFT convolutions, three separate sparse-LU solves in the
preconditioner, and MATLAB-style Householder GMRES with its stagnation logic.

Third-party arithmetic the reference relies on is replaced by: numpy.fft (pocketfft)
for FFTW, scipy.sparse.linalg.splu (SuperLU) for UMFPACK. Both return the same
mathematical quantities; only rounding differs.

Parity status: parity unpinned. The reference ships no tests or golden vectors for this
path and no Julia runtime is available, so this restatement cannot be checked against the
reference's own outputs. It is held to known answers instead (closed-form self and
far-field integrals, reciprocity, GMRES on known systems, a dense solve of the assembled
operator, the lumped element networks) in tests/test_oracle_known_answers.py, and to its
committed regression fixtures on the reference's own request files (tests/golden/).
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import build as _obuild

_fill = None

# FFT backend of the oracle operator: None -> numpy.fft (single thread); an int -> scipy.fft
# with that many workers (the reference runs FFTW with 2 x Julia threads,
# compute_FFT_mutual_coupling_mats.jl:4).
FFT_WORKERS = None


def _fftn(a):
    if FFT_WORKERS:
        import scipy.fft as sf
        return sf.fftn(a, workers=FFT_WORKERS)
    return np.fft.fftn(a)


def _ifftn(a):
    if FFT_WORKERS:
        import scipy.fft as sf
        return sf.ifftn(a, workers=FFT_WORKERS)
    return np.fft.ifftn(a)


def _fill_lib():
    global _fill
    if _fill is None:
        lib = ctypes.CDLL(str(_obuild.build()))
        for sfx in ("_d", "_ld"):
            f = getattr(lib, "oracle_lp_row" + sfx)
            f.restype = ctypes.c_int64
            f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                          ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_int,
                          ctypes.c_void_p, ctypes.c_void_p]
            q = getattr(lib, "oracle_lp_row_qs" + sfx)
            q.restype = ctypes.c_int64
            q.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                          ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_void_p,
                          ctypes.c_void_p]
            g = getattr(lib, "oracle_p_row" + sfx)
            g.restype = ctypes.c_int64
            g.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                          ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                          ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        _fill = lib
    return _fill


# ----------------------------------------------------------------------------------------
# fill (compute_FFT_mutual_coupling_mats.jl, compute_Lp_Voxels.jl, compute_row_P_sup.jl)
# ----------------------------------------------------------------------------------------

def lp_row(dc, centers, sx, sy, sz, precision="double", with_scale=False, suppression=True,
           count_far=False):
    """compute_Lp_Voxels(centers[0], centers, ...) for one direction dc in 1..3
    (compute_Lp_Voxels.jl:1-63), unescaled. suppression=False evaluates every entry by
    the full volume-volume closed form instead of the reference's far-field branches.
    count_far=True also returns how many entries took a far-field branch."""
    centers = np.ascontiguousarray(centers, dtype=np.float64)
    N = centers.shape[0]
    out = np.empty(N)
    scale = np.empty(N) if with_scale else None
    src = np.ascontiguousarray(centers[0])
    fn = getattr(_fill_lib(), "oracle_lp_row" + ("_ld" if precision == "long" else "_d"))
    far = fn(dc, src.ctypes.data, centers.ctypes.data, N, sx, sy, sz, int(bool(suppression)),
             out.ctypes.data, scale.ctypes.data if with_scale else None)
    res = (out, scale) if with_scale else out
    return (res, int(far)) if count_far else res


def p_row(caser, caser2, centers, sx, sy, sz, escal_P, precision="double", with_scale=False,
          suppression=True, count_far=False):
    """escal_P * compute_row_P_sup(centers[0], centers, ..., caser, caser2)
    (compute_row_P_sup.jl:1-104); suppression / count_far as for lp_row."""
    centers = np.ascontiguousarray(centers, dtype=np.float64)
    N = centers.shape[0]
    out = np.empty(N)
    scale = np.empty(N) if with_scale else None
    src = np.ascontiguousarray(centers[0])
    fn = getattr(_fill_lib(), "oracle_p_row" + ("_ld" if precision == "long" else "_d"))
    far = fn(caser, caser2, src.ctypes.data, centers.ctypes.data, N, sx, sy, sz, escal_P,
             int(bool(suppression)), out.ctypes.data, scale.ctypes.data if with_scale else None)
    res = (out, scale) if with_scale else out
    return (res, int(far)) if count_far else res


# (lattice key, caser, caser2, reference dims) of the six P rows, in the order
# compute_Circulant_P_sup fills them (compute_FFT_mutual_coupling_mats.jl:96-125)
P_ROWS = (((0, 0), "p12_se", 1, 1), ((1, 1), "p34_se", 3, 3), ((2, 2), "p56_se", 5, 5),
          ((0, 1), "p1234", 3, 2), ((0, 2), "p1256", 5, 2), ((1, 2), "p3456", 5, 4))
LP_ROWS = ((0, "Lpx", 1), (1, "Lpy", 2), (2, "Lpz", 3))


def ref_dims(Nx, Ny, Nz):
    return {"Lpx": (Nx - 1, Ny, Nz), "Lpy": (Nx, Ny - 1, Nz), "Lpz": (Nx, Ny, Nz - 1),
            "p12_se": (Nx, Ny + 1, Nz), "p34_se": (Nx + 1, Ny, Nz), "p56_se": (Nx, Ny, Nz + 1),
            "p1234": (2 * (Nx + 1) - 1, 2 * (Ny + 1) - 1, Nz),
            "p1256": (Nx, 2 * (Ny + 1) - 1, 2 * (Nz + 1) - 1),
            "p3456": (2 * (Nx + 1) - 1, Ny, 2 * (Nz + 1) - 1)}


def fill_rows(circulant_centers, escalings, Nx, Ny, Nz, precision="double", with_scale=False,
              far_counts=None):
    """The nine generating rows (escaled; Lp self entries zeroed as at
    compute_FFT_mutual_coupling_mats.jl:56,68,80). Returns {key: row or (row, scale)}.
    far_counts, a dict, receives per row the number of entries that took a far-field
    (suppressed) branch."""
    cc = circulant_centers
    sx, sy, sz = cc["sx"], cc["sy"], cc["sz"]
    out = {}
    for _, key, dc in LP_ROWS:
        if np.prod(ref_dims(Nx, Ny, Nz)[key]) == 0:
            continue
        r, far = lp_row(dc, cc[key], sx, sy, sz, precision, with_scale, count_far=True)
        if far_counts is not None:
            far_counts[key] = far
        if with_scale:
            row = escalings["Lp"] * r[0]
            row[0] = 0.0
            out[key] = (row, escalings["Lp"] * r[1])
        else:
            row = escalings["Lp"] * r
            row[0] = 0.0
            out[key] = row
    for _, key, c1, c2 in P_ROWS:
        out[key], far = p_row(c1, c2, cc[key], sx, sy, sz, escalings["P"], precision, with_scale,
                              count_far=True)
        if far_counts is not None:
            far_counts[key] = far
    return out


def store_circulant_fft(row, Nx, Ny, Nz):
    """Even mirror embedding of a column-major row into a 2Nx x 2Ny x 2Nz grid with a
    zero plane at index N (compute_FFT_mutual_coupling_mats.jl:130-155)."""
    circ = np.reshape(np.asarray(row, dtype=np.complex128), (Nx, Ny, Nz), order="F")

    def idx(N):
        j = np.arange(2 * N)
        src = np.where(j < N, j, 2 * N - j)
        src[N] = N  # points at the appended zero
        return src

    pad = np.zeros((Nx + 1, Ny + 1, Nz + 1), dtype=np.complex128)
    pad[:Nx, :Ny, :Nz] = circ
    return pad[np.ix_(idx(Nx), idx(Ny), idx(Nz))]


def spectra_from_rows(rows, Nx, Ny, Nz):
    """FFTCLp (3 x 1) and FFTCP (3 x 3 upper triangle) as the reference builds them."""
    d = ref_dims(Nx, Ny, Nz)
    FFTCLp = [None, None, None]
    for c, key, _ in LP_ROWS:
        if key not in rows:
            ext = [2 * Nx, 2 * Ny, 2 * Nz]
            ext[c] = 0
            FFTCLp[c] = np.zeros(ext, dtype=np.complex128)
            continue
        r = rows[key][0] if isinstance(rows[key], tuple) else rows[key]
        FFTCLp[c] = _fftn(store_circulant_fft(r, *d[key]))
    FFTCP = [[None] * 3 for _ in range(3)]
    for (i, j), key, _, _ in P_ROWS:
        r = rows[key][0] if isinstance(rows[key], tuple) else rows[key]
        FFTCP[i][j] = _fftn(store_circulant_fft(r, *d[key]))
    return FFTCP, FFTCLp


def compute_FFT_mutual_coupling_mats(circulant_centers, escalings, Nx, Ny, Nz):
    """compute_FFT_mutual_coupling_mats.jl:1-33 for QS_Rcc_FW == 1."""
    return spectra_from_rows(fill_rows(circulant_centers, escalings, Nx, Ny, Nz), Nx, Ny, Nz)


# ----------------------------------------------------------------------------------------
# operator (compute_Matrix_vector_fft.jl)
# ----------------------------------------------------------------------------------------

def _conv(spec, vec_lattice):
    """fft -> x spectrum -> scaled ifft on the 2N grid, return the first octant
    (fft_and_ifft_both_in_place!, compute_Matrix_vector_fft.jl:149-161)."""
    Nx, Ny, Nz = (s // 2 for s in spec.shape)
    circ = np.reshape(vec_lattice, (Nx, Ny, Nz), order="F")
    padded = np.zeros(spec.shape, dtype=np.complex128)
    padded[:Nx, :Ny, :Nz] = circ
    res = _ifftn(spec * _fftn(padded))
    return np.reshape(res[:Nx, :Ny, :Nz], Nx * Ny * Nz, order="F")


def ComputeMatrixVectorFTT(x, w, incidence_selection, FFTCP, FFTCLp, DZ, Yle, expansions,
                           invZ, invP, lu):
    """y = M^-1 K x (compute_Matrix_vector_fft.jl:1-81)."""
    A = incidence_selection["A"]
    Gamma = incidence_selection["Gamma"]
    m = A.shape[0]
    ns = Gamma.shape[1]
    x = np.asarray(x, dtype=np.complex128).ravel()
    I = x[:m]
    Q = x[m:m + ns]
    Phi = x[m + ns:]
    mx, my, mz = incidence_selection["mx"], incidence_selection["my"], incidence_selection["mz"]
    ranges = [slice(0, mx), slice(mx, mx + my), slice(mx + my, mx + my + mz)]
    Y1 = np.zeros(m, dtype=np.complex128)
    for c in range(3):
        if FFTCLp[c].size == 0:
            continue
        M = expansions["mat_map_Lp"][c][0]
        I_exp = M @ I[ranges[c]]
        Y1[ranges[c]] = Y1[ranges[c]] + M.T @ _conv(FFTCLp[c], I_exp)
    Y1 = (1j * w) * Y1 + np.asarray(DZ).ravel() * I + A @ Phi
    Y2 = np.zeros(ns, dtype=np.complex128)
    Y3 = np.zeros(Yle.shape[0], dtype=np.complex128)
    E = expansions["exp_P"]
    for c1 in range(3):
        for c2 in range(c1, 3):
            spec = FFTCP[c1][c2]
            Y2 = Y2 + E[c2][c1].T @ _conv(spec, E[c1][c2] @ Q)
            if c1 != c2:
                Y2 = Y2 + E[c1][c2].T @ _conv(spec, E[c2][c1] @ Q)
    Y2 = Y2 - Gamma.T @ Phi
    Y3 = Y3 - A.T @ I
    Y3 = Y3 + Yle @ Phi
    Y3 = Y3 + (1j * w) * (Gamma @ Q)
    return precond_3_3_vector(lu, invZ, invP, A, Gamma, w, Y1, Y2, Y3)


def precond_3_3_vector(F, invZ, invP, A, Gamma, w, X1, X2, X3):
    """compute_Matrix_vector_fft.jl:84-146 with its three separate LU solves."""
    n1, n2 = X1.size, X2.size
    Y = np.zeros(n1 + n2 + X3.size, dtype=np.complex128)
    i1, i2, i3 = slice(0, n1), slice(n1, n1 + n2), slice(n1 + n2, None)
    iz = invZ @ X1
    Y[i1] += iz
    M2 = F(A.T @ iz)
    ip = invP @ X2
    Y[i2] += ip
    M4 = F(Gamma @ ip)
    M5 = F(X3)
    Y[i1] -= invZ @ (A @ M2)
    Y[i1] += (1j * w) * (invZ @ (A @ M4))
    Y[i1] -= invZ @ (A @ M5)
    Y[i2] += invP @ (Gamma.T @ M2)
    Y[i2] -= (1j * w) * (invP @ (Gamma.T @ M4))
    Y[i2] += invP @ (Gamma.T @ M5)
    Y[i3] += M2 - (1j * w) * M4 + M5
    return Y


def precond_3_3_Kt_fft(F, invZ, invP, A, Gamma, n1, n2, X3):
    """Right-hand side M^-1 [0; 0; X3] (FFT_solver_QS_S_type.jl:237-262)."""
    M5 = F(X3)
    return np.concatenate([-(invZ @ (A @ M5)), invP @ (Gamma.T @ M5), M5])


# ----------------------------------------------------------------------------------------
# Householder GMRES (gmres_custom.jl:1-331, scalarsignfft :661-668)
# ----------------------------------------------------------------------------------------

def scalarsign(d):
    if d == 0:
        return 1.0
    return d / abs(d)


def gmres_custom(b, restarted, tol, maxit, x, matvec, restart=None, stop=None):
    """MATLAB-semantics Householder GMRES. ``matvec(v)`` applies the (left
    preconditioned) operator. Returns (x, flag, relres, iter, resvec).

    ``restarted=True`` runs the MATLAB restart loop with ``restart`` inner steps
    (the reference's restart branch reads an undefined variable, gmres_custom.jl:6;
    here ``restart`` is an explicit argument)."""
    b = np.asarray(b, dtype=np.complex128).ravel()
    n = b.size
    if restarted:
        outer = maxit
        inner = min(restart, n)
    else:
        outer = 1
        if maxit > n:
            maxit = n
        inner = maxit
    n2b = np.linalg.norm(b)
    if n2b == 0:
        return np.zeros(n, dtype=np.complex128), 0, 0.0, [0, 0], np.array([0.0])
    x = np.zeros(n, dtype=np.complex128) if x is None or np.size(x) == 0 else \
        np.array(x, dtype=np.complex128).ravel()
    flag = 1
    xmin = x
    imin = jmin = 0
    tolb = tol * n2b
    xm = x
    evalxm = 0
    stag = 0
    moresteps = 0
    maxmsteps = min(math.floor(n / 50), 5, n - maxit)
    maxstagsteps = 3
    minupdated = 0
    r = b - matvec(x)
    normr = np.linalg.norm(r)
    if normr <= tolb:
        return x, 0, normr / n2b, [0, 0], np.array([normr])
    n2minv_b = np.linalg.norm(b)
    tolb = tol * n2minv_b
    resvec = np.zeros(inner * outer + 1)
    resvec[0] = normr
    normrmin = normr
    J = np.zeros((2, inner), dtype=np.complex128)
    U = np.zeros((n, inner + 1), dtype=np.complex128)
    R = np.zeros((inner, inner), dtype=np.complex128)
    w = np.zeros(inner + 1, dtype=np.complex128)
    outitercount = 0
    initercount = 0
    normr_act = normr
    it = [0, 0]
    for outiter in range(1, outer + 1):
        outitercount += 1
        u = r.copy()
        beta = scalarsign(r[0]) * normr
        u[0] += beta
        u = u / np.linalg.norm(u)
        U[:, 0] = u
        w[0] = -beta
        initercount = 0
        for initer in range(1, inner + 1):
            if stop is not None and stop():
                return x, 99, 0.0, [outiter, initer], np.array([0.0])
            initercount += 1
            j = initer - 1  # 0-based column of the current reflector
            v = -2 * np.conj(u[j]) * u
            v[j] += 1
            for k in range(initer - 2, -1, -1):
                v = v - U[:, k] * (2 * np.vdot(U[:, k], v))
            v = v / np.linalg.norm(v)
            v = matvec(v)
            for k in range(0, initer):
                v = v - U[:, k] * (2 * np.vdot(U[:, k], v))
            if initer != v.size:
                u = v.copy()
                u[:initer] = 0
                alpha = np.linalg.norm(u)
                if alpha != 0:
                    alpha = scalarsign(v[initer]) * alpha
                    u[initer] += alpha
                    u = u / np.linalg.norm(u)
                    U[:, initer] = u
                    v[initer + 1:] = 0
                    v[initer] = -alpha
            for colJ in range(0, initer - 1):
                tmpv = v[colJ]
                v[colJ] = np.conj(J[0, colJ]) * v[colJ] + np.conj(J[1, colJ]) * v[colJ + 1]
                v[colJ + 1] = -J[1, colJ] * tmpv + J[0, colJ] * v[colJ + 1]
            if initer != v.size:
                rho = np.linalg.norm(v[j:j + 2])
                J[:, j] = v[j:j + 2] / rho
                w[j + 1] = -J[1, j] * w[j]
                w[j] = np.conj(J[0, j]) * w[j]
                v[j] = rho
                v[j + 1] = 0
            R[:, j] = v[:inner]
            normr = abs(w[j + 1])
            resvec[(outiter - 1) * inner + initer] = normr
            normr_act = normr
            if normr <= tolb or stag >= maxstagsteps or moresteps == 1:
                if evalxm == 0:
                    ytmp = np.linalg.solve(R[:initer, :initer], w[:initer])
                    additive = U[:, j] * (-2 * ytmp[j] * np.conj(U[j, j]))
                    additive[j] += ytmp[j]
                    for k in range(initer - 2, -1, -1):
                        additive[k] += ytmp[k]
                        additive = additive - U[:, k] * (2 * np.vdot(U[:, k], additive))
                    if np.linalg.norm(additive) < np.finfo(float).eps * np.linalg.norm(x):
                        stag += 1
                    else:
                        stag = 0
                    xm = x + additive
                    evalxm = 1
                elif evalxm == 1:
                    wr = w[j] / R[j, j]
                    if initer > 1:
                        head = -np.linalg.solve(R[:initer - 1, :initer - 1], R[:initer - 1, j]) * wr
                    else:
                        head = np.zeros(0, dtype=np.complex128)
                    addvc = np.concatenate([head, [wr]])
                    if np.linalg.norm(addvc) < np.finfo(float).eps * np.linalg.norm(xm):
                        stag += 1
                    else:
                        stag = 0
                    additive = U[:, j] * (-2 * addvc[j] * np.conj(U[j, j]))
                    additive[j] += addvc[j]
                    for k in range(initer - 2, -1, -1):
                        additive[k] += addvc[k]
                        additive = additive - U[:, k] * (2 * np.vdot(U[:, k], additive))
                    xm = xm + additive
                r = b - matvec(xm)
                if np.linalg.norm(r) <= tol * n2b:
                    x = xm
                    flag = 0
                    it = [outiter, initer]
                    break
                normr_act = np.linalg.norm(r)
                resvec[(outiter - 1) * inner + initer] = normr_act
                if normr_act <= normrmin:
                    normrmin = normr_act
                    imin, jmin = outiter, initer
                    xmin = xm
                    minupdated = 1
                if normr_act <= tolb:
                    x = xm
                    flag = 0
                    it = [outiter, initer]
                    break
                else:
                    if stag >= maxstagsteps and moresteps == 0:
                        stag = 0
                    moresteps += 1
                    if moresteps >= maxmsteps:
                        flag = 3
                        it = [outiter, initer]
                        break
            if normr_act <= normrmin:
                normrmin = normr_act
                imin, jmin = outiter, initer
                minupdated = 1
            if stag >= maxstagsteps:
                flag = 3
                break
        evalxm = 0
        if flag != 0:
            idx = jmin if minupdated == 1 else initercount
            if idx > 0:
                y = np.linalg.solve(R[:idx, :idx], w[:idx])
                additive = U[:, idx - 1] * (-2 * y[idx - 1] * np.conj(U[idx - 1, idx - 1]))
                additive[idx - 1] += y[idx - 1]
                for k in range(idx - 2, -1, -1):
                    additive[k] += y[k]
                    additive = additive - U[:, k] * (2 * np.vdot(U[:, k], additive))
                x = x + additive
            xmin = x
            r = b - matvec(x)
            normr_act = np.linalg.norm(r)
        if normr_act <= normrmin:
            xmin = x
            normrmin = normr_act
            imin = outiter
            jmin = initercount
        if flag == 3:
            break
        if normr_act <= tolb:
            flag = 0
            it = [outitercount, initercount]
            break
        minupdated = 0
    if flag == 0:
        relres = normr_act / n2minv_b
    else:
        x = xmin
        it = [imin, jmin]
        relres = normr_act / n2minv_b
    resvec = resvec[:max(outitercount - 1, 0) * inner + initercount + 1]
    return x, flag, relres, it, resvec


# ----------------------------------------------------------------------------------------
# frequency / port loop (FFT_solver_QS_S_type.jl:1-285, build_Yle_FFT.jl, compute_Z_self.jl)
# ----------------------------------------------------------------------------------------

def lumped_admittance(typ, R, L, C, w):
    """get_lumped_elements_admittance_fft (build_Yle_FFT.jl:128-209), statement by
    statement; numpy scalars give Julia's IEEE results for divisions by zero."""
    R, L, C = np.float64(R), np.float64(L), np.float64(C)
    jw = np.complex128(1j * w)

    def bad(v):
        return np.isnan(v) or np.isinf(v) or abs(v) < 1e-16

    with np.errstate(all="ignore"):
        y = np.complex128(0.0)
        if typ == 1:
            z = R + jw * L + 1 / (jw * C)
            if np.isnan(z) or np.isinf(z) or abs(z) < 1e-16:
                z = R + jw * L
            y = 1 / z
        elif typ == 2:
            y = 1 / (R + jw * L) + jw * C
            if bad(y):
                y = 1 / R + jw * C
            if bad(y):
                y = 1 / (R + jw * L)
            if bad(y):
                y = 1 / R
            if bad(y):
                y = 1 / (jw * L) + jw * C
            if bad(y):
                y = jw * C
        elif typ == 3:
            y = 1 / (R + 1 / (jw * C)) + 1 / (jw * L)
            if bad(y):
                y = 1 / (R + 1 / (jw * C))
            if bad(y):
                y = 1 / R + 1 / (jw * L)
            if bad(y):
                y = 1 / R
            if bad(y):
                y = 1 / (1 / (jw * C)) + 1 / (jw * L)
            if bad(y):
                y = 1 / (jw * L)
            if bad(y):
                y = 1 / (1 / (jw * C))
        elif typ == 4:
            y = 1 / R + jw * C + 1 / (jw * L)
            if bad(y):
                y = 1 / R + jw * C
            if bad(y):
                y = jw * C + 1 / (jw * L)
            if bad(y):
                y = jw * C
        elif typ == 5:
            y = 1 / R + 1 / (jw * L + 1 / (jw * C))
            if bad(y):
                y = 1 / R + 1 / (1 / (jw * C))
            if bad(y):
                y = 1 / R + 1 / (jw * L)
            if bad(y):
                y = 1 / R
            if bad(y):
                y = 1 / (jw * L + 1 / (jw * C))
            if bad(y):
                y = 1 / (jw * L)
            if bad(y):
                y = 1 / (1 / (jw * C))
        if np.isnan(y) or np.isinf(y):
            y = 0.0
        return complex(y)


def build_Yle(lumped_elements, ports, escalings, n, w, z0):
    """Sparse n x n termination / lumped admittance (build_Yle_FFT.jl:1-126)."""
    r, c, v = [], [], []

    def stamp(n1, n2, y):
        r.extend([n1, n2, n1, n2]); c.extend([n1, n2, n2, n1]); v.extend([y, y, -y, -y])

    le = lumped_elements
    for k in range(len(le.get("le_nodes", []))):
        y = lumped_admittance(int(le["type"][k]), le["R_value"][k], le["L_value"][k],
                              le["C_value"][k], w)
        stamp(int(le["le_nodes"][k][0]), int(le["le_nodes"][k][1]), y)
    for k in range(len(ports["port_nodes"])):
        stamp(int(ports["port_nodes"][k][0]), int(ports["port_nodes"][k][1]), 1.0 / z0)
    return sp.csr_matrix((np.asarray(v, dtype=np.complex128) * escalings["Yle"], (r, c)),
                         shape=(n, n))


def compute_Z_self(R, Cd, w):
    """compute_Z_self.jl:1-15."""
    Z = np.zeros(R.shape[0], dtype=np.complex128)
    for aux in range(4):
        r = R[:, aux]
        cd = Cd[:, aux]
        both = (r != 0) & (cd != 0)
        onlyr = (r != 0) & ~both
        onlyc = (cd != 0) & ~both
        Z[both] += 1 / (1 / r[both] + 1j * w * cd[both])
        Z[onlyr] += r[onlyr]
        Z[onlyc] += 1 / (1j * w * cd[onlyc])
    return Z


def frequency_setup(k_w, escalings, incidence_selection, diagonals, Zs_info, lumped_elements,
                    ports, z0):
    """Per-frequency DZ, invZ, Yle and the factorised SS (FFT_solver_QS_S_type.jl:105-119)."""
    A = incidence_selection["A"]
    Gamma = incidence_selection["Gamma"]
    m, n = A.shape
    ns = Gamma.shape[1]
    w = k_w
    Yle = build_Yle(lumped_elements, ports, escalings, n, w / escalings["freq"], z0)
    Z_self = compute_Z_self(diagonals["R"], diagonals["Cd"], w)
    Zs = escalings["R"] * (Zs_info["Zs"] * math.sqrt(w / escalings["freq"]))
    se = Zs_info["surface_edges"]
    diff = Zs[se].real - Z_self[se].real
    put0_self = se[diff > 0]
    put0_zs = se[diff < 0]
    Z_self[put0_self] = 1j * Z_self[put0_self].imag
    Zs = Zs.copy()
    Zs[put0_zs] = 1j * Zs[put0_zs].imag
    DZ = Z_self + Zs.real
    DZ = DZ + 1j * w * diagonals["Lp"]
    invZ = sp.diags(1.0 / DZ)
    invP = sp.diags(1.0 / diagonals["P"])
    SS = (Yle + A.T @ (invZ @ A) + 1j * w * ((Gamma @ invP) @ Gamma.T)).tocsc()
    F = spla.splu(SS)
    return {"DZ": DZ, "invZ": invZ, "invP": invP, "Yle": Yle, "F": F.solve, "SS": SS, "lu": F}


def s2z(S, z0):
    npt, _, nf = S.shape
    Id = np.eye(npt)
    return np.stack([z0 * np.linalg.solve(Id - S[:, :, k], Id + S[:, :, k]) for k in range(nf)], axis=2)


def s2y(S, z0):
    npt, _, nf = S.shape
    Id = np.eye(npt)
    return np.stack([z0 * np.linalg.solve(Id + S[:, :, k], Id - S[:, :, k]) for k in range(nf)], axis=2)


def FFT_solver_QS_S_type(freq, escalings, incidence_selection, FFTCP, FFTCLp, diagonals, ports,
                         ports_scatter_value, lumped_elements, expansions, GMRES_settings,
                         Zs_info, callback=None):
    """Frequency x port loop with warm starts (FFT_solver_QS_S_type.jl:1-234)."""
    freq = np.asarray(freq, dtype=np.float64).ravel() * escalings["freq"]
    inner = GMRES_settings["Inner_Iter"]
    A = incidence_selection["A"]
    m, n = A.shape
    ns = incidence_selection["Gamma"].shape[1]
    w = 2 * np.pi * freq
    nfreq = w.size
    pn = np.asarray(ports["port_nodes"], dtype=np.int64)
    npt = pn.shape[0]
    S = np.zeros((npt, npt, nfreq), dtype=np.complex128)
    Vrest = np.zeros((m + n + ns, npt), dtype=np.complex128)
    info = []
    tol = GMRES_settings["tol"]
    for k in range(nfreq):
        fs = frequency_setup(w[k], escalings, incidence_selection, diagonals, Zs_info,
                             lumped_elements, ports, ports_scatter_value)

        def mv(x, fs=fs, wk=w[k]):
            return ComputeMatrixVectorFTT(x, wk, incidence_selection, FFTCP, FFTCLp, fs["DZ"],
                                          fs["Yle"], expansions, fs["invZ"], fs["invP"], fs["F"])

        for c1 in range(npt):
            n1, n2 = pn[c1]
            is_ = np.zeros(n)
            is_[n1] = escalings["Is"]
            is_[n2] = -escalings["Is"]
            tn = precond_3_3_Kt_fft(fs["F"], fs["invZ"], fs["invP"], A,
                                    incidence_selection["Gamma"], m, ns, is_)
            tk = tol[k] if np.ndim(tol) else tol
            V, flag, relres, it, resvec = gmres_custom(tn, False, tk, inner, Vrest[:, c1], mv)
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
    return {"S": S, "Z": s2z(S, ports_scatter_value), "Y": s2y(S, ports_scatter_value),
            "f": freq / escalings["freq"], "info": info, "Vrest": Vrest}


def dense_operator(matvec, N):
    """Explicit K by columns, for tiny grids."""
    cols = []
    for j in range(N):
        e = np.zeros(N, dtype=np.complex128)
        e[j] = 1
        cols.append(matvec(e))
    return np.stack(cols, axis=1)
