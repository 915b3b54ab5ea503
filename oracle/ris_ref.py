"""ORACLE -- test infrastructure only. CPU restatement of the reference's dense RIS solver
(src/lib/solverRis), used by tests/ as the checker; never imported by the product.

Parity unpinned: the reference (Julia) cannot run here and ships no outputs for this
path (its only numeric test is the unrelated electric-field solver). The restatement is
checked against itself where the formulas allow (tests/test_oracle_ris.py): the single
LU solve of the product equals the reference's three by linearity, the S parameters of
a port pair are symmetric, and a dense operator built from the voxel path's circulant
blocks reproduces the voxel path's products block by block.

Follows:
  src/lib/solverRis/compute_matrix_vector.jl:1-33    ComputeMatrixVectorRis
  src/lib/solverRis/compute_matrix_vector.jl:35-57   precond_3_3_vector (three LU solves)
  src/lib/solverRis/compute_matrix_vector.jl:59-64   prod_real_complex_Ris
  src/lib/solverRis/iter_solver_QS_S_type.jl:1-165   frequency x port loop, Z_self, S
  src/lib/solverRis/iter_solver_QS_S_type.jl:167-187 precond_3_3_Kt_S!
  src/lib/solverRis/build_Yle_S.jl:1-151             lumped elements and port closures
  src/lib/solverRis/gmres_custom.jl:1-334            the same Householder GMRES as the
                                                      voxel path (oracle.peec_oracle)
"""
from __future__ import annotations

import math

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from . import peec_oracle as O

MU0 = 4 * math.pi * 1e-7
EPS0 = 8.854187816997944e-12


def prod_real_complex(A, x):
    """A real, x complex: A re(x) + i A im(x) (compute_matrix_vector.jl:59-64)."""
    x = np.asarray(x)
    return A @ x.real + 1j * (A @ x.imag)


def ComputeMatrixVectorRis(x, w, incidence_selection, P_data, Lp_data, Z_self, Yle, invZ, invP,
                           F):
    """y = M^-1 K x with dense Lp blocks and a dense P (compute_matrix_vector.jl:1-33)."""
    A = incidence_selection["A"]
    Gamma = incidence_selection["Gamma"]
    m = A.shape[0]
    ns = Gamma.shape[1]
    x = np.asarray(x, dtype=np.complex128).ravel()
    I, Q, Phi = x[:m], x[m:m + ns], x[m + ns:]
    mx, my, mz = incidence_selection["mx"], incidence_selection["my"], incidence_selection["mz"]
    # real matrices times complex vectors as two real products (what the reference's
    # real-by-complex multiplication amounts to)
    mul = lambda M, v: prod_real_complex(M, v) if np.isrealobj(M) else M @ v
    Y1 = np.zeros(m, dtype=np.complex128)
    Y1[:mx] = mul(Lp_data["Lp_x"], I[:mx])
    Y1[mx:mx + my] = mul(Lp_data["Lp_y"], I[mx:mx + my])
    Y1[mx + my:mx + my + mz] = mul(Lp_data["Lp_z"], I[mx + my:mx + my + mz])
    Y1 = 1j * w * Y1 + np.asarray(Z_self).ravel() * I + A @ Phi
    Y2 = mul(P_data["P"], Q) - Gamma.T @ Phi
    Y3 = -(A.T @ I) + Yle @ Phi + 1j * w * (Gamma @ Q)
    return precond_3_3_vector(F, invZ, invP, A, Gamma, w, Y1, Y2, Y3)


def precond_3_3_vector(F, invZ, invP, A, Gamma, w, X1, X2, X3):
    """compute_matrix_vector.jl:35-57: three LU solves, real factors applied to the real
    and imaginary parts."""
    n1, n2 = X1.size, X2.size
    Y = np.zeros(n1 + n2 + X3.size, dtype=np.complex128)
    M1 = prod_real_complex(invZ, X1)
    M2 = F(prod_real_complex(A.T, M1))
    M3 = prod_real_complex(invP, X2)
    M4 = F(prod_real_complex(Gamma, M3))
    M5 = F(X3)
    pz = lambda v: invZ @ v
    Y[:n1] = (M1 - pz(prod_real_complex(A, M2)) + 1j * w * pz(prod_real_complex(A, M4))
              - pz(prod_real_complex(A, M5)))
    Y[n1:n1 + n2] = (prod_real_complex(invP, prod_real_complex(Gamma.T, M2)) + M3
                     - 1j * w * prod_real_complex(invP, prod_real_complex(Gamma.T, M4))
                     + prod_real_complex(invP, prod_real_complex(Gamma.T, M5)))
    Y[n1 + n2:] = M2 - 1j * w * M4 + M5
    return Y


def precond_3_3_Kt_S(F, invZ, invP, A, Gamma, m, ns, X3):
    """Right-hand side M^-1 [0; 0; is] (iter_solver_QS_S_type.jl:167-187)."""
    M5 = F(X3)
    return np.concatenate([-(invZ @ (A @ M5)), invP @ (Gamma.T @ M5), M5])


def lumped_admittance_S(typ, R, L, C, w):
    """get_lumped_elements_admittance_S (build_Yle_S.jl:70-151), statement by statement
    (numpy scalars give Julia's IEEE results for divisions by zero). Its type-2 case differs
    from the voxel path's in the fifth network: 1/(1/(jwC)) + jwC."""
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
                y = 1 / (1 / (jw * C)) + jw * C
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


def build_Yle_S(lumped_elements, grounding_nodes, ports, escalings, n, w, val_chiusura):
    """build_Yle_S.jl:1-68: lumped elements, port closures 1/R and grounding nodes 1e-12,
    summed per (row, column). The reference keeps the sums in a Float64 dictionary, which
    holds only real admittances (resistive elements and the port closures); complex ones
    are kept complex here."""
    acc = {}

    def add(r, c, v):
        acc[(r, c)] = acc.get((r, c), 0.0) + v

    le = lumped_elements
    for k in range(len(le.get("le_nodes", []))):
        n1, n2 = int(le["le_nodes"][k][0]), int(le["le_nodes"][k][1])
        y = lumped_admittance_S(int(le["type"][k]), le["R"][k], le["L"][k], le["C"][k], w)
        add(n1, n1, y)
        add(n2, n2, y)
        add(n1, n2, -y)
        add(n2, n1, -y)
    for k in range(len(ports["port_nodes"])):
        n1, n2 = int(ports["port_nodes"][k][0]), int(ports["port_nodes"][k][1])
        add(n1, n1, 1 / val_chiusura)
        add(n2, n2, 1 / val_chiusura)
        add(n1, n2, -1 / val_chiusura)
        add(n2, n1, -1 / val_chiusura)
    for g in grounding_nodes:
        add(int(g), int(g), 1 / 1e12)
    if not acc:
        return sp.csr_matrix((n, n), dtype=np.complex128)
    rc = np.array(list(acc.keys()), dtype=np.int64)
    v = np.array(list(acc.values()), dtype=np.complex128) * escalings["Yle"]
    return sp.csr_matrix((v, (rc[:, 0], rc[:, 1])), shape=(n, n))


def z_self(volumi, w, use_Zs_in):
    """Z_self of iter_solver_QS_S_type.jl:82-101: R (or the surface impedance where it is
    larger, with use_Zs_in) plus 1/(jw Cd) on the dielectric volumes."""
    R = np.asarray(volumi["R"], dtype=np.float64).ravel()
    diel = np.asarray(volumi.get("indici_dielettrici", []), dtype=np.int64).ravel()
    ncd = len(volumi["Cd"]) if diel.size else R.size
    invCd = np.zeros(ncd, dtype=np.complex128)
    if diel.size:
        Cd = np.asarray(volumi["Cd"], dtype=np.float64).ravel()
        invCd[diel] = 1 / (1j * w * Cd[diel])
    if use_Zs_in:
        Zs = (np.sqrt(1j * w) * np.asarray(volumi["Zs_part"], dtype=np.complex128).ravel()).real
        Z = np.zeros(R.size, dtype=np.complex128)
        indR = R > Zs
        Z[indR] = R[indR]
        Z[~indR] = Zs[~indR]
        return Z + invCd
    return R + invCd


def frequency_setup(w, escalings, incidence_selection, P_data, Lp_data, ports, lumped_elements,
                    volumi, use_Zs_in, val_chiusura, QS_Rcc_FW=1, freq_unscaled=None):
    """One frequency's operator state (iter_solver_QS_S_type.jl:31-115)."""
    A = incidence_selection["A"]
    Gamma = incidence_selection["Gamma"]
    m, n = A.shape
    if QS_Rcc_FW == 2:
        beta = 2 * math.pi * freq_unscaled * math.sqrt(EPS0 * MU0)
        Lp = {k: Lp_data[k] * np.exp(-1j * beta * Lp_data[r])
              for k, r in (("Lp_x", "Rx"), ("Lp_y", "Ry"), ("Lp_z", "Rz"))}
        P = {"P": P_data["P"] * np.exp(-1j * beta * P_data["R_cc"])}
        diag_Lp = np.concatenate([np.diag(Lp[k]).real for k in ("Lp_x", "Lp_y", "Lp_z")])
    else:
        Lp, P = Lp_data, P_data
        diag_Lp = np.concatenate([np.diag(Lp_data[k]).real for k in ("Lp_x", "Lp_y", "Lp_z")])
    Yle = build_Yle_S(lumped_elements, [], ports, escalings, n, w / escalings["freq"], val_chiusura)
    Zs = z_self(volumi, w, use_Zs_in)
    invZ = sp.diags(1.0 / (Zs + 1j * w * diag_Lp))
    invP = sp.diags(1.0 / np.diag(P_data["P"]).real)
    SS = (Yle + A.T @ (invZ @ A) + 1j * w * ((Gamma @ invP) @ Gamma.T)).tocsc()
    lu = spla.splu(SS)
    return dict(Lp=Lp, P=P, Z_self=Zs, diag_Lp=diag_Lp, Yle=Yle, invZ=invZ, invP=invP, SS=SS,
                lu=lu, F=lu.solve)


def iter_solver_QS_S_type(freq, escalings, incidence_selection, P_data, Lp_data, ports,
                          lumped_elements, GMRES_settings, volumi, use_Zs_in, QS_Rcc_FW,
                          ports_scatter_value):
    """iter_solver_QS_S_type.jl:1-165: per frequency the state, per port the right-hand
    side, GMRES warm-started from that port's previous solution, and the S column."""
    freq = np.asarray(freq, dtype=np.float64).ravel() * escalings["freq"]
    A = incidence_selection["A"]
    Gamma = incidence_selection["Gamma"]
    m, n = A.shape
    ns = Gamma.shape[1]
    pn = np.asarray(ports["port_nodes"], dtype=np.int64).reshape(-1, 2)
    npt = pn.shape[0]
    R = ports_scatter_value
    S = np.zeros((npt, npt, freq.size), dtype=np.complex128)
    Vrest = np.zeros((m + ns + n, npt), dtype=np.complex128)
    info = []
    for k, f in enumerate(freq):
        w = 2 * math.pi * f
        st = frequency_setup(w, escalings, incidence_selection, P_data, Lp_data, ports,
                             lumped_elements, volumi, use_Zs_in, R, QS_Rcc_FW,
                             f / escalings["freq"])
        mv = lambda x, st=st, w=w: ComputeMatrixVectorRis(x, w, incidence_selection, st["P"],
                                                          st["Lp"], st["Z_self"], st["Yle"],
                                                          st["invZ"], st["invP"], st["F"])
        for c1 in range(npt):
            n1, n2 = pn[c1]
            isv = np.zeros(n)
            isv[n1] = escalings["Is"]
            isv[n2] = -escalings["Is"]
            tn = precond_3_3_Kt_S(st["F"], st["invZ"], st["invP"], A, Gamma, m, ns, isv)
            V, flag, relres, it, _rv = O.gmres_custom(tn, False, GMRES_settings["tol"][k],
                                                      GMRES_settings["Inner_Iter"],
                                                      Vrest[:, c1].copy(), mv)
            info.append(dict(freq=k, port=c1, flag=flag, relres=relres, iter=list(it)))
            Vrest[:, c1] = V
            for c2 in range(c1, npt):
                n3, n4 = pn[c2]
                d = 2 * (V[m + ns + n3] - V[m + ns + n4])
                S[c1, c2, k] = (d - R) / R if c1 == c2 else d / R
                S[c2, c1, k] = S[c1, c2, k]
    return {"S": S, "Z": O.s2z(S, R), "Y": O.s2y(S, R), "f": freq / escalings["freq"],
            "info": info, "Vrest": Vrest}
