"""CPU check of the octant storage of the circulant spectra.

Every block kernel K(e) = row[|s*e + o|] on its circulant is, along each axis, either
even (s = 1, o = 0) or even about a half-sample shift: K(c - e) = K(e) with c = -o for
s = 2, and the embedding window [-(nb-1), na-1] is symmetric about c/2 because
c = na - nb. Then R(k) = K^(k) * prod_a exp(+i*pi*c_a*k_a/L_a), with the signed
frequency k_a in (-L_a/2, L_a/2], is real and even in each axis, and
    K^(k) = R(|k_1|, |k_2|, |k_3|) * prod_a exp(-i*pi*c_a*k_a/L_a),
so the (L_x/2+1)(L_y/2+1)(L_z/2+1) real octant values hold the whole spectrum.
"""
import numpy as np
import pytest

from oracle import peec_oracle as O
from solver_gb300 import configs, mesher
from solver_gb300.operator import row_dims
from test_reduced_conv import FAM_DIMS, fft_len

# (row key, out family, in family, s, o) of the nine stored spectra
SPECS = [("p12_se", 0, 0, (1, 1, 1), (0, 0, 0)), ("p34_se", 1, 1, (1, 1, 1), (0, 0, 0)),
         ("p56_se", 2, 2, (1, 1, 1), (0, 0, 0)), ("p1234", 0, 1, (2, 2, 1), (1, -1, 0)),
         ("p1256", 0, 2, (1, 2, 2), (0, -1, 1)), ("p3456", 1, 2, (2, 1, 2), (-1, 0, 1)),
         ("Lpx", 3, 3, (1, 1, 1), (0, 0, 0)), ("Lpy", 4, 4, (1, 1, 1), (0, 0, 0)),
         ("Lpz", 5, 5, (1, 1, 1), (0, 0, 0))]


def embed(row, M, na, nb, s, o, L):
    idx = []
    for k in range(3):
        j = np.arange(L[k])
        e = np.where(j < na[k], j, np.where(j > L[k] - nb[k], j - L[k], 10 ** 9))
        t = np.abs(s[k] * e + o[k])
        idx.append(np.where((e != 10 ** 9) & (t < M[k]), t, -1))
    R = np.reshape(row, M, order="F")
    ix, iy, iz = np.meshgrid(*idx, indexing="ij")
    ok = (ix >= 0) & (iy >= 0) & (iz >= 0)
    K = np.zeros(L)
    K[ok] = R[ix[ok], iy[ok], iz[ok]]
    return K


@pytest.mark.parametrize("shape,seed", [((17, 13, 9), 11), ((8, 9, 5), 3)])
def test_octant_reconstructs_spectra(shape, seed):
    out, freqs, settings, z0, grid = mesher.parse_request(
        configs.random_mixed(shape, p=0.4, seed=seed, nports=1))
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    rows = O.fill_rows(cc, esc, *grid)
    fam = FAM_DIMS(*grid)
    # the face families share one grid (the largest requirement over the six P blocks)
    LP = [max(fft_len(fam[a][k], fam[b][k], a == b) for _, a, b, _, _ in SPECS[:6])
          for k in range(3)]
    for key, a, b, s, o in SPECS:
        na, nb = fam[a], fam[b]
        if min(na) < 1 or min(nb) < 1:
            continue
        L = LP if a < 3 else [fft_len(na[k], na[k], True) for k in range(3)]
        M = list(row_dims(*grid)[key])
        K = embed(rows[key], M, na, nb, s, o, L)
        S = np.fft.fftn(K)
        c = [(-o[k] if s[k] == 2 else 0) for k in range(3)]
        assert all(c[k] == 0 or c[k] == na[k] - nb[k] for k in range(3)), (key, c)
        ks = [np.where(np.arange(L[k]) <= L[k] // 2, np.arange(L[k]), np.arange(L[k]) - L[k])
              for k in range(3)]
        ph = [np.exp(1j * np.pi * c[k] * ks[k] / L[k]) for k in range(3)]
        Rfull = S * ph[0][:, None, None] * ph[1][None, :, None] * ph[2][None, None, :]
        scale = np.max(np.abs(S))
        assert np.max(np.abs(Rfull.imag)) <= 1e-12 * scale, key
        oc = [np.abs(ks[k]) for k in range(3)]
        Roct = Rfull.real[:L[0] // 2 + 1, :L[1] // 2 + 1, :L[2] // 2 + 1]
        rec = Roct[oc[0][:, None, None], oc[1][None, :, None], oc[2][None, None, :]]
        rec = rec / (ph[0][:, None, None] * ph[1][None, :, None] * ph[2][None, None, :])
        assert np.max(np.abs(rec - S)) <= 1e-12 * scale, key
