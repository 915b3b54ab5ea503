"""CPU check of the reduced-circulant formulation the CUDA kernels implement.

The GPU applies each Toeplitz block between two lattices (face families / edge
directions) on a power-of-two circulant of length L >= 2N-2 (symmetric blocks) or
L >= Na+Nb-1 (cross blocks, whose interleaved lattice offsets are odd), with the
kernel K(e) = row[|s*e + o|]. This test re-implements exactly that with numpy FFTs
and compares it with the reference's 2N-extent embedding (the oracle) applied
through the reference exp_P / mat_map_Lp maps, block by block.
"""
import numpy as np
import pytest

from oracle import peec_oracle as O
from solver_gb300 import configs, mesher

FAM_DIMS = lambda Nx, Ny, Nz: [(Nx, Ny + 1, Nz), (Nx + 1, Ny, Nz), (Nx, Ny, Nz + 1),
                               (Nx - 1, Ny, Nz), (Nx, Ny - 1, Nz), (Nx, Ny, Nz - 1)]
# (row key, in family, out family, conj, s, o, symmetric) -- as in ctx.cu
APPS = [("Lpx", 3, 3, 0, (1, 1, 1), (0, 0, 0), True), ("Lpy", 4, 4, 0, (1, 1, 1), (0, 0, 0), True),
        ("Lpz", 5, 5, 0, (1, 1, 1), (0, 0, 0), True),
        ("p12_se", 0, 0, 0, (1, 1, 1), (0, 0, 0), True),
        ("p34_se", 1, 1, 0, (1, 1, 1), (0, 0, 0), True),
        ("p56_se", 2, 2, 0, (1, 1, 1), (0, 0, 0), True),
        ("p1234", 1, 0, 0, (2, 2, 1), (1, -1, 0), False), ("p1234", 0, 1, 1, (2, 2, 1), (1, -1, 0), False),
        ("p1256", 2, 0, 0, (1, 2, 2), (0, -1, 1), False), ("p1256", 0, 2, 1, (1, 2, 2), (0, -1, 1), False),
        ("p3456", 2, 1, 0, (2, 1, 2), (-1, 0, 1), False), ("p3456", 1, 2, 1, (2, 1, 2), (-1, 0, 1), False)]


def pow2(v):
    r = 1
    while r < v:
        r <<= 1
    return r


def fft_len(na, nb, sym):
    need = (2 * na - 2 if na > 1 else 1) if sym else na + nb - 1
    return pow2(max(need, 1))


def reduced_apply(row, M, na, nb, s, o, sym, conj, x_in):
    """y_out (na lattice) = K x_in (nb lattice) the way k_embed/k_yz/k_xinv do it."""
    fa, fb = (nb, na) if conj else (na, nb)  # lattices of the conj=0 application
    L = [fft_len(fa[k], fb[k], sym) for k in range(3)]
    Kc = np.zeros(L)
    idx = []
    for k in range(3):
        j = np.arange(L[k])
        e = np.where(j < fa[k], j, np.where(j > L[k] - fb[k], j - L[k], 10 ** 9))
        t = np.abs(s[k] * e + o[k])
        t = np.where((e != 10 ** 9) & (t < M[k]), t, -1)
        idx.append(t)
    R = np.reshape(row, M, order="F")
    ix, iy, iz = np.meshgrid(*idx, indexing="ij")
    ok = (ix >= 0) & (iy >= 0) & (iz >= 0)
    Kc[ok] = R[ix[ok], iy[ok], iz[ok]]
    S = np.fft.fftn(Kc)
    if conj:
        S = np.conj(S)
    X = np.zeros(L, dtype=complex)
    X[:nb[0], :nb[1], :nb[2]] = np.reshape(x_in, nb, order="F")
    Y = np.fft.ifftn(S * np.fft.fftn(X))
    return np.reshape(Y[:na[0], :na[1], :na[2]], -1, order="F")


GOLDEN = __import__("pathlib").Path(__file__).resolve().parent / "golden"

REQS = {
    "crossbar_20x20x4": configs.crossbar_20x20x4,
    "first_run_data": lambda: mesher.load_request(GOLDEN / "first_run_data.json"),
    "random_17x13x9": lambda: configs.random_mixed((17, 13, 9), p=0.35, seed=11, nports=1),
    "random_8x9x5": lambda: configs.random_mixed((8, 9, 5), p=0.5, seed=3, nports=1),
}


@pytest.mark.parametrize("name", sorted(REQS))
def test_reduced_blocks_match_reference_embedding(name):
    out, freqs, settings, z0, grid = mesher.parse_request(REQS[name]())
    esc, inc, cc, diag, exp, ports, le, li, Zs = out
    Nx, Ny, Nz = grid
    rows = O.fill_rows(cc, esc, Nx, Ny, Nz)
    FFTCP, FFTCLp = O.spectra_from_rows(rows, Nx, Ny, Nz)
    fd = FAM_DIMS(Nx, Ny, Nz)
    rd = O.ref_dims(Nx, Ny, Nz)
    rng = np.random.default_rng(0)
    m = inc["A"].shape[0]
    ns = inc["Gamma"].shape[1]
    mx, my = inc["mx"], inc["my"]
    offs = [0, mx, mx + my, m]
    I = rng.standard_normal(m) + 1j * rng.standard_normal(m)
    Q = rng.standard_normal(ns) + 1j * rng.standard_normal(ns)
    E = exp["exp_P"]
    # family maps: lattice cell -> compact index
    fam_of = {0: (0, 0), 1: (1, 1), 2: (2, 2)}

    def gather(f, vec):
        if f >= 3:
            M_ = exp["mat_map_Lp"][f - 3][0]
            return M_ @ vec[offs[f - 3]:offs[f - 2]]
        return E[f][f] @ vec

    def scatter(f, lat):
        if f >= 3:
            return exp["mat_map_Lp"][f - 3][0].T @ lat
        return E[f][f].T @ lat

    pairs = {"p1234": (0, 1), "p1256": (0, 2), "p3456": (1, 2)}
    for key, fin, fout, conj, s, o, sym in APPS:
        if key not in rows or min(fd[fin]) <= 0:
            continue
        vec = I if fin >= 3 else Q
        got = scatter(fout, reduced_apply(rows[key], rd[key], fd[fout], fd[fin], s, o, sym, conj,
                                          gather(fin, vec)))
        # reference: the same block through the 2N embedding and reference maps
        if fin >= 3:
            c = fin - 3
            ref = exp["mat_map_Lp"][c][0].T @ O._conv(FFTCLp[c], gather(fin, vec))
        elif key in pairs:
            c1, c2 = pairs[key]
            if not conj:   # in = exp_P[c1][c2] family, out = exp_P[c2][c1]'
                ref = E[c2][c1].T @ O._conv(FFTCP[c1][c2], E[c1][c2] @ Q)
            else:
                ref = E[c1][c2].T @ O._conv(FFTCP[c1][c2], E[c2][c1] @ Q)
        else:
            ref = E[fin][fin].T @ O._conv(FFTCP[fin][fin], E[fin][fin] @ Q)
        if ref.size == 0:
            continue
        err = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)
        assert err < 1e-12, (name, key, conj, err)
